"""Form-factor tables and radii (host side) against the reference's own
atomic_form_factors (compiled from resaxslib/include/ff_coef.hpp)."""
import ctypes
import os
import platform

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def test_tables_match_reference():
    from resaxs_gb300 import _lib
    L = _lib.lib()
    g = np.load(os.path.join(HERE, "golden", "ff_ref.npz"))
    q = g["q"]
    for name in ("c100", "c103", "c095"):
        c, rm = g[name + "_args"]
        out = np.zeros((len(q), 16), np.float32)
        _lib.check(L.rsx_ff_atomic_table(q, len(q), ctypes.c_float(rm), ctypes.c_float(c),
                                         out.reshape(-1)))
        if platform.machine() == "x86_64":
            assert np.array_equal(out.view(np.uint32), g[name].view(np.uint32)), name
        else:  # another C library may round exp / pow differently in the last bit
            assert np.allclose(out, g[name], rtol=1e-6, atol=1e-6), name


def test_radii_and_avg_radius():
    from resaxs_gb300 import _lib
    from resaxs_gb300 import workloads as W
    L = _lib.lib()
    g = np.load(os.path.join(HERE, "golden", "ff_ref.npz"))
    r = np.zeros(16, np.float32)
    _lib.check(L.rsx_ff_radii(r))
    assert np.allclose(r, g["radii"], rtol=1e-6)
    b = W.pack_bodies(np.zeros((4, 3)), np.array([1, 1, 3, 14]))
    avg = ctypes.c_float()
    _lib.check(L.rsx_ff_avg_radius(b.reshape(-1), 4, ctypes.byref(avg)))
    assert abs(avg.value - (2 * r[1] + r[3] + r[14]) / 4) < 1e-6
    assert L.rsx_ff_type_count() == 16 and L.rsx_ff_water_index() == 14
