// C entry points over the reference's own host_debye templates
// (resaxslib/src/host_debye.cpp:54-109, resaxslib/include/host_debye.hpp:30-40),
// compiled together with that unmodified source file into oracle/_ref/.
// Test infrastructure only: the product never loads it.
#include "host_debye.hpp"

#include <memory>

extern "C" void ref_host_debye_df(const float *q, int n_q, const float *bodies, int n_bodies,
                                  const float *ff, int n_factors, float *out)
{
    resaxs::host_debye<double, float, cl_float4>::calc_curve(
        q, n_q, reinterpret_cast<const cl_float4 *>(bodies), n_bodies, ff, n_factors, out);
}

extern "C" void ref_host_debye_ff(const float *q, int n_q, const float *bodies, int n_bodies,
                                  const float *ff, int n_factors, float *out)
{
    resaxs::host_debye<float, float, cl_float4>::calc_curve(
        q, n_q, reinterpret_cast<const cl_float4 *>(bodies), n_bodies, ff, n_factors, out);
}

// bodies as cl_double4 with the type index stored as a 64-bit integer in .w
// (utils.hpp:68-73, 84-88)
extern "C" void ref_host_debye_dd(const double *q, int n_q, const double *bodies, int n_bodies,
                                  const double *ff, int n_factors, double *out)
{
    resaxs::host_debye<double, double, cl_double4>::calc_curve(
        q, n_q, reinterpret_cast<const cl_double4 *>(bodies), n_bodies, ff, n_factors, out);
}

// Form-factor tables of the reference (header-only resaxslib/include/ff_coef.hpp:104-212).
#include "ff_coef.hpp"

extern "C" void ref_ff_generate(const float *q, int n_q, float avg_radius, float expansion,
                                float *out /* [n_q][16] */)
{
    std::vector<float> qq(q, q + n_q), t;
    resaxs::atomic_form_factors<float>::generate(qq, avg_radius, expansion, t);
    for (size_t i = 0; i < t.size(); ++i)
        out[i] = t[i];
}

extern "C" void ref_ff_radii(float *out /* [16] */)
{
    std::vector<float> r;
    resaxs::atomic_form_factors<float>::calc_radii(r);
    for (size_t i = 0; i < r.size(); ++i)
        out[i] = r[i];
}

// PDB reader of the reference (resaxslib/src/parse_pdb.cpp:63-108, 309-363 with
// the atom maps of resaxslib/src/utils.cpp:200-317), compiled from those
// unmodified files.  Writes the bodies of all models back to back (x, y, z,
// type bits) and the body count of each model; returns the number of models,
// -1 when the file cannot be opened, -2 when out or model_sizes is too small.
#include "parse_pdb.hpp"

extern "C" int ref_parse_pdb(const char *path, float *out, int cap_bodies, int *model_sizes,
                             int max_models)
{
    try {
        resaxs::parse_pdb<float> p(path);
        p.set_verbose_level(resaxs::parse_pdb<float>::QUIET);
        auto models = p.all_models_as_complex_atoms();
        if ((int)models.size() > max_models)
            return -2;
        int k = 0;
        for (size_t m = 0; m < models.size(); ++m) {
            model_sizes[m] = (int)models[m].size();
            for (const auto &b : models[m]) {
                if (k >= cap_bodies)
                    return -2;
                std::memcpy(out + 4 * k, b.s, 16);
                ++k;
            }
        }
        return (int)models.size();
    } catch (...) {
        return -1;
    }
}

// Dot-sphere SASA of the reference (resaxslib/src/rsasa_algorithm.cpp:60-208,
// resaxslib/src/rsasa_cpu_alg.cpp:33-185), compiled from those unmodified
// files together with the OpenCL SASA class their factory instantiates
// (never called here; see shim/CL/cl.hpp).
#include "rsasa_algorithm.hpp"

namespace {
typedef resaxs::algorithm::rsasa<float, float> rsasa_ff;
}

// One type's dot sphere as dot_spheres_params generates it for a body of
// `radius`: kind 0 = create_dots (latitude rings, the CPU algorithm's set,
// rsasa_algorithm.cpp:60-89), 1 = create_32_dots, 2 = create_fibonacci_dots
// (:96-116), 3 = create_dodecahedron_dots, 4 = create_dodeca_icosa_dots
// (:156-208, the OpenCL algorithm's set).  out_xyzw receives the dots as
// x, y, z, w (w = radius, as the reference stores it); returns the number of
// dots, or -1 for a bad kind, -2 when cap is too small.
extern "C" int ref_sasa_dots(int kind, float radius, float dot_density, float probe,
                             float *out_xyzw, int cap)
{
    rsasa_ff::dot_spheres_params p(dot_density, probe);
    std::vector<cl_float4> d;
    switch (kind) {
    case 0: d = p.create_dots(radius); break;
    case 1: d = p.create_32_dots(radius); break;
    case 2: d = p.create_fibonacci_dots(radius); break;
    case 3: d = p.create_dodecahedron_dots(radius); break;
    case 4: d = p.create_dodeca_icosa_dots(radius); break;
    default: return -1;
    }
    if ((int)d.size() > cap)
        return -2;
    for (size_t i = 0; i < d.size(); ++i)
        std::memcpy(out_xyzw + 4 * i, d[i].s, 16);
    return (int)d.size();
}

// rsasa_cpu_alg<float,float> through the reference's own factory and
// interface: rsasa<float>::create<algorithm>(rsasa_dot_spheres), initialize
// with dot_spheres_params(dot_density, probe), calc_rsasa.  atoms are float4
// bodies with the type index bits in .w; out_rsasa[i] = accessible dots /
// dots of atom i's type.  Returns 0, or the resaxs::error code on failure.
extern "C" int ref_rsasa_cpu(const float *atoms, int n_atoms, float dot_density, float probe,
                             float *out_rsasa)
{
    try {
        std::unique_ptr<resaxs::algorithm::i_rsasa<float, float, resaxs::algorithm::algorithm>> alg(
            rsasa_ff::create<resaxs::algorithm::algorithm>(resaxs::algorithm::rsasa_dot_spheres));
        rsasa_ff::dot_spheres_params p(dot_density, probe);
        alg->initialize(&p);
        std::vector<cl_float4> a((size_t)n_atoms);
        std::memcpy(a.data(), atoms, 16 * (size_t)n_atoms);
        std::vector<float> r((size_t)n_atoms);
        alg->calc_rsasa(a, r);
        std::memcpy(out_rsasa, r.data(), sizeof(float) * (size_t)n_atoms);
        return 0;
    } catch (const resaxs::error &e) {
        return e.err() != 0 ? e.err() : -1;
    } catch (...) {
        return -1;
    }
}
