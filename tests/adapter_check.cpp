// Test driver for the header-only C++ adapter rsx/saxs_algorithm.hpp, used the
// way a C++ caller of resaxslib's algorithm interface uses it
// (saxs_algorithm.hpp:118-244: params, initialize, calc_curve, recalc_curve,
// commit, revert; rsasa_algorithm.hpp:42-61: calc_rsasa).  Built and run by
// tests/test_adapter.py.
//
//   adapter_check nogpu
//       error paths that need no device; prints "ok"
//   adapter_check gpu <in.bin> <out.bin>
//       in.bin:  int32 n, n_q, n_types, water_index, start, length;
//                float q[n_q], factors[n_q][n_types], bodies[n][4], rsasa[n],
//                radius_of_type[n_types]
//       out.bin: float curves[8][n_q], then float rsasa_out[n],
//                water_rsasa[n], water_rsasa_moved[n], typed_rsasa[n]
//         0 calc_curve(bodies)
//         1 recalc_curve after bodies [start, start+length) moved by +0.3 A in x
//         2 after revert() to the committed state of curve 0, recalc_curve
//           with the same bodies moved by +0.6 A instead
//         3 calc_curve of the +0.6 A bodies after commit()
//         4 calc_curve(bodies) with water weight 0.7, the given rsasa and
//           no_rsasa_recalc_ set (the given values are kept)
//         5 the same after a second initialize() (water params already pushed)
//         6 calc_curve(bodies) with water weight 0.7 and no_rsasa_recalc_
//           cleared: rsasa comes from the adapter's own SASA (water_rsasa)
//         7 then recalc_curve of the +0.3 A bodies: rsasa recomputed
//           (water_rsasa_moved)
//       rsasa_out: calc_rsasa with 960 Fibonacci dots, probe 1.4
//       typed_rsasa: calc_rsasa of an rsasa_gpu initialized with
//         dot_spheres_params(5 dots/A^2, probe 1.4) and the latitude sets of
//         the reference's CPU algorithm (one per atomic radius)
#include "rsx/saxs_algorithm.hpp"

#include <cstdint>
#include <cstdio>
#include <fstream>
#include <vector>

using rsx::error;

namespace {

template <typename F> bool throws_code(F &&f, int code)
{
    try {
        f();
    } catch (const error &e) {
        if (e.err() == code)
            return true;
        std::fprintf(stderr, "wrong code %d (want %d): %s\n", e.err(), code, e.what());
        return false;
    }
    std::fprintf(stderr, "no exception (want code %d)\n", code);
    return false;
}

int run_nogpu()
{
    std::vector<float> q = {0.f, 0.1f, 0.2f}, ff = {1.f, 2.f, 1.f, 2.f, 1.f, 2.f}, out;
    std::vector<rsx_body> bodies(4);
    for (unsigned i = 0; i < bodies.size(); ++i) {
        bodies[i] = rsx_body{float(i), 0.f, 0.f, 0.f};
        rsx::set_factor_index(bodies[i], i & 1);
    }
    bool ok = true;
    auto alg = rsx::algorithm::create_saxs_gpu();
    // no params: initialize() and calc_curve() refuse
    ok &= throws_code([&] { alg->initialize(); }, error::SAXS_ARGS_NOT_SET);
    ok &= throws_code([&] { alg->calc_curve(bodies, out); }, error::SAXS_ARGS_NOT_SET);
    ok &= throws_code([&] { alg->recalc_curve(bodies, 0, 1, out); }, error::SAXS_NO_INITIAL_CALC);
    ok &= throws_code([&] { alg->commit(); }, error::SAXS_NO_INITIAL_CALC);
    ok &= throws_code([&] { alg->revert(); }, error::SAXS_NO_INITIAL_CALC);
    // a table whose size is not a multiple of n_q
    alg->access_params().initialize(q, bodies);
    alg->access_params().get_ff_params().access_factors() = {1.f, 2.f};
    ok &= throws_code([&] { alg->initialize(); }, error::SAXS_ARGS_NOT_SET);
    // a valid set-up cannot create a handle without a CUDA device: no CPU path
    alg->access_params().get_ff_params().access_factors() = ff;
    try {
        alg->initialize();
        std::fprintf(stderr, "initialize() succeeded without a GPU\n");
        ok = false;
    } catch (const error &e) {
        if (e.err() != RSX_INVALID_DEVICE && e.err() != RSX_PROGRAM_NOT_LOADED) {
            std::fprintf(stderr, "unexpected code %d: %s\n", e.err(), e.what());
            ok = false;
        }
    }
    rsx::algorithm::rsasa_gpu sasa;
    std::vector<float> rs(4);
    ok &= throws_code([&] { sasa.calc_rsasa(bodies, rs); }, error::SAXS_ARGS_NOT_SET);
    ok &= throws_code([&] { sasa.recalc_rsasa(bodies, rs); }, error::SAXS_NO_INITIAL_CALC);
    if (!ok)
        return 1;
    std::printf("ok\n");
    return 0;
}

template <typename T> void read_into(std::ifstream &f, std::vector<T> &v, size_t n)
{
    v.resize(n);
    f.read(reinterpret_cast<char *>(v.data()), std::streamsize(n * sizeof(T)));
}

int run_gpu(const char *in_path, const char *out_path)
{
    std::ifstream f(in_path, std::ios::binary);
    std::vector<int32_t> hdr;
    read_into(f, hdr, 6);
    const int n = hdr[0], n_q = hdr[1], n_t = hdr[2], widx = hdr[3];
    const unsigned start = (unsigned)hdr[4], length = (unsigned)hdr[5];
    std::vector<float> q, ff, flat, rsasa, radius_of_type;
    read_into(f, q, n_q);
    read_into(f, ff, (size_t)n_q * n_t);
    read_into(f, flat, (size_t)n * 4);
    read_into(f, rsasa, n);
    read_into(f, radius_of_type, n_t);
    if (!f) {
        std::fprintf(stderr, "short input file\n");
        return 2;
    }
    std::vector<rsx_body> bodies(n);
    std::memcpy(bodies.data(), flat.data(), flat.size() * sizeof(float));
    std::vector<rsx_body> moved = bodies, moved2 = bodies;
    for (unsigned i = start; i < start + length; ++i) {
        moved[i].x += 0.3f;
        moved2[i].x += 0.6f;
    }

    std::vector<std::vector<float>> curves(8);
    auto alg = rsx::algorithm::create_saxs_gpu();
    auto &params = alg->access_params();
    params.initialize(q, bodies, {0});
    params.get_ff_params().access_factors() = ff;
    params.get_ff_params().set_water_ff_index(widx);
    alg->initialize();
    alg->calc_curve(bodies, curves[0]);
    alg->commit();
    alg->recalc_curve(moved, start, length, curves[1]);
    alg->revert();
    alg->recalc_curve(moved2, start, length, curves[2]);
    alg->commit();
    alg->calc_curve(moved2, curves[3]);

    auto &water = params.get_implicit_water_params();
    water.set_water_weight(0.7f);
    water.no_rsasa_recalc_ = true;
    water.access_rsasa() = rsasa;
    alg->calc_curve(bodies, curves[4]);
    alg->initialize(); // a new handle; the water params are no longer dirty
    alg->calc_curve(bodies, curves[5]);
    water.no_rsasa_recalc_ = false;
    alg->calc_curve(bodies, curves[6]);
    const std::vector<float> water_rsasa = water.rsasa();
    alg->recalc_curve(moved, start, length, curves[7]);
    const std::vector<float> water_rsasa_moved = water.rsasa();

    std::vector<float> dots(960 * 3);
    rsx::check(rsx_sasa_fibonacci_dots(960, dots.data()));
    rsx::algorithm::rsasa_gpu sasa;
    sasa.initialize((unsigned)n, radius_of_type, 1.4f, dots, 0);
    std::vector<float> rsasa_out(n);
    sasa.calc_rsasa(bodies, rsasa_out);
    rsx::algorithm::rsasa_gpu typed;
    typed.initialize((unsigned)n, rsx::algorithm::dot_spheres_params(5.f, 1.4f),
                     RSX_DOTS_LATITUDE, 0);
    std::vector<float> typed_rsasa(n);
    typed.calc_rsasa(bodies, typed_rsasa);
    typed.recalc_rsasa(bodies, typed_rsasa);

    std::ofstream o(out_path, std::ios::binary);
    for (const auto &c : curves) {
        if ((int)c.size() != n_q) {
            std::fprintf(stderr, "curve of %zu values, want %d\n", c.size(), n_q);
            return 3;
        }
        o.write(reinterpret_cast<const char *>(c.data()), std::streamsize(c.size() * 4));
    }
    const std::vector<float> *tails[] = {&rsasa_out, &water_rsasa, &water_rsasa_moved,
                                         &typed_rsasa};
    for (const std::vector<float> *v : tails) {
        if ((int)v->size() != n) {
            std::fprintf(stderr, "rsasa of %zu values, want %d\n", v->size(), n);
            return 3;
        }
        o.write(reinterpret_cast<const char *>(v->data()), std::streamsize(v->size() * 4));
    }
    return o ? 0 : 4;
}

} // namespace

int main(int argc, char **argv)
{
    try {
        if (argc == 2 && std::string(argv[1]) == "nogpu")
            return run_nogpu();
        if (argc == 4 && std::string(argv[1]) == "gpu")
            return run_gpu(argv[2], argv[3]);
    } catch (const error &e) {
        std::fprintf(stderr, "rsx::error %d: %s\n", e.err(), e.what());
        return 5;
    }
    std::fprintf(stderr, "usage: adapter_check nogpu | gpu <in.bin> <out.bin>\n");
    return 2;
}
