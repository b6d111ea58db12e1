// calc_saxs: SAXS curve of one or more PDB models, optionally fitted to an
// experimental profile -- the reference's calc_saxs CLI (calc_saxs/main.cpp,
// calc_saxs.hpp, calc_saxs.cpp) over librsx.  Same flags, same output file
// format, same fitting procedure; the curves are computed on the GPU.
//
//   calc_saxs -f profile.dat [-s scale] [-w ww|[lo,hi]] [-e ef|[lo,hi]]
//             [-n q_n] [--q_min x] [--q_max x] [-d device] [-v level] [-t]
//             [--double] -o out.dat model1.pdb [model2.pdb ...]
#include "rsx.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iostream>
#include <limits>
#include <random>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

namespace {

enum Verbose { QUIET = 0, NORMAL, DETAILS, DEBUG };

struct CliError {
    std::string msg, arg;
};

struct RsxError {
    int code;
    std::string msg;
};

void check(rsx_status s)
{
    if (s != RSX_OK)
        throw RsxError{s, rsx_last_error()};
}

// trim / split with the reference's semantics (resaxslib/src/utils.cpp:300-350)
std::string trim(const std::string &s, const std::string &delim = " ")
{
    const auto p1 = s.find_first_not_of(delim);
    const auto p2 = s.find_last_not_of(delim);
    return s.substr(p1 == std::string::npos ? 0 : p1,
                    p2 == std::string::npos ? s.length() - 1 : p2 - p1 + 1);
}

std::vector<std::string> split(const std::string &s, char delim)
{
    std::vector<std::string> out;
    std::stringstream ss(s);
    std::string item;
    while (std::getline(ss, item, delim))
        out.push_back(item);
    return out;
}

// ---------------------------------------------------------------- arguments

struct Range {
    float min_, max_, lo, hi;
    bool set = false;
    bool singular() const { return lo == hi; }
};

void parse_range(Range &r, const std::string &text, const char *name)
{
    const std::string s = trim(text, "[](){} ");
    const auto elems = split(s, ',');
    auto num = [&](const std::string &e) {
        std::istringstream iss(trim(e));
        float v;
        if (!(iss >> v))
            throw CliError{trim(e) + " is not a real number", name};
        return v;
    };
    auto mm = [&] {
        return "[" + std::to_string(r.min_) + "," + std::to_string(r.max_) + "]";
    };
    if (elems.size() == 2) {
        r.lo = num(elems[0]);
        r.hi = num(elems[1]);
        if (r.lo < r.min_ || r.hi > r.max_ || r.lo > r.hi)
            throw CliError{s + " is not a valid range in " + mm(), name};
    } else if (elems.size() == 1) {
        r.lo = r.hi = num(elems[0]);
        if (r.lo < r.min_ || r.hi > r.max_)
            throw CliError{elems[0] + " is not in the valid range " + mm(), name};
    } else {
        throw CliError{s + " is not a real number or a valid range", name};
    }
    r.set = true;
}

struct Args {
    Verbose verbose = NORMAL;
    bool test = false, dbl = false;
    std::string device = "cpu", fit, out;
    float scale = 1.0f;
    bool scale_set = false;
    Range water{-2.0f, 4.0f, 0.0f, 0.0f};
    Range exp_factor{0.95f, 1.05f, 1.0f, 1.0f};
    unsigned q_n = 500;
    float q_max = 0.75f, q_min = 0.0f;
    std::vector<std::string> pdbs;
};

void usage(std::ostream &os)
{
    os << "USAGE: calc_saxs [-v quiet|normal|details|debug] [-t] [--double] [-d device]\n"
          "                 [-f fit_file] [-s scale] [-w ww|[lo,hi]] [-e ef|[lo,hi]]\n"
          "                 [-n q_n] [--q_max q] [--q_min q] -o outfile pdb_files...\n";
}

Args parse_args(int argc, char **argv)
{
    Args a;
    bool out_set = false;
    for (int i = 1; i < argc; ++i) {
        std::string tok = argv[i], val;
        bool has_eq = false;
        if (tok.rfind("--", 0) == 0) {
            const auto eq = tok.find('=');
            if (eq != std::string::npos) {
                val = tok.substr(eq + 1);
                tok = tok.substr(0, eq);
                has_eq = true;
            }
        }
        auto value = [&](const char *name) {
            if (has_eq)
                return val;
            if (i + 1 >= argc)
                throw CliError{"Missing a value for this argument!", name};
            return std::string(argv[++i]);
        };
        auto number = [&](const char *name) {
            std::istringstream iss(value(name));
            float v;
            if (!(iss >> v))
                throw CliError{"Couldn't read argument value", name};
            return v;
        };
        if (tok == "-h" || tok == "--help") {
            usage(std::cout);
            std::exit(0);
        } else if (tok == "--version") {
            std::cout << "calc_saxs  version: 0.1 (librsx " << rsx_version() << ")\n";
            std::exit(0);
        } else if (tok == "-v" || tok == "--verbose") {
            const std::string v = value("-v");
            const char *names[] = {"quiet", "normal", "details", "debug"};
            int k = -1;
            for (int j = 0; j < 4; ++j)
                if (v == names[j])
                    k = j;
            if (k < 0)
                throw CliError{"Value '" + v + "' does not meet constraint: quiet|normal|details|debug",
                               "-v"};
            a.verbose = Verbose(k);
        } else if (tok == "-t" || tok == "--test") {
            a.test = true;
        } else if (tok == "--double") {
            a.dbl = true;
        } else if (tok == "-d" || tok == "--device") {
            a.device = value("-d");
        } else if (tok == "-f" || tok == "--fit") {
            a.fit = value("-f");
        } else if (tok == "-s" || tok == "--scale") {
            a.scale = number("-s");
            a.scale_set = true;
        } else if (tok == "-w" || tok == "--water") {
            parse_range(a.water, value("-w"), "-w");
        } else if (tok == "-e" || tok == "--exp_factor") {
            parse_range(a.exp_factor, value("-e"), "-e");
        } else if (tok == "-n" || tok == "--q_n") {
            const float v = number("-n");
            if (v < 0 || v != std::floor(v))
                throw CliError{"Couldn't read argument value", "-n"};
            a.q_n = (unsigned)v;
        } else if (tok == "--q_max") {
            a.q_max = number("--q_max");
        } else if (tok == "--q_min") {
            a.q_min = number("--q_min");
        } else if (tok == "-o" || tok == "--outfile") {
            a.out = value("-o");
            out_set = true;
        } else if (!tok.empty() && tok[0] == '-' && tok.size() > 1) {
            throw CliError{"Couldn't find match for argument", tok};
        } else {
            a.pdbs.push_back(tok);
        }
    }
    if (!out_set)
        throw CliError{"Required argument missing: outfile", "-o"};
    if (a.pdbs.empty())
        throw CliError{"Required argument missing: pdb_files", "pdb_files"};
    return a;
}

// ----------------------------------------------------------------- PDB input

// All models of one PDB file as complex-atom bodies (librsx's reader of
// parse_pdb::all_models_as_complex_atoms).
std::vector<std::vector<rsx_body>> read_pdb(const std::string &path, Verbose verbose)
{
    int n_models = 0, n_bodies = 0;
    check(rsx_pdb_count(path.c_str(), &n_models, &n_bodies));
    std::vector<rsx_body> all(std::max(n_bodies, 1));
    std::vector<int> sizes(std::max(n_models, 1));
    check(rsx_pdb_read(path.c_str(), verbose >= NORMAL ? 1 : 0, all.data(), n_bodies, sizes.data(),
                       n_models));
    std::vector<std::vector<rsx_body>> models(n_models);
    size_t k = 0;
    for (int m = 0; m < n_models; ++m) {
        models[m].assign(all.begin() + k, all.begin() + k + sizes[m]);
        k += sizes[m];
    }
    return models;
}

// ------------------------------------------------------------ SAXS profile

// saxs_profile (resaxslib/include/saxs_profile.hpp): q, I, sigma columns,
// '#' comments; missing errors are simulated as 15% of I scaled by q and a
// Poisson factor, from the same standard-library generators.
struct Profile {
    std::vector<float> q, iq, err, prec2;

    static Profile read(const std::string &path)
    {
        std::ifstream f(path.c_str());
        if (!f)
            throw RsxError{-1101, path + " file not found"};
        Profile p;
        std::string line;
        while (!f.eof()) {
            std::getline(f, line);
            line = trim(line);
            if (line.empty() || line.find_first_of('#') == 0)
                continue;
            float qv, iv, ev;
            std::istringstream ls(line);
            ls >> qv >> iv;
            if (!ls)
                continue;
            p.q.push_back(qv);
            p.iq.push_back(iv);
            ls >> ev;
            if (ls)
                p.err.push_back(ev);
        }
        if (p.err.size() < p.q.size()) {
            p.err.resize(p.q.size());
            std::default_random_engine gen;
            std::poisson_distribution<int> poisson(10.0);
            for (size_t i = 0; i < p.q.size(); ++i) {
                const auto rnd = std::abs(poisson(gen) / 10.0 - 1.0) + 1.0;
                p.err[i] = float(0.15 * p.iq[i] * (p.q[i] + 0.001) * rnd);
            }
        }
        p.prec2.resize(p.q.size());
        for (size_t i = 0; i < p.q.size(); ++i)
            p.prec2[i] = 1 / (p.err[i] * p.err[i]);
        return p;
    }

    float optimize_scale_for(const std::vector<float> &other) const
    {
        float num = 0, den = 0;
        for (size_t i = 0; i < q.size(); ++i) {
            num += iq[i] * other[i] * prec2[i];
            den += other[i] * other[i] * prec2[i];
        }
        return num / den;
    }

    float chi(const std::vector<float> &other) const
    {
        float c2 = 0;
        for (size_t i = 0; i < q.size(); ++i) {
            const float d = iq[i] - other[i];
            c2 += d * d * prec2[i];
        }
        return std::sqrt(c2 / q.size());
    }
};

// --------------------------------------------------------------- evaluator

struct Fit {
    float scale = 1, water_weight = 0, exp_factor = 1;
    float chi = std::numeric_limits<float>::max();
    std::vector<float> intensity;
};

// All models in one librsx batch handle: each grid point of the fit is one
// graph-captured persistent pass over the whole ensemble (the reference runs
// one i_saxs::calc_curve per model).  The factor table follows the expansion
// factor (generated with the mean radius of the first model, as the
// reference's atomic_ff_params does) and the water weight enters with
// per-model rsasa from the dot-sphere SASA on the reference GPU algorithm's
// own dot map (create_dodeca_icosa_dots per atomic radius, probe 1.8 A:
// saxs_alg_cl_gpu_pt_wf.cpp:82-96, rsasa_cl_gpu_alg.cpp:60-89).
class Evaluator {
public:
    Evaluator(const std::vector<std::vector<rsx_body>> &models, const std::vector<float> &q,
              int device)
        : models_(models), q_(q), device_(device)
    {
        check(rsx_ff_avg_radius(models_[0].data(), (int)models_[0].size(), &avg_radius_));
        table_.resize(q_.size() * 16);
        check(rsx_ff_atomic_table(q_.data(), (int)q_.size(), avg_radius_, 1.0f, table_.data()));
        std::vector<int> sizes;
        for (const auto &m : models_) {
            sizes.push_back((int)m.size());
            bodies_.insert(bodies_.end(), m.begin(), m.end());
        }
        rsx_debye_options o;
        rsx_debye_default_options(&o);
        o.device = device_;
        check(rsx_batch_create(q_.data(), (int)q_.size(), table_.data(), 16, sizes.data(),
                               (int)sizes.size(), &o, &batch_));
        curves_.resize(models_.size() * q_.size());
    }
    ~Evaluator() { rsx_batch_destroy(batch_); }

    // avg_ensemble (calc_saxs.hpp:611-624): the mean of the models' curves,
    // summed in model order
    std::vector<float> average(float exp_factor, float water_weight)
    {
        ++calls;
        if (exp_factor != cur_ef_) {
            check(rsx_ff_atomic_table(q_.data(), (int)q_.size(), avg_radius_, exp_factor,
                                      table_.data()));
            check(rsx_batch_set_factors(batch_, table_.data(), 16));
            cur_ef_ = exp_factor;
        }
        if (water_weight != cur_ww_) {
            const float *rs = nullptr;
            if (water_weight != 0 && rsasa_.empty()) {
                compute_rsasa();
                rs = rsasa_.data();
            }
            check(rsx_batch_set_water(batch_, water_weight, rsx_ff_water_index(), rs));
            cur_ww_ = water_weight;
        }
        check(rsx_batch_forward(batch_, bodies_.data(), curves_.data()));
        std::vector<float> avg(q_.size(), 0.f);
        for (size_t m = 0; m < models_.size(); ++m)
            for (size_t k = 0; k < q_.size(); ++k)
                avg[k] += curves_[m * q_.size() + k];
        for (auto &v : avg)
            v /= models_.size();
        return avg;
    }

    unsigned calls = 0;

private:
    // rsasa of every model, concatenated in model order
    void compute_rsasa()
    {
        float radii[16];
        check(rsx_ff_radii(radii));
        std::vector<std::vector<float>> sets(16);
        int stride = 1;
        for (int t = 0; t < 16; ++t) {
            int n = 0;
            rsx_status st = rsx_sasa_sphere_dots(RSX_DOTS_DODECA_ICOSA, radii[t], 0.f, 1.8f,
                                                 nullptr, 0, &n);
            if (st != RSX_OK && n == 0)
                check(st);
            sets[t].resize(4 * (size_t)n);
            check(rsx_sasa_sphere_dots(RSX_DOTS_DODECA_ICOSA, radii[t], 0.f, 1.8f,
                                       sets[t].data(), n, &n));
            stride = std::max(stride, n);
        }
        std::vector<float> map(16 * (size_t)stride * 4, -std::numeric_limits<float>::infinity());
        for (int t = 0; t < 16; ++t)
            std::copy(sets[t].begin(), sets[t].end(), map.begin() + (size_t)t * stride * 4);
        rsasa_.resize(bodies_.size());
        size_t off = 0;
        for (const auto &m : models_) {
            rsx_sasa *s = nullptr;
            check(rsx_sasa_create_typed((int)m.size(), map.data(), 16, stride, radii, 1.8f,
                                        device_, &s));
            const rsx_status st = rsx_sasa_calc_typed(s, m.data(), rsasa_.data() + off);
            rsx_sasa_destroy(s);
            check(st);
            off += m.size();
        }
    }

    const std::vector<std::vector<rsx_body>> &models_;
    std::vector<float> q_;
    int device_;
    float avg_radius_ = 0;
    std::vector<float> table_;
    std::vector<rsx_body> bodies_;
    std::vector<float> curves_;
    rsx_batch *batch_ = nullptr;
    std::vector<float> rsasa_;
    float cur_ef_ = 1.0f, cur_ww_ = 0.0f;
};

struct ParamSpec {
    float lo, hi;
    bool fit;
};

Fit fit_point(Evaluator &ev, const Profile &ref, const ParamSpec &scale, float ef, float ww)
{
    Fit f;
    f.exp_factor = ef;
    f.water_weight = ww;
    f.intensity = ev.average(ef, ww);
    f.scale = scale.fit ? ref.optimize_scale_for(f.intensity) : scale.lo;
    for (auto &v : f.intensity)
        v *= f.scale;
    f.chi = ref.chi(f.intensity);
    return f;
}

// fit_ensemble grid search (calc_saxs.hpp:531-607)
Fit fit_ensemble(Evaluator &ev, const Profile &ref, const ParamSpec &scale, const ParamSpec &ef_p,
                 const ParamSpec &ww_p, Verbose verbose, size_t n_models)
{
    if (verbose >= NORMAL)
        std::cout << "Calculating ensemble average for " << n_models << " conformations." << std::endl;
    const float ef_eps = 0.0001f, ww_eps = 0.001f, chi_threshold = 0.00001f;
    const unsigned slices = 5, fixed = 0;
    unsigned ef_slices = ef_p.fit ? slices : fixed, ww_slices = ww_p.fit ? slices : fixed;
    float ef_min = ef_p.lo, ef_max = ef_p.hi, ww_min = ww_p.lo, ww_max = ww_p.hi;
    float ef_delta, ww_delta;
    Fit best;
    float prev_round_chi;
    bool reached = false;
    do {
        prev_round_chi = best.chi;
        ef_delta = (ef_max - ef_min) / std::max(ef_slices, 1u);
        ww_delta = (ww_max - ww_min) / std::max(ww_slices, 1u);
        for (unsigned i = 0; i <= ef_slices; ++i) {
            float prev_pt_chi = std::numeric_limits<float>::max();
            for (unsigned j = 0; j <= ww_slices; ++j) {
                Fit f = fit_point(ev, ref, scale, ef_min + i * ef_delta, ww_min + j * ww_delta);
                if (prev_pt_chi < f.chi)
                    break;
                prev_pt_chi = f.chi;
                if (f.chi < best.chi)
                    best = std::move(f);
            }
        }
        if (verbose >= DETAILS && best.chi < prev_round_chi)
            std::cout << "found min: # scale: " << best.scale << ", water weight: " << best.water_weight
                      << ", expansion factor: " << best.exp_factor << ", Chi: " << best.chi << std::endl;
        ef_slices = ef_delta > ef_eps ? slices : fixed;
        ww_slices = ww_delta > ww_eps ? slices : fixed;
        ef_delta = ef_delta > ef_eps ? ef_delta : 0;
        ww_delta = ww_delta > ww_eps ? ww_delta : 0;
        ef_min = std::max(best.exp_factor - ef_delta, ef_p.lo);
        ef_max = std::min(best.exp_factor + ef_delta, ef_p.hi);
        ww_min = std::max(best.water_weight - ww_delta, ww_p.lo);
        ww_max = std::min(best.water_weight + ww_delta, ww_p.hi);
        const float chi_delta = std::fabs(prev_round_chi - best.chi);
        reached = chi_delta / prev_round_chi < chi_threshold && chi_delta < 0.0001f;
    } while ((ef_delta > ef_eps || ww_delta > ww_eps) && !reached);
    if (verbose >= DETAILS)
        std::cout << ev.calls << " calculations." << std::endl;
    return best;
}

// device spec: cpu | gpu | host -> current CUDA device; P-D -> ordinal D
int device_from_spec(const std::string &spec)
{
    const auto dash = spec.find('-');
    if (dash != std::string::npos) {
        std::istringstream iss(spec.substr(dash + 1));
        int d;
        if (iss >> d)
            return d;
    }
    return -1;
}

} // namespace

int main(int argc, char **argv)
{
    Args a;
    try {
        a = parse_args(argc, argv);
    } catch (const CliError &e) {
        std::cerr << "PARSE ERROR: Argument: " << e.arg << "\n             " << e.msg << "\n\n";
        usage(std::cerr);
        return 1;
    }
    try {
        if (!a.water.singular() && a.fit.empty())
            throw CliError{"Range can't be used without an experimental profile; use a single value instead.", " "};
        if (!a.exp_factor.singular() && a.fit.empty())
            throw CliError{"Range can't be used without an experimental profile; use a single value instead.", " "};
        if (a.verbose >= NORMAL)
            std::cout << std::endl << "----- Calculating SAXS curve -----" << std::endl << std::endl;
        std::clock_t t1 = std::clock();
        // make_param (calc_saxs/main.cpp:156-171)
        const bool fitting = !a.fit.empty();
        ParamSpec scale{a.scale, a.scale, false};
        if (!a.scale_set && fitting)
            scale = {std::numeric_limits<float>::min(), std::numeric_limits<float>::max(), true};
        auto range_spec = [&](const Range &r) {
            const bool dflt = !r.set && fitting;
            ParamSpec p{dflt ? r.min_ : r.lo, dflt ? r.max_ : r.hi, true};
            if (p.lo == p.hi)
                p.fit = false;
            return p;
        };
        const ParamSpec ww = range_spec(a.water), ef = range_spec(a.exp_factor);
        const Profile ref = Profile::read(a.fit);

        std::vector<std::vector<rsx_body>> models;
        for (const auto &path : a.pdbs)
            for (auto &m : read_pdb(path, a.verbose))
                models.push_back(std::move(m));
        if (models.empty() || models[0].empty())
            throw RsxError{RSX_INVALID_ARG, "no atoms read from the PDB files"};
        for (const auto &m : models)
            if (m.size() != models[0].size())
                throw RsxError{RSX_INVALID_ARG,
                               "RESAXS::error -- different number of bodies expected in calc_curve()"};
        if (a.verbose > QUIET)
            std::cout << models[0].size() << " bodies generated." << std::endl;
        if (a.dbl && a.verbose > QUIET)
            std::cout << "note: librsx computes in FP32 with FP64 accumulation on the GPU" << std::endl;
        std::cout << std::endl
                  << "Preprocessing time: " << double(std::clock() - t1) * 1000 / CLOCKS_PER_SEC
                  << "ms" << std::endl
                  << std::endl;
        t1 = std::clock();

        std::vector<float> q = ref.q;
        if (q.empty()) {
            q.resize(a.q_n);
            // one q value is q_min (the reference divides by q_n - 1 = 0 there
            // and writes NaN, calc_saxs.cpp:60-62)
            const float step = (a.q_n > 1) ? (a.q_max - a.q_min) / (a.q_n - 1) : 0;
            for (unsigned i = 0; i < a.q_n; ++i)
                q[i] = a.q_min + i * step;
        }
        const int device = device_from_spec(a.device);
        Evaluator ev(models, q, device);
        Fit best = fit_ensemble(ev, ref, scale, ef, ww, a.verbose, models.size());
        std::cout << std::endl
                  << "SAXS calc time: " << double(std::clock() - t1) * 1000 / CLOCKS_PER_SEC << "ms"
                  << std::endl
                  << std::endl;

        std::ofstream out(a.out);
        out << "# scale: " << best.scale << ", water weight: " << best.water_weight
            << ", expansion factor: " << best.exp_factor << ", Chi: " << best.chi << std::endl;
        for (size_t i = 0; i < q.size(); ++i)
            out << std::fixed << q[i] << "     \t" << best.intensity[i] << std::endl;

        if (a.test) {
            // verify_result (calc_saxs.cpp:100-113): chi-square of the written
            // curve against the first model recomputed with expansion factor 1
            // and no water.  The reference recomputes on its FP64 host path;
            // here the second curve comes from the direct-sine kernels (no q
            // recurrence), an independent GPU evaluation.
            rsx_debye_options o;
            rsx_debye_default_options(&o);
            o.device = device;
            o.force_general_q = 1;
            o.no_pair_tables = 1; // per pair*q, not the gridded distribution
            std::vector<float> tab(q.size() * 16), host(q.size());
            check(rsx_ff_atomic_table(q.data(), (int)q.size(), 0.0f, 1.0f, tab.data()));
            rsx_debye *h = nullptr;
            check(rsx_debye_create(q.data(), (int)q.size(), tab.data(), 16, (int)models[0].size(), &o, &h));
            const rsx_status st = rsx_debye_calc(h, models[0].data(), host.data());
            rsx_debye_destroy(h);
            check(st);
            double chisq = 0;
            for (size_t i = 0; i < q.size(); ++i)
                chisq += double(best.intensity[i] - host[i]) * (best.intensity[i] - host[i]) / host[i];
            std::cout << "Chi square: " << chisq << std::endl;
        }
    } catch (const CliError &e) {
        std::cerr << "error: " << e.msg << " for arg " << e.arg << std::endl;
    } catch (const RsxError &e) {
        std::cerr << "ERROR: " << e.msg << "(" << e.code << ")" << std::endl;
        return -1;
    } catch (const std::exception &e) {
        std::cerr << "ERROR: " << e.what() << std::endl;
        return -1;
    }
    return 0;
}
