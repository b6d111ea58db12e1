// C entry points over the reference's own host_debye templates
// (resaxslib/src/host_debye.cpp:54-109, resaxslib/include/host_debye.hpp:30-40),
// compiled together with that unmodified source file into oracle/_ref/.
// Test infrastructure only: the product never loads it.
#include "host_debye.hpp"

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
