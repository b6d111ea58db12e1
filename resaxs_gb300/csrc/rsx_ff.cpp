// Form-factor tables (host C++): the step before the Debye kernels in the
// reference's CLI.  Implements the physics of resaxslib/include/ff_coef.hpp
// and constants.hpp for the 16 atom types of the reference:
//
//   f(q) = f_vacuum(k) - f_excluded(k) * E(k),   k = q / (4 pi)
//   f_vacuum  = c + sum_{i=1..4} a_i exp(-b_i k^2)            (Cromer & Mann 1968)
//   f_excluded = rho V exp(-pi V^(2/3) k^2)                   (Fraser, MacRae & Suzuki 1978)
//   E(k) = c_x^3 exp(-pi (4 pi / 3)^(2/3) k^2 r_m^2 (c_x^2 - 1))  (expansion factor c_x, mean radius r_m)
//   complex groups (CH, CH2, ...) = simple atom + n_H * f(H)
//   radius of a type = (3 / (4 pi rho) * f_excluded(0))^(1/3)
//
// computed in FP32 in the reference's order of operations.  The reference
// calls exp and pow unqualified from a header that includes <cmath> only, so
// they resolve to the C double-precision functions; the same calls are made
// here, which keeps the tables bit-identical to the reference's on the same
// C library.
#include "rsx_host.h"

#include <cmath>
#include <cstring>

namespace {

constexpr int kSimple = 7;
constexpr int kTypes = 16;
constexpr float kRho = 0.334f; // e/A^3, water

// Cromer-Mann coefficients a1..a4, c, b1..b4 of H, C, N, O, P, S, Zn (the
// published table the reference uses, resaxslib/include/ff_coef.hpp:39-48)
const float kCromerMann[kSimple][9] = {
    {0.4930020f, 0.3229120f, 0.1401910f, 4.0810000E-02f, 3.0380001E-03f, 10.51090f, 26.12570f,
     3.142360f, 57.79970f},
    {2.310000f, 1.020000f, 1.588600f, 0.8650000f, 0.2156000f, 20.84390f, 10.20750f, 0.5687000f,
     51.65120f},
    {12.21260f, 3.132200f, 2.012500f, 1.166300f, -11.52900f, 5.7000001E-03f, 9.893300f,
     28.99750f, 0.5826000f},
    {3.048500f, 2.286800f, 1.546300f, 0.8670000f, 0.2508000f, 13.27710f, 5.701100f, 0.3239000f,
     32.90890f},
    {6.434500f, 4.179100f, 1.780000f, 1.490800f, 1.114900f, 1.906700f, 27.15700f, 0.5260000f,
     68.16450f},
    {6.905300f, 5.203400f, 1.437900f, 1.586300f, 0.8669000f, 1.467900f, 22.21510f, 0.2536000f,
     56.17200f},
    {14.07430f, 7.031800f, 5.165200f, 2.410000f, 1.304100f, 3.265500f, 0.2333000f, 10.31630f,
     58.70970f},
};

// excluded volumes in A^3 (resaxslib/include/constants.hpp:61-69)
const float kExclVolume[kSimple] = {5.15f, 16.44f, 2.49f, 9.13f, 5.73f, 19.86f, 9.85f};

// complex groups: base simple type and number of hydrogens (constants.hpp:71-81)
const unsigned kComplex[kTypes - kSimple][2] = {{1, 1}, {1, 2}, {1, 3}, {2, 1}, {2, 2},
                                                {2, 3}, {3, 1}, {3, 2}, {5, 1}};

const float kPi = (float)3.14159265358979323846;

float vacuum_ff(int t, float k_sq)
{
    const float *c = kCromerMann[t];
    float r = c[4];
    for (int i = 0; i < 4; ++i)
        r += c[i] * ::exp((double)(-c[5 + i] * k_sq));
    return r;
}

float excluded_ff(int t, float k_sq)
{
    return kRho * kExclVolume[t] * ::exp(-kPi * ::pow((double)kExclVolume[t], (double)(2.0f / 3.0f)) * k_sq);
}

float expansion(float c, float k_sq, float rm)
{
    const float c_sq = c * c;
    static const float four_thirds_pi = ::pow((double)(4 * kPi / 3), (double)(2.0f / 3.0f));
    return c_sq * c * ::exp((double)(-kPi * four_thirds_pi * k_sq * rm * rm * (c_sq - 1)));
}

} // namespace

extern "C" {

int rsx_ff_type_count(void) { return kTypes; }
int rsx_ff_water_index(void) { return 14; } // OH2

rsx_status rsx_ff_atomic_table(const float *q, int n_q, float avg_radius, float expansion_factor,
                               float *out)
{
    if (!q || !out || n_q <= 0)
        return rsx::fail(RSX_INVALID_ARG, "q / output null or n_q <= 0");
    if (!std::isfinite(avg_radius) || !std::isfinite(expansion_factor))
        return rsx::fail(RSX_INVALID_ARG, "radius and expansion factor must be finite");
    for (int i = 0; i < n_q; ++i) {
        float *page = out + (size_t)i * kTypes;
        const float k = q[i] / (4 * kPi);
        const float k_sq = k * k;
        const float e = expansion_factor != 1 ? expansion(expansion_factor, k_sq, avg_radius) : 1.0f;
        for (int t = 0; t < kSimple; ++t)
            page[t] = vacuum_ff(t, k_sq) - excluded_ff(t, k_sq) * e;
        const float fh = page[0];
        for (int t = kSimple; t < kTypes; ++t)
            page[t] = page[kComplex[t - kSimple][0]] + kComplex[t - kSimple][1] * fh;
    }
    return rsx::ok();
}

rsx_status rsx_ff_radii(float *out)
{
    if (!out)
        return rsx::fail(RSX_INVALID_ARG, "output is null");
    float ff[kTypes];
    for (int t = 0; t < kSimple; ++t)
        ff[t] = excluded_ff(t, 0.0f);
    for (int t = kSimple; t < kTypes; ++t)
        ff[t] = ff[kComplex[t - kSimple][0]] + kComplex[t - kSimple][1] * ff[0];
    const float coef = static_cast<float>(3.0 / (4.0 * 3.14159265358979323846 * kRho));
    for (int t = 0; t < kTypes; ++t)
        out[t] = std::pow(coef * ff[t], static_cast<float>(1.0 / 3));
    return rsx::ok();
}

rsx_status rsx_ff_avg_radius(const rsx_body *bodies, int n, float *out)
{
    if (!out || (n > 0 && !bodies) || n <= 0)
        return rsx::fail(RSX_INVALID_ARG, "need bodies and n > 0");
    float radii[kTypes];
    rsx_ff_radii(radii);
    float sum = 0.f;
    for (int i = 0; i < n; ++i) {
        unsigned t;
        std::memcpy(&t, &bodies[i].w, 4);
        if (t >= (unsigned)kTypes)
            return rsx::fail(RSX_INVALID_ARG, "body type outside the 16 atom types");
        sum += radii[t];
    }
    *out = sum / n;
    return rsx::ok();
}

} // extern "C"
