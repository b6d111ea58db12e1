// rsx/saxs_algorithm.hpp -- header-only C++ adapter over the librsx C ABI
// (include/rsx.h) with the shape of resaxslib's algorithm interface, so that
// C++ callers of the reference switch by changing includes and the factory:
//
//   reference (resaxslib/include/saxs_algorithm.hpp:118-244)   here
//   resaxs::algorithm::i_saxs<float, cl_base<float>>           rsx::algorithm::i_saxs<float>
//   saxs_params::initialize(qq, bodies, devices, wf)           same signature (devices: CUDA ordinals)
//   get_ff_params().access_factors() / set_water_ff_index     same
//   get_implicit_water_params().set_water_weight / access_rsasa same
//   initialize(); calc_curve(bodies, out); recalc_curve(...)   same
//   commit(); revert()                                         same
//   resaxs::error with codes -1..-6                            rsx::error, same codes
//   create_saxs_ocl<float>()                                   rsx::algorithm::create_saxs_gpu()
//   i_rsasa<float>::calc_rsasa / recalc_rsasa                  rsx::algorithm::rsasa_gpu
//
// Bodies are rsx_body (4 floats, the reference's cl_float4 layout with the
// uint32 type bits in .w; utils.hpp:61-88).
#ifndef RSX_SAXS_ALGORITHM_HPP
#define RSX_SAXS_ALGORITHM_HPP

#include "../rsx.h"

#include <algorithm>
#include <cstring>
#include <exception>
#include <limits>
#include <memory>
#include <string>
#include <vector>

namespace rsx {

// resaxs::error (resaxslib/include/resaxs.hpp:187-221)
class error : public std::exception {
public:
    enum code {
        SAXS_INVALID_DEVICE = RSX_INVALID_DEVICE,
        SAXS_ALG_NOT_INITIALIZED = RSX_ALG_NOT_INITIALIZED,
        SAXS_INVALID_ARG = RSX_INVALID_ARG,
        SAXS_PROGRAM_NOT_LOADED = RSX_PROGRAM_NOT_LOADED,
        SAXS_ARGS_NOT_SET = RSX_ARGS_NOT_SET,
        SAXS_NO_INITIAL_CALC = RSX_NO_INITIAL_CALC,
    };
    error(int err, std::string msg) : err_(err), msg_(std::move(msg)) {}
    const char *what() const noexcept override { return msg_.empty() ? "empty" : msg_.c_str(); }
    int err() const { return err_; }

private:
    int err_;
    std::string msg_;
};

inline void check(rsx_status s)
{
    if (s != RSX_OK)
        throw error(s, rsx_last_error());
}

inline void set_factor_index(rsx_body &b, unsigned index) { std::memcpy(&b.w, &index, 4); }
inline unsigned get_factor_index(const rsx_body &b)
{
    unsigned t;
    std::memcpy(&t, &b.w, 4);
    return t;
}

namespace algorithm {

// params_base (resaxslib/include/re_algorithm.hpp:66-89)
class params_base {
public:
    virtual ~params_base() = default;
    bool is_dirty() const { return dirty_; }
    void clear_dirty() { dirty_ = false; }

protected:
    void set_dirty() { dirty_ = true; }

private:
    bool dirty_ = false;
};

template <typename FLT_T> class implicit_water_params : public params_base {
public:
    FLT_T water_weight_ = 0;
    bool no_rsasa_recalc_ = false;
    void set_water_weight(FLT_T w)
    {
        if (water_weight_ != w) {
            water_weight_ = w;
            this->set_dirty();
        }
    }
    std::vector<FLT_T> &access_rsasa()
    {
        this->set_dirty();
        return rsasa_;
    }
    const std::vector<FLT_T> &rsasa() const { return rsasa_; }

private:
    std::vector<FLT_T> rsasa_;
};

template <typename FLT_T> class form_factor_params : public params_base {
public:
    std::vector<FLT_T> factors_; // row-major [n_q][n_factors]
    int water_ff_index_ = -1;
    FLT_T expansion_factor_ = 1;
    void set_water_ff_index(int index)
    {
        if (water_ff_index_ != index) {
            water_ff_index_ = index;
            this->set_dirty();
        }
    }
    std::vector<FLT_T> &access_factors()
    {
        this->set_dirty();
        return factors_;
    }
};

template <typename FLT_T> struct saxs_params : public params_base {
    std::vector<FLT_T> qq_;
    unsigned n_bodies_ = 0;
    int device_ = -1;
    unsigned workgroup_size_ = 64; // accepted for interface parity; tiles are fixed
    void initialize(const std::vector<FLT_T> &qq, const std::vector<rsx_body> &bodies,
                    const std::vector<int> &devices = {}, unsigned workgroup_size = 64)
    {
        qq_ = qq;
        n_bodies_ = (unsigned)bodies.size();
        device_ = devices.empty() ? -1 : devices.front();
        workgroup_size_ = workgroup_size;
        this->set_dirty();
    }
    form_factor_params<FLT_T> &get_ff_params() { return ff_; }
    implicit_water_params<FLT_T> &get_implicit_water_params() { return water_; }

private:
    form_factor_params<FLT_T> ff_;
    implicit_water_params<FLT_T> water_;
};

// i_saxs<float> (resaxslib/include/saxs_algorithm.hpp:147-183) over rsx_debye
// A typed rsx_sasa handle over the reference's per-type dot spheres for the
// 16 atomic radii (atomic_form_factors::calc_radii, ff_coef.hpp:164-188),
// padded with -inf dots as rsasa_cl_gpu::create_sphere_dots pads dots_map_.
inline rsx_sasa *create_atomic_sasa(int n_atoms, int dot_kind, float dot_density, float probe,
                                    int device)
{
    float radii[16];
    check(rsx_ff_radii(radii));
    std::vector<std::vector<float>> sets(16);
    int stride = 1;
    for (int t = 0; t < 16; ++t) {
        int n = 0;
        const rsx_status st =
            rsx_sasa_sphere_dots(dot_kind, radii[t], dot_density, probe, nullptr, 0, &n);
        if (st != RSX_OK && n == 0)
            check(st);
        sets[t].resize(4 * (size_t)n);
        check(rsx_sasa_sphere_dots(dot_kind, radii[t], dot_density, probe, sets[t].data(), n, &n));
        stride = std::max(stride, n);
    }
    const float pad = -std::numeric_limits<float>::infinity();
    std::vector<float> map(16 * (size_t)stride * 4, pad);
    for (int t = 0; t < 16; ++t)
        std::copy(sets[t].begin(), sets[t].end(), map.begin() + (size_t)t * stride * 4);
    rsx_sasa *h = nullptr;
    check(rsx_sasa_create_typed(n_atoms, map.data(), 16, stride, radii, probe, device, &h));
    return h;
}

template <typename FLT_T = float> class i_saxs {
    static_assert(sizeof(FLT_T) == 4, "librsx computes in FP32 with FP64 reductions");

public:
    i_saxs() = default;
    i_saxs(const i_saxs &) = delete;
    i_saxs &operator=(const i_saxs &) = delete;
    virtual ~i_saxs()
    {
        if (h_)
            rsx_debye_destroy(h_);
        if (sasa_)
            rsx_sasa_destroy(sasa_);
    }

    saxs_params<FLT_T> &access_params() { return params_; }

    void initialize()
    {
        if (params_.qq_.empty())
            throw error(error::SAXS_ARGS_NOT_SET, "saxs_params::initialize() was not called");
        auto &ff = params_.get_ff_params();
        if (ff.factors_.empty() || ff.factors_.size() % params_.qq_.size())
            throw error(error::SAXS_ARGS_NOT_SET, "form-factor table missing or malformed");
        if (h_)
            rsx_debye_destroy(h_);
        h_ = nullptr;
        if (sasa_)
            rsx_sasa_destroy(sasa_);
        sasa_ = nullptr;
        rsx_debye_options o;
        rsx_debye_default_options(&o);
        o.device = params_.device_;
        const int n_f = (int)(ff.factors_.size() / params_.qq_.size());
        check(rsx_debye_create(params_.qq_.data(), (int)params_.qq_.size(), ff.factors_.data(),
                               n_f, (int)params_.n_bodies_, &o, &h_));
        ff.clear_dirty();
        computing_ = false;
    }

    void calc_curve(const std::vector<rsx_body> &bodies, std::vector<FLT_T> &out_Iqq)
    {
        require(h_ != nullptr, error::SAXS_ARGS_NOT_SET, "initialize() was not called");
        require(bodies.size() == params_.n_bodies_, error::SAXS_INVALID_ARG,
                "different number of bodies expected in calc_curve()");
        // a full calculation always takes the current water parameters, dirty
        // or not, as the reference's calc_curve sets the weight argument on
        // every call (saxs_alg_cl_gpu_pt_wf.cpp:433-438); this also carries
        // them into a handle made by a later initialize()
        update_rsasa(bodies, true);
        push_params(true);
        out_Iqq.resize(params_.qq_.size());
        check(rsx_debye_calc(h_, bodies.data(), out_Iqq.data()));
        computing_ = true;
    }

    void recalc_curve(const std::vector<rsx_body> &bodies, unsigned upd_start, unsigned upd_length,
                      std::vector<FLT_T> &out_Iqq)
    {
        require(computing_, error::SAXS_NO_INITIAL_CALC,
                "recalc_curve() called before an initial call to calc_curve()");
        require(bodies.size() >= (size_t)upd_start + upd_length, error::SAXS_INVALID_ARG,
                "bodies vector too small in recalc_curve()");
        update_rsasa(bodies, upd_length > 0);
        push_params();
        out_Iqq.resize(params_.qq_.size());
        check(rsx_debye_recalc_range(h_, bodies.data(), upd_start, upd_length, out_Iqq.data()));
    }

    void commit()
    {
        require(computing_, error::SAXS_NO_INITIAL_CALC,
                "commit() called before an initial call to calc_curve()");
        check(rsx_debye_commit(h_));
    }

    void revert()
    {
        require(computing_, error::SAXS_NO_INITIAL_CALC,
                "revert() called before an initial call to calc_curve()");
        check(rsx_debye_revert(h_));
    }

    rsx_debye *handle() { return h_; }

private:
    static void require(bool c, int code, const char *msg)
    {
        if (!c)
            throw error(code, msg);
    }

    void push_params(bool water_always = false)
    {
        auto &ff = params_.get_ff_params();
        auto &w = params_.get_implicit_water_params();
        if (ff.is_dirty()) {
            const int n_f = (int)(ff.factors_.size() / params_.qq_.size());
            check(rsx_debye_set_factors(h_, ff.factors_.data(), n_f));
            ff.clear_dirty();
        }
        if (w.is_dirty() || water_always) {
            const int widx = ff.water_ff_index_ >= 0 ? ff.water_ff_index_ : 0;
            const auto &rs = w.rsasa();
            check(rsx_debye_set_water(h_, (float)w.water_weight_, widx,
                                      rs.size() >= params_.n_bodies_ ? rs.data() : nullptr));
            w.clear_dirty();
        }
    }

    // The water term's rsasa, as the reference's GPU algorithm keeps it
    // (saxs_alg_cl_gpu_pt_wf.cpp:82-96, 333-401): with a non-zero water
    // weight every update of the bodies recomputes rsasa from all bodies with
    // the reference's own OpenCL dot map (rsasa_cl_gpu_alg.cpp:60-89: the
    // create_dodeca_icosa_dots sphere of each of the 16 atomic radii, probe
    // 1.8 A), unless no_rsasa_recalc_ is set and rsasa values are present.
    // Values a caller wrote through access_rsasa() therefore survive only
    // with no_rsasa_recalc_ set (the reference overwrites them on the first
    // update in any case).
    void update_rsasa(const std::vector<rsx_body> &bodies, bool moved)
    {
        auto &w = params_.get_implicit_water_params();
        if (w.water_weight_ == 0)
            return;
        const size_t n = params_.n_bodies_;
        const bool present = w.rsasa().size() >= n;
        if (present && (w.no_rsasa_recalc_ || !moved))
            return;
        require(bodies.size() >= n, error::SAXS_INVALID_ARG,
                "the water term's SASA needs every body");
        for (size_t i = 0; i < n; ++i)
            require(get_factor_index(bodies[i]) < 16, error::SAXS_INVALID_ARG,
                    "the water term's SASA needs an atomic type (0..15) on every body");
        if (!sasa_)
            sasa_ = create_atomic_sasa((int)n, RSX_DOTS_DODECA_ICOSA, 0.f, 1.8f, params_.device_);
        auto &rs = w.access_rsasa(); // marks the water params dirty: pushed next
        rs.resize(n);
        check(rsx_sasa_calc_typed(sasa_, bodies.data(), rs.data()));
    }

    saxs_params<FLT_T> params_;
    rsx_debye *h_ = nullptr;
    rsx_sasa *sasa_ = nullptr;
    bool computing_ = false;
};

// create_saxs_ocl<float>() (saxs_algorithm.hpp:240-244) counterpart
inline std::unique_ptr<i_saxs<float>> create_saxs_gpu() { return std::make_unique<i_saxs<float>>(); }

// i_rsasa<float> (resaxslib/include/rsasa_algorithm.hpp:42-61) over rsx_sasa.
// initialize(n_atoms, dot_spheres_params) builds the reference's own per-type
// dot map for the 16 atomic radii (atomic_form_factors::calc_radii): the
// create_dodeca_icosa_dots spheres of rsasa_cl_gpu (rsasa_cl_gpu_alg.cpp:60-89)
// by default, or the create_dots spheres of rsasa_cpu_alg
// (rsasa_cpu_alg.cpp:46-61) with RSX_DOTS_LATITUDE.  The other initialize()
// takes one unit dot set and a radius per body type.
struct dot_spheres_params {
    float dot_density = 0.f;  // dots per A^2 (create_dots)
    float probe_radius = 0.f;
    dot_spheres_params() = default;
    dot_spheres_params(float density, float probe) : dot_density(density), probe_radius(probe) {}
};

class rsasa_gpu {
public:
    ~rsasa_gpu()
    {
        if (h_)
            rsx_sasa_destroy(h_);
    }
    void initialize(unsigned n_atoms, const dot_spheres_params &p,
                    int dot_kind = RSX_DOTS_DODECA_ICOSA, int device = -1)
    {
        release();
        h_ = create_atomic_sasa((int)n_atoms, dot_kind, p.dot_density, p.probe_radius, device);
        typed_ = true;
    }
    void initialize(unsigned n_atoms, const std::vector<float> &radius_of_type, float probe_radius,
                    const std::vector<float> &unit_dots, int device = -1)
    {
        release();
        radii_ = radius_of_type;
        check(rsx_sasa_create((int)n_atoms, unit_dots.data(), (int)(unit_dots.size() / 3),
                              probe_radius, device, &h_));
        typed_ = false;
    }
    void calc_rsasa(const std::vector<rsx_body> &atoms, std::vector<float> &rsasa)
    {
        if (!h_)
            throw error(error::SAXS_ARGS_NOT_SET, "initialize() was not called");
        if (rsasa.size() < atoms.size())
            throw error(error::SAXS_INVALID_ARG, "rsasa vector too small");
        if (typed_) {
            check(rsx_sasa_calc_typed(h_, atoms.data(), rsasa.data()));
        } else {
            std::vector<float> r(atoms.size());
            for (size_t i = 0; i < atoms.size(); ++i) {
                const unsigned t = get_factor_index(atoms[i]);
                if (t >= radii_.size())
                    throw error(error::SAXS_INVALID_ARG, "atom type without a radius");
                r[i] = radii_[t];
            }
            check(rsx_sasa_calc(h_, atoms.data(), r.data(), rsasa.data()));
        }
        computing_ = true;
    }
    void recalc_rsasa(const std::vector<rsx_body> &atoms, std::vector<float> &rsasa)
    {
        if (!computing_)
            throw error(error::SAXS_NO_INITIAL_CALC, "recalc_rsasa() before calc_rsasa()");
        calc_rsasa(atoms, rsasa);
    }

private:
    void release()
    {
        if (h_)
            rsx_sasa_destroy(h_);
        h_ = nullptr;
        computing_ = false;
    }
    rsx_sasa *h_ = nullptr;
    std::vector<float> radii_;
    bool typed_ = false;
    bool computing_ = false;
};

} // namespace algorithm
} // namespace rsx

#endif
