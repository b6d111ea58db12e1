/*
 * rsx.h -- C ABI of librsx, the GB300-native (sm_103a) Debye / incremental
 * recalculation / dot-sphere SASA path of resaxslib.
 *
 * Plain C types only: pointers to host memory, sizes and int status codes.
 * Every entry point names the reference interface it replaces
 * (paths relative to the ldantonov/resaxs tree).
 *
 * Body layout (same bytes as the reference's cl_float4 bodies,
 * resaxslib/include/utils.hpp:61-88): 4 floats per body, x y z and the
 * uint32 form-factor type index stored bit-for-bit in the 4th float.
 * Form-factor tables are row-major [n_q][n_factors]
 * (resaxslib/src/host_debye.cpp:64-72).
 *
 * Threading: a handle is used by one host thread at a time; each handle owns
 * one CUDA stream on one device.  All calls that take host output pointers
 * return after the result is in host memory.
 */
#ifndef RSX_H
#define RSX_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RSX_VERSION_MAJOR 1
#define RSX_VERSION_MINOR 0

/* Status codes.  -1..-6 are the reference's resaxs::error codes
 * (resaxslib/include/resaxs.hpp:212-220) with the same meaning. */
typedef int rsx_status;
#define RSX_OK 0
#define RSX_INVALID_DEVICE -1      /* no usable CUDA device / wrong device */
#define RSX_ALG_NOT_INITIALIZED -2 /* handle not created / destroyed */
#define RSX_INVALID_ARG -3         /* bad pointer, size, index or type */
#define RSX_PROGRAM_NOT_LOADED -4  /* kernels not available for this GPU */
#define RSX_ARGS_NOT_SET -5        /* required parameters missing */
#define RSX_NO_INITIAL_CALC -6     /* recalc/commit/revert/backward before calc */
#define RSX_CUDA_ERROR -100        /* a CUDA runtime call failed */
#define RSX_OUT_OF_MEMORY -101     /* device or pinned allocation failed */
#define RSX_TIMEOUT -102           /* a bounded device-side wait gave up */
#define RSX_NOT_SUPPORTED -103     /* valid request this build does not implement */
#define RSX_INJECTED_FAULT -104    /* failure produced by the host fault-injection hook */
#define RSX_PDB_FILE_NOT_FOUND -1100 /* SAXS_PDB_FILE_NOT_FOUND (resaxslib/include/parse_pdb.hpp:30) */

/* Body as 4 floats (x, y, z, type bits). */
typedef struct rsx_body {
    float x, y, z, w;
} rsx_body;

/* Library-level calls ------------------------------------------------- */

/* "major.minor cuda-runtime device" string; never NULL. */
const char *rsx_version(void);
/* Message of the last failing call on this host thread ("" if none). */
const char *rsx_last_error(void);
/* Kernels launched by this process through librsx so far. */
unsigned long long rsx_launch_count(void);
/* Host-side fault injection for tests: the n-th subsequent device allocation
 * or kernel launch inside librsx (counting from 1) fails with
 * RSX_INJECTED_FAULT; 0 disables.  kind: 0 = allocation, 1 = launch. */
void rsx_debug_inject_fault(int kind, int nth);

/* Host-only check of the device layout librsx derives from the body types
 * (type-sorted block tiles of <= 128 bodies, upper-triangle work items with
 * at most max_items items): counts, and *pairs_covered_ok = 1 when every block
 * pair (bi <= bj) is covered exactly once.  Touches no GPU; for tests. */
rsx_status rsx_debug_layout(const rsx_body *bodies, int n_bodies, int n_factors, int max_items,
                            int min_adj_items, int *n_blocks, int *n_items, int *n_adj_items,
                            int *pairs_covered_ok);

/* Host-only view of the small-angle level the kernels are chosen by, for a
 * q grid (uniform or not) with step dq over bodies whose bounding-box
 * diagonal is diag: 2 when |dq| * diag * 1.0001 <= 0.7 (|theta| < pi/4 for
 * every pair), 1 when it is <= 1.4 (|theta / 2| < pi/4), else 0. */
int rsx_debug_theta_level(int uniform, double dq, double diag);

/* Host-only view of the slab plan of the wide uniform kernels for n_q q and
 * q_slab 64 or 128: out[0..4] = main slab width, number of main slabs, first
 * q of the remainder slab, q it covers, width of its kernel (0: none). */
rsx_status rsx_debug_wide_plan(int n_q, int q_slab, int *out);

/* Host-only view of the chain plan of the uniform forward (q_slab 192, no
 * water) over n_q q: out[0..4] = chains of two 192-q slabs from the first q,
 * first q of the rest chain, its 192-q slabs, its tail slab's width (8 for a
 * remainder of 1..8 q, else a multiple of 16; 0 for none), 1 if there is a
 * rest chain.  A grid that starts at q = 0 is planned over the n_q - 1 q past
 * it (I(0) needs no pair sums). */
rsx_status rsx_debug_chain_plan(int n_q, int *out);

/* Host-only check of the shard split used by rsx_debye_calc_shard: item
 * bounds[0..n_shards] (shard s = items [bounds[s], bounds[s+1])) and, if
 * pairs is not NULL, the body pairs of each shard. */
rsx_status rsx_debug_shard_items(const rsx_body *bodies, int n_bodies, int n_factors,
                                 int max_items, int n_shards, int *bounds, double *pairs);

/* Host-only view of the autotuning cache (the tile-shape winners, loaded once
 * from the file named by RSX_AUTOTUNE_CACHE when it is set): 1 and *q_slab
 * when `key` has an entry, else 0.  The value is q_slab + 1000 when the wide
 * main slabs step four pairs at a time; lines of the file whose value is not
 * a shape librsx has kernels for (8, 16, 32, 64, 128, 192, 1128, 1192) are
 * ignored. */
int rsx_debug_autotune_lookup(const char *key, int *q_slab);

/* Measures the sustained FP32 FMA rate of `device` (-1 = current) with a
 * register-resident FMA-chain kernel on every SM: *fma_per_s = lane FMAs per
 * second.  The denominator of the pair*q roofline. */
rsx_status rsx_measure_fp32_fma_rate(int device, double *fma_per_s);

/* C-style function-pointer ABI: same signature and semantics as
 * resaxs::CalcSaxsCurveFn (resaxslib/include/host_debye.hpp:30), i.e.
 * host_debye<...>::calc_curve (resaxslib/src/host_debye.cpp:54-109), computed
 * on the current CUDA device.  Errors are reported through rsx_last_error()
 * (the reference signature has no status); out_v_Iq is left untouched then. */
void rsx_calc_saxs_curve(const float *v_q, int n_q, const rsx_body *v_bodies, int n_bodies,
                         const float *t_factors, int n_factors, float *out_v_Iq);
/* Same computation returning a status. */
rsx_status rsx_calc_saxs_curve_status(const float *v_q, int n_q, const rsx_body *v_bodies,
                                      int n_bodies, const float *t_factors, int n_factors,
                                      float *out_v_Iq);

/* Debye curve without any device allocation, for callers that cannot
 * allocate: code running inside a host framework that owns all device memory
 * through its own pool and forbids cudaMalloc from plug-ins, or work queued on
 * a stream whose scheduler must see no allocator calls.  No counterpart in the
 * reference.  All pointers are DEVICE pointers the caller owns: d_q (n_q
 * floats), d_bodies (n_bodies bodies, caller order), d_factors
 * ([n_q][n_factors]) and d_out_iq (n_q floats); `stream` is a cudaStream_t
 * (NULL = legacy default stream) on the current device.  Same sum as
 * rsx_calc_saxs_curve, to the same 1e-5 tolerance, but several times slower
 * (caller-order bodies, one range-reduced sine per pair and q).
 * Working memory is one static 8 MiB device array per GPU that loads librsx,
 * held until process exit; problems need ceil(n_bodies/128) * n_q <= 1048544
 * (larger ones are rejected with RSX_INVALID_ARG before any launch).
 * The first call on a device looks up that array's device address (with the
 * device current), and so does the first call after the device's context was
 * recreated (cudaDeviceReset).  Every call reuses the array and leaves its
 * contents behind; calls on the same device that overlap on the GPU (several
 * streams or threads) race on it and must be serialised by the caller (each
 * device has its own array).  Returns after the stream finished the call (the error word of the
 * array is read back with a synchronisation of `stream`). */
rsx_status rsx_calc_saxs_curve_device_noalloc(const float *d_q, int n_q, const rsx_body *d_bodies,
                                              int n_bodies, const float *d_factors, int n_factors,
                                              float *d_out_iq, void *stream);

/* Debye algorithm handle: replaces resaxs::algorithm::i_saxs<float, cl_base>
 * implemented by saxs_cl_gpu<float> (resaxslib/include/saxs_algorithm.hpp:147-183,
 * resaxslib/src/saxs_alg_cl_gpu_pt_wf.cpp) ----------------------------- */

typedef struct rsx_debye rsx_debye;

typedef struct rsx_debye_options {
    int device;          /* CUDA ordinal; -1 = current device */
    int q_slab;          /* q values per CTA slab: 8, 16, 32, 64, 128 or 192; 0 = tuned /
                            default (192 on uniform grids of 64 q or more).  On
                            uniform grids 64, 128 and 192 select the wide slabs
                            (64, up to 128, or up to 192 q per recurrence seed);
                            192 runs the forward without water as chains of up
                            to two 192-q slabs and a tail on one seed per pair
                            (with pairs_per_step 4: 192-q slabs); the other
                            kernels take at most 128. */
    int max_items;       /* cap on forward work items (scratch = items*n_q*8 B); 0 = default */
    int force_general_q; /* 1: never use the uniform-grid recurrence */
    int timing;          /* 1: record CUDA events around the pair kernel */
    int autotune;        /* 1: time the tile shapes (q-slab plan x pairs per step) on first
                            use and cache the winner per problem class */
    int no_pair_tables;  /* 1: evaluate every pair*q term instead of the tabulated pair
                            functions (adjoint) and the gridded pair-distance distribution
                            (forward on non-uniform grids): the recurrence adjoint and the
                            direct-sine forward, at their pair*q cost */
    int pairs_per_step;  /* pairs a thread steps together in the wide forward's main
                            slabs of 128 q or more: 2 or 4; 0 = tuned / default (2) */
} rsx_debye_options;

/* Forgets every autotuned tile choice of this process (the file named by
 * RSX_AUTOTUNE_CACHE, if any, is not reloaded afterwards). */
void rsx_autotune_clear(void);

/* Fills the defaults (device -1, everything else 0). */
void rsx_debye_default_options(rsx_debye_options *opts);

/* saxs_params::initialize(qq, bodies, devices, wf) + saxs_cl_gpu::initialize()
 * (saxs_algorithm.hpp:124-132; saxs_alg_cl_gpu_pt_wf.cpp:176-263): q vector,
 * form-factor table [n_q][n_factors] and body count are fixed for the handle.
 * opts may be NULL. */
rsx_status rsx_debye_create(const float *q, int n_q, const float *t_factors, int n_factors,
                            int n_bodies, const rsx_debye_options *opts, rsx_debye **out);
/* delete of the algorithm object (re_algorithm.hpp:33). NULL is a no-op. */
rsx_status rsx_debye_destroy(rsx_debye *h);

/* form_factor_params::access_factors()/set_expansion_factor() then a dirty
 * params flag (saxs_algorithm.hpp:79-109; saxs_alg_cl_gpu_pt_wf.cpp:479-495):
 * replaces the table; the next recalc does a full recompute. */
rsx_status rsx_debye_set_factors(rsx_debye *h, const float *t_factors, int n_factors);

/* implicit_water_params (saxs_algorithm.hpp:55-77) + water_ff_index:
 * f_i(q) = F[q][t_i] + rsasa_i * F[q][water_index] * weight
 * (gpu_saxs_pt_wf.cl:130-138).  rsasa (n_bodies floats, caller order) may be
 * NULL to keep the current values (initially 0).  Marks params dirty. */
rsx_status rsx_debye_set_water(rsx_debye *h, float weight, int water_index, const float *rsasa);

/* i_saxs::calc_curve (saxs_algorithm.hpp:162; saxs_alg_cl_gpu_pt_wf.cpp:414-458):
 * full I(q) of n_bodies bodies. */
rsx_status rsx_debye_calc(rsx_debye *h, const rsx_body *bodies, float *out_iq);

/* One shard of the full forward, for sharding one structure over ranks (no
 * reference counterpart; the reference runs one device per structure).  The
 * forward work items are split into n_shards contiguous runs balanced by pair
 * count; shard `shard` computes its run and writes its additive FP64
 * contribution to I(q) (shard 0 also carries the self terms and I(0)), so the
 * sum over shards -- one all-reduce of n_q doubles -- is the curve of
 * rsx_debye_calc.  Afterwards recalc needs a full rsx_debye_calc first. */
rsx_status rsx_debye_calc_shard(rsx_debye *h, const rsx_body *bodies, int shard, int n_shards,
                                double *out_iq);

/* i_saxs::recalc_curve (saxs_algorithm.hpp:172; saxs_alg_cl_gpu_pt_wf.cpp:468-577):
 * bodies is the full caller vector; bodies [upd_start, upd_start+upd_length)
 * moved.  Computed incrementally (delta of the moved pairs, FP64 running
 * totals); a full recompute when params are dirty or most bodies moved. */
rsx_status rsx_debye_recalc_range(rsx_debye *h, const rsx_body *bodies, unsigned upd_start,
                                  unsigned upd_length, float *out_iq);

/* Incremental recalc for an arbitrary moved set (no reference counterpart;
 * the reference accepts one contiguous range only): moved[m] is the new body
 * of caller index idx[m]; indices must be distinct and types unchanged. */
rsx_status rsx_debye_recalc_indices(rsx_debye *h, const rsx_body *moved, const unsigned *idx,
                                    unsigned k, float *out_iq);

/* i_saxs::commit / revert (saxs_algorithm.hpp:177-182;
 * saxs_alg_cl_gpu_pt_wf.cpp:592-620): checkpoint / restore positions, water
 * factors and the FP64 running curve.  revert before any commit is a no-op,
 * as in the reference. */
rsx_status rsx_debye_commit(rsx_debye *h);
rsx_status rsx_debye_revert(rsx_debye *h);

/* FP64 running curve held on the device (after calc/recalc). */
rsx_status rsx_debye_curve_f64(rsx_debye *h, double *out_iq);

/* Recompute I(q) from the bodies already on the device (no host copies),
 * leaving the result on the device; used to time the resident path.
 * rsx_debye_sync waits for it. */
rsx_status rsx_debye_forward_resident(rsx_debye *h);
rsx_status rsx_debye_sync(rsx_debye *h);

/* The handle's cudaStream_t (as an opaque pointer) for callers that record
 * their own events or order their own work against librsx. */
void *rsx_debye_stream(rsx_debye *h);

/* Milliseconds of the last pair kernel and of the last whole call, measured
 * with CUDA events on the handle's stream (options.timing = 1). */
rsx_status rsx_debye_timing(rsx_debye *h, float *ms_pair_kernel, float *ms_call);

/* Adjoint (no reference counterpart): given dL/dI(q) (n_q floats) for the
 * curve of the last calc/recalc, writes dL/dx for every body
 * (n_bodies x 3 floats, caller order) in one pair pass. */
rsx_status rsx_debye_backward(rsx_debye *h, const float *dl_diq, float *grad_xyz);

/* Same as rsx_debye_backward with the FP64 gradient. */
rsx_status rsx_debye_backward_f64(rsx_debye *h, const float *dl_diq, double *grad_xyz);

/* chi^2 = sum_q ((I(q) - target(q)) / sigma(q))^2 of the current curve and its
 * gradient dchi^2/dx (the loss of saxs_profile::chi_square_chi,
 * resaxslib/include/saxs_profile.hpp:154-166, with unit scale). */
rsx_status rsx_debye_chi2_backward(rsx_debye *h, const float *target, const float *sigma,
                                   double *chi2, float *grad_xyz);

/* Tuning in effect: q-slab, work items, whether the uniform-q recurrence is used. */
/* Tile shape of the forward (the q-slab option in effect and the pairs per
 * step of the wide main slabs), after autotuning when it was requested.  No
 * reference counterpart (the reference's tile is its fixed GROUP_SIZE,
 * saxs_alg_cl_gpu_pt_wf.cpp:203-207). */
rsx_status rsx_debye_tile_shape(rsx_debye *h, int *q_slab, int *pairs_per_step);
rsx_status rsx_debye_config(rsx_debye *h, int *q_slab, int *n_items, int *uniform_q);

/* Form-factor tables (host side, no GPU): resaxs::atomic_form_factors<float>
 * (resaxslib/include/ff_coef.hpp:104-212) for the reference's 16 atom types
 * H C N O P S Zn CH CH2 CH3 NH NH2 NH3 OH OH2 SH (constants.hpp:37-59). ---- */

/* Number of atom types (16) and the index of the water group OH2 (14). */
int rsx_ff_type_count(void);
int rsx_ff_water_index(void);
/* atomic_form_factors::generate(v_q, avg_radius, c, t_factors)
 * (ff_coef.hpp:112-162): out is [n_q][16], vacuum minus excluded-volume
 * factors with expansion factor c (1 = none). */
rsx_status rsx_ff_atomic_table(const float *q, int n_q, float avg_radius, float expansion_factor,
                               float *out);
/* atomic_form_factors::calc_radii (ff_coef.hpp:164-188): 16 radii in A. */
rsx_status rsx_ff_radii(float *out);
/* atomic_form_factors::calc_avg_radius (ff_coef.hpp:190-198). */
rsx_status rsx_ff_avg_radius(const rsx_body *bodies, int n, float *out);

/* PDB input of calc_saxs: parse_pdb<float>::all_models_as_complex_atoms
 * (resaxslib/include/parse_pdb.hpp:36-53, resaxslib/src/parse_pdb.cpp:63-108,
 * 309-363).  Every model of the file as complex-atom bodies: waters, hydrogens
 * and alternate locations other than ' '/'A' are dropped, atoms get their
 * group type (CH, NH2, ...) from the reference's atom tables.  rsx_pdb_count
 * gives the sizes; rsx_pdb_read writes the models back to back into out and
 * their body counts into model_sizes.  verbose >= 1 prints the reference's
 * warning for unknown elements on stderr.  A missing file returns
 * RSX_PDB_FILE_NOT_FOUND. */
rsx_status rsx_pdb_count(const char *path, int *n_models, int *n_bodies);
rsx_status rsx_pdb_read(const char *path, int verbose, rsx_body *out, int cap_bodies,
                        int *model_sizes, int max_models);

/* Dot-sphere SASA: replaces resaxs::algorithm::i_rsasa<float,float,cl_base>
 * implemented by rsasa_cl_gpu (resaxslib/include/rsasa_algorithm.hpp:42-61,
 * resaxslib/src/rsasa_cl_gpu_alg.cpp, kernel rsasa_dot_spheres.cl:94-163) ---- */

typedef struct rsx_sasa rsx_sasa;

/* Unit dots of create_fibonacci_dots (resaxslib/src/rsasa_algorithm.cpp:96-116)
 * with n = n_dots/2 (n_dots even): out_xyz is n_dots x 3 FP32, the factors the
 * reference multiplies by (radius + probe). */
rsx_status rsx_sasa_fibonacci_dots(int n_dots, float *out_xyz);
/* The 32 unit directions of create_dodeca_icosa_dots
 * (rsasa_algorithm.cpp:156-208), the reference GPU path's dot set: 32 x 3. */
rsx_status rsx_sasa_dodeca_icosa_dots(float *out_xyz);

/* The reference's dot spheres, pre-scaled for one atom radius:
 * dot_spheres_params::create_dots / create_32_dots / create_fibonacci_dots /
 * create_dodecahedron_dots / create_dodeca_icosa_dots
 * (resaxslib/src/rsasa_algorithm.cpp:60-208), the same FP32 values.  Each dot
 * is x, y, z (on the sphere of radius + probe) and w = radius.  *n_out gets
 * the set's size; RSX_INVALID_ARG when it exceeds cap (or dot_density < 0 for
 * the latitude set, whose size is about 4 pi r^2 density). */
#define RSX_DOTS_LATITUDE 0      /* create_dots: rsasa_cpu_alg's set (density) */
#define RSX_DOTS_32 1            /* create_32_dots */
#define RSX_DOTS_FIBONACCI 2     /* create_fibonacci_dots: 64 dots */
#define RSX_DOTS_DODECAHEDRON 3  /* create_dodecahedron_dots: 20 dots */
#define RSX_DOTS_DODECA_ICOSA 4  /* create_dodeca_icosa_dots: 32 dots, rsasa_cl_gpu's set */
rsx_status rsx_sasa_sphere_dots(int kind, float radius, float dot_density, float probe,
                                float *out_xyzw, int cap, int *n_out);

/* rsasa_cl_gpu::initialize(dot_spheres_cl_params) (rsasa_cl_gpu_alg.cpp:38-57):
 * atom count (at most 2^28), unit dot set (n_dots <= 4096, finite) and probe
 * radius fixed per handle.  Dot k of atom i sits at p_i + unit_k * (r_i + P).
 * A call checks the atoms (finite positions; radii >= 0 and finite, or types
 * inside the dot map) on the GPU with the bounding box and reports the first
 * bad atom with RSX_INVALID_ARG. */
rsx_status rsx_sasa_create(int n_atoms, const float *unit_dots, int n_dots, float probe,
                           int device, rsx_sasa **out);
/* The reference's own dot layout: rsasa_cl_gpu::create_sphere_dots
 * (rsasa_cl_gpu_alg.cpp:59-89) builds dots_map_[type * 32 + dot] from
 * pre-scaled per-type dot spheres padded with -inf dots, and
 * rsasa_cpu_alg::create_sphere_dots (rsasa_cpu_alg.cpp:46-61) keeps one
 * pre-scaled set per type.  dot_map holds n_types x stride dots as x, y, z,
 * w (w unused); a dot whose x is not finite is padding.  Dot k of an atom of
 * type t sits at p_i + dot_map[t][k] (FP32 add, rsasa_dot_spheres.cl:108-110),
 * and atom radii are type_radii[t] (rsasa_cl_gpu_alg.cpp:140-151).
 * n_types <= 256, stride <= 4096. */
rsx_status rsx_sasa_create_typed(int n_atoms, const float *dot_map, int n_types, int stride,
                                 const float *type_radii, float probe, int device,
                                 rsx_sasa **out);
rsx_status rsx_sasa_destroy(rsx_sasa *h);

/* Accessible-dot counts per atom (the uint buffer of do_recalc_rsasa,
 * rsasa_cl_gpu_alg.cpp:177-197): a dot is occluded by atom b when
 * (P + r_b)^2 - |dot - p_b|^2 > 1e-4, each operation rounded to FP32 without
 * contraction; every atom, the dot's own included, is tested.  Unit-dot
 * handles; radii are per atom. */
rsx_status rsx_sasa_counts(rsx_sasa *h, const rsx_body *atoms, const float *radii,
                           unsigned *out_counts);

/* i_rsasa::calc_rsasa / recalc_rsasa: rsasa_i = count_i / n_dots
 * (rsasa_cl_gpu_alg.cpp:153-197).  Unit-dot handles. */
rsx_status rsx_sasa_calc(rsx_sasa *h, const rsx_body *atoms, const float *radii, float *out_rsasa);

/* The same for typed handles: atoms carry their type in .w; rsasa_i =
 * count_i / dots of the atom's type (rsasa_cl_gpu_alg.cpp:189-196,
 * rsasa_cpu_alg.cpp:181).  A type index >= n_types is RSX_INVALID_ARG. */
rsx_status rsx_sasa_counts_typed(rsx_sasa *h, const rsx_body *atoms, unsigned *out_counts);
rsx_status rsx_sasa_calc_typed(rsx_sasa *h, const rsx_body *atoms, float *out_rsasa);

/* Occlusion tests to the first occluder (in the order the kernel visits the
 * candidates) and GPU milliseconds (cell list + occlusion pass) of the last
 * call. */
rsx_status rsx_sasa_stats(rsx_sasa *h, unsigned long long *tests, float *ms_kernel);

/* Batched ensembles (no reference counterpart: the reference evaluates an
 * ensemble one model at a time, calc_saxs/calc_saxs.hpp:611-624).  M members
 * with their own body counts share q and the factor table; each pass runs as
 * one CUDA graph holding persistent pair kernels. --------------------------- */

typedef struct rsx_batch rsx_batch;

/* member_sizes[m] bodies per member; bodies of all members are passed
 * concatenated in member order.  opts as for rsx_debye_create (autotune = 1
 * picks the q-slab by timing the first pass). */
rsx_status rsx_batch_create(const float *q, int n_q, const float *t_factors, int n_factors,
                            const int *member_sizes, int n_members,
                            const rsx_debye_options *opts, rsx_batch **out);
rsx_status rsx_batch_destroy(rsx_batch *h);
/* I(q) of every member: out_iq is n_members x n_q. */
rsx_status rsx_batch_forward(rsx_batch *h, const rsx_body *bodies, float *out_iq);
/* Per-member targets and sigmas (n_members x n_q each) of the chi^2 loss. */
rsx_status rsx_batch_set_targets(rsx_batch *h, const float *targets, const float *sigma);
/* Replaces the factor table (n_q x n_factors, the handle's n_factors), as
 * rsx_debye_set_factors does for one structure. */
rsx_status rsx_batch_set_factors(rsx_batch *h, const float *t_factors, int n_factors);
/* Implicit water for every member (f~_i = f_t(i) + weight * rsasa_i * f_water),
 * as rsx_debye_set_water does for one structure: rsasa holds one value per
 * body in the concatenated caller order of rsx_batch_forward (NULL keeps the
 * values already set); weight 0 turns the term off.  Forward only:
 * rsx_batch_forward_chi2_backward returns RSX_NOT_SUPPORTED while the weight
 * is non-zero. */
rsx_status rsx_batch_set_water(rsx_batch *h, float weight, int water_index, const float *rsasa);
/* Forward, chi^2_m = sum_q ((I_m - t_m)/sigma_m)^2 and dchi^2_m/dx for every
 * body of every member, in one pass (out_iq, chi2, grad_xyz may be NULL). */
rsx_status rsx_batch_forward_chi2_backward(rsx_batch *h, const rsx_body *bodies, float *out_iq,
                                           double *chi2, float *grad_xyz);
/* Milliseconds of the last pass (graph launch to completion, CUDA events). */
rsx_status rsx_batch_timing(rsx_batch *h, float *ms_last_pass);
rsx_status rsx_batch_config(rsx_batch *h, int *q_slab, int *n_items, int *persistent_ctas,
                            int *uniform_q);

#ifdef __cplusplus
}
#endif
#endif /* RSX_H */
