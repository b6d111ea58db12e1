/*
 * CPU oracle for the resaxs hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Nothing in the product library links, loads or calls this code.  It is used
 * by tests/, by __graft_entry__.smoke() as the checker, and by bench.py's CPU
 * baseline leg.  Every function restates an algorithm of the reference
 * (ldantonov/resaxs) and cites the file:line it follows.
 *
 * Body layout (same as the reference's cl_float4 bodies, utils.hpp:61-88):
 *   bodies[4*i + 0..2] = x, y, z (float), bodies[4*i + 3] = uint32 type index
 *   stored bit-for-bit in the float slot.
 * Form-factor table: row-major [n_q][n_factors] (host_debye.cpp:64-72).
 */
#ifndef RSX_ORACLE_H
#define RSX_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* FP64 Debye curve: restates host_debye<double,float,cl_float4>::calc_curve
 * (resaxslib/src/host_debye.cpp:54-109) without the N*N distance matrix.
 * I(q) = sum_i f_i^2 + 2 sum_{i<j} f_i f_j sinc(q r_ij), sinc = 1 when q*r == 0
 * (gpu_saxs_pt_wf.cl:55 maps the 0/0 case to 1; host_debye.cpp:93 for q == 0).
 * Uses the oracle's own FP64 sine (reduction modulo 2*pi + Taylor series;
 * the curve agrees with the libm form to ~1e-14 relative) in vectorisable loops.
 * Effective factor with the implicit water layer (gpu_saxs_pt_wf.cl:130-138):
 *   f_i(q) = F[q][t_i] + rsasa_i * (F[q][water_index] * water_weight).
 * rsasa may be NULL (no water).  n_threads <= 0 uses every online core. */
void orc_debye_f64(const double *q, int n_q, const float *bodies, int n_bodies,
                   const float *ff, int n_factors, const float *rsasa,
                   double water_weight, int water_index, double *out_iq,
                   int n_threads);

/* The same with libm sin per term (slower; cross-checks orc_debye_f64). */
void orc_debye_f64_libm(const double *q, int n_q, const float *bodies, int n_bodies,
                        const float *ff, int n_factors, const float *rsasa,
                        double water_weight, int water_index, double *out_iq,
                        int n_threads);

/* The oracle's own FP64 sine (tests compare it with libm). */
double orc_sin_probe(double x);

/* Same sum for a uniform q grid q_k = q0 + k*dq (k < n_q), evaluated with an
 * FP64 rotation recurrence seeded by libm sin/cos per pair; used where the
 * direct form is too slow (N >= 50k).  Accuracy ~1e-13 relative. */
void orc_debye_f64_uniform(double q0, double dq, int n_q, const float *bodies,
                           int n_bodies, const float *ff_rows, int n_factors,
                           double *out_iq, int n_threads);

/* FP64 gradient of L = sum_q w_q * I(q) with respect to every body position:
 *   dL/dx_i = sum_{j != i} 2 f_i f_j sum_q w_q (cos(q r) - sinc(q r)) / r^2 * (x_i - x_j)
 * (derivative of the sum in host_debye.cpp:74-108; the factors are held
 * constant).  grad is [n_bodies][3]. */
void orc_debye_grad_f64(const double *q, int n_q, const double *w_q,
                        const float *bodies, int n_bodies, const float *ff,
                        int n_factors, const float *rsasa, double water_weight,
                        int water_index, double *grad, int n_threads);

/* The same gradient for the bodies rows[0..n_rows) only (no water):
 * grad is [n_rows][3], row r for body rows[r]. */
void orc_debye_grad_rows_f64(const double *q, int n_q, const double *w_q,
                             const float *bodies, int n_bodies, const float *ff,
                             int n_factors, const int *rows, int n_rows, double *grad,
                             int n_threads);

/* FP64 central differences of L = sum_q w_q I(q): out[c] = (L with body
 * atom[c]'s coordinate axis[c] set to plus[c] - L with it set to minus[c]) /
 * (plus[c] - minus[c]), from the pairs of that body only (the rest of the
 * sum of host_debye.cpp:74-108 cancels), libm sin per term (no water). */
void orc_debye_fd_f64(const double *q, int n_q, const double *w_q, const float *bodies,
                      int n_bodies, const float *ff, int n_factors, const int *atom,
                      const int *axis, const float *plus, const float *minus, int n_coords,
                      double *out, int n_threads);

/* Reference-faithful port of host_debye<double,float,cl_float4>::calc_curve
 * (host_debye.cpp:54-109): same N*N distance matrix, same loop order, same
 * mixed float/double arithmetic.  Single threaded, exactly as the reference.
 * Used to time the reference CPU path where its compiled original is absent. */
void orc_refport_host_debye(const float *v_q, int n_q, const float *v_bodies,
                            int n_bodies, const float *t_factors, int n_factors,
                            float *out_v_iq);

/* The same port with its q loop split across threads sharing one distance
 * matrix (the reference has no threaded CPU path; this is its loop body run
 * on several cores).  Returns the seconds spent building the matrix. */
double orc_refport_host_debye_mt(const float *v_q, int n_q, const float *v_bodies,
                                 int n_bodies, const float *t_factors,
                                 int n_factors, float *out_v_iq, int n_threads);

/* The loop of orc_refport_host_debye_mt restricted to the rows `rows` of the
 * lower triangle (host_debye.cpp:74-104 for y in rows, x < y): out_partial[k]
 * = sum over those rows of F_q(y) * sum_{x<y} F_q(x) sinc(q r_xy), in the
 * reference's order and mixed float/double arithmetic, with the distance
 * rows built as host_debye.cpp:58-61 builds its matrix.  The q loop is split
 * over n_threads.  This times the reference's CPU path on a bounded sample of
 * a structure whose N x N matrix does not fit in memory (host_debye indexes
 * that matrix with int, so it cannot run past N = 46,340 at all).  Returns 0,
 * -1 for a row index outside [0, n_bodies), -2 when allocation fails. */
int orc_refport_host_debye_rows(const float *v_q, int n_q, const float *v_bodies,
                                int n_bodies, const float *t_factors, int n_factors,
                                const int *rows, int n_rows, double *out_partial,
                                int n_threads);

/* Strict-FP32 dot-sphere SASA counts: restates the occlusion test of
 * calc_rsasa (resaxslib/src/rsasa_dot_spheres.cl:94-163):
 *   ext_i = r_i + P;  dot = unit_k * ext_i;  sdot = dot + p_i     (per component)
 *   w_b = (P + r_b) * (P + r_b);  d = sdot - p_b;
 *   dist2 = (dx*dx + dy*dy) + dz*dz;  occluded iff (w_b - dist2) > 1e-4f
 * every operation rounded to FP32, no contraction.  counts[i] = accessible
 * dots of atom i.  Brute force over all atoms when use_cells == 0, else an
 * exact cell-list prune (a dot can only be occluded by an atom within
 * r_i + r_b + 2P of atom i). */
void orc_sasa_counts(const float *atoms, const float *radii, int n_atoms,
                     const float *unit_dots, int n_dots, float probe,
                     unsigned *counts, int use_cells, int n_threads);

/* The same occlusion test with pre-scaled dots per atom type, the layout of
 * the reference's OpenCL dot map (rsasa_cl_gpu_alg.cpp:59-89): dot k of an
 * atom of type t is dot_map[4*(t*stride + k) + 0..2] (x, y, z; w unused), a
 * dot whose x is not finite is padding and never counts; atom radii come
 * from type_radii[t].  dot = d + p_i (per component, FP32); occluded iff
 * (P + r_b)^2 - |dot - p_b|^2 > 1e-4f as above.  Exact (cell list sized by
 * the largest dot distance).  Returns 0, or -1 for a type index >= n_types
 * or a non-finite position. */
int orc_sasa_counts_typed(const float *atoms, int n_atoms, const float *type_radii,
                          int n_types, const float *dot_map, int stride, float probe,
                          unsigned *counts, int n_threads);

/* Port of rsasa_cpu_alg<float,float>::calc_rsasa (rsasa_cpu_alg.cpp:112-185)
 * with its 6 A voxel grid (bb_grid.hpp:130-266), in FP32 without
 * contraction, bit-identical to the compiled reference on x86; its neighbour
 * prune assumes radii <= 1.5 A (max_radius) as the reference's does.  Typed
 * form: radii and pre-scaled dot sets per type as the reference builds them
 * (type_radii[t]; dots_xyzw[4*k], k in [dot_start[t], dot_start[t+1]) for
 * type t); out_rsasa[i] = accessible / dots of the type.  Unit form: per-atom
 * radii, dot k of atom i at unit_k * (r_i + P), out_counts[i] = accessible
 * dots.  Atoms are split over n_threads (the reference runs one thread).
 * Return 0, -1 for a type index >= n_types, -2 when allocation fails. */
int orc_refport_rsasa_typed(const float *atoms, int n_atoms, const float *type_radii,
                            int n_types, const float *dots_xyzw, const int *dot_start,
                            float probe, float *out_rsasa, int n_threads);
int orc_refport_rsasa_unit(const float *atoms, int n_atoms, const float *radii,
                           const float *unit_dots, int n_dots, float probe,
                           unsigned *out_counts, int n_threads);

/* Fibonacci unit dots as generated by create_fibonacci_dots
 * (resaxslib/src/rsasa_algorithm.cpp:96-116) with n = n_dots / 2 (n_dots
 * even) and ext_radius = 1: out is [n_dots][3] FP32, bit-for-bit the unit
 * factors the reference multiplies by ext_radius. */
void orc_fibonacci_unit_dots(int n_dots, float *out_xyz);

#ifdef __cplusplus
}
#endif
#endif
