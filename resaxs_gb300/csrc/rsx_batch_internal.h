// Batched ensembles: argument blocks and launchers of batch_kernels.cu.
#pragma once
#include "rsx_internal.h"

namespace rsx {

// I(q) of every member from the per-item cross sums.
struct BatchAssembleArgs {
    const double *partial;   // [n_q][n_items]
    const float *ff;         // [n_q][n_types]
    const float *q;          // [n_q]
    const int *type_count;   // [n_members][n_types]
    const int2 *item_range;  // [n_members] items [x, y) of each member
    int n_q, n_types, n_items, n_members;
    double *iq64;            // [n_members][n_q]
    float *iq32;             // [n_members][n_q]
    // implicit water (f~ = f_t + w rsasa f_w): per member sums of rsasa by
    // type, of rsasa^2 and of rsasa; has_water 0 leaves them unread
    const double *rsasa_sum; // [n_members][n_types]
    const double *rsasa_sq;  // [n_members]
    const double *rsasa_tot; // [n_members]
    float water_weight;
    int water_index, has_water;
};

// chi^2 of every member against its target and dL/dI = 2 (I - t) / sigma^2.
struct BatchLossArgs {
    const double *iq64;      // [n_members][n_q]
    const float *target;     // [n_members][n_q]
    const float *sigma;      // [n_members][n_q]
    int n_q, n_members;
    float *lambda;           // [n_members][n_q]
    double *chi2;            // [n_members]
};

// Persistent forward over work units (item, slab) handed out by an atomic
// counter, largest items first (work_order).  k_base: first q of slab 0.
// water: the implicit water term (a.rsasa set), q_slab 8 or 16.
cudaError_t launch_batch_forward(const DebyeArgs &a, const int *work_order, int n_work_items,
                                 int q_slab, int n_slabs, int k_base, bool uniform,
                                 int *counter, int grid, cudaStream_t st, bool water = false);
// Wide uniform slabs (q_slab 64 / 128 / 192; with water at most 128):
// persistent main and tail launches over counters[0] and counters[1].
cudaError_t launch_batch_forward_wide(const DebyeArgs &a, const int *work_order,
                                      int n_work_items, int q_slab, int *counters, int sms,
                                      cudaStream_t st, bool water = false);
// Chained forward (uniform grid, no water, q_slab 192): persistent launches
// over the full chains (counters[0]) and the rest chain (counters[1]).
cudaError_t launch_batch_forward_chain(const DebyeArgs &a, const int *work_order,
                                       int n_work_items, int *counters, int sms, cudaStream_t st);
cudaError_t launch_batch_adjoint(const DebyeArgs &a, const int *work_order, int n_work_items,
                                 int q_slab, bool uniform, int *counter, int grid,
                                 cudaStream_t st);
// The pair pass of the adjoint through tabulated pair functions (the tables
// are built by launch_adjoint_tables), persistent over counter.
cudaError_t launch_batch_adjoint_table(const DebyeArgs &a, const int *work_order,
                                       int n_work_items, int *counter, int grid, cudaStream_t st);
cudaError_t launch_batch_assemble(const BatchAssembleArgs &a, cudaStream_t st);
cudaError_t launch_batch_loss(const BatchLossArgs &a, cudaStream_t st);
// CTAs of the persistent kernels that fit on the device at once (water: the
// 8- or 16-q water kernels)
int batch_forward_grid(int q_slab, bool uniform, int sms, bool water = false);
int batch_adjoint_grid(int q_slab, bool uniform, int n_q, int sms);
int batch_adjoint_table_grid(int sms);

} // namespace rsx
