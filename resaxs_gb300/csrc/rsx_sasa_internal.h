// Arguments of the dot-sphere SASA kernel (sasa_kernels.cu).
#pragma once
#include <cuda_runtime.h>

namespace rsx {

struct SasaArgs {
    const float4 *atoms;      // [n_atoms] in cell order: x, y, z, radius
    const int *orig_index;    // [n_atoms] caller index of each cell-ordered atom
    const int *cell_of;       // [n_atoms][3] cell coordinates (cell order)
    const int *cell_start;    // [n_cells + 1]
    const float *unit;        // [n_dots][3] unit-sphere dots
    unsigned *counts;         // [n_atoms] accessible dots, caller order
    unsigned long long *tests; // optional: occlusion tests performed
    int n_atoms, n_dots;
    int dims[3];
    float probe, max_radius;
};

cudaError_t launch_sasa(const SasaArgs &a, cudaStream_t st);

} // namespace rsx
