// Arguments of the dot-sphere SASA kernels (sasa_kernels.cu).
#pragma once
#include <cuda_runtime.h>

namespace rsx {

// Upper bounds of the kernels' tables.
constexpr int kSasaMaxGroups = 128;   // 32-dot groups per atom: <= 4096 dots
constexpr int kSasaMaxTypes = 256;    // dot tables of the typed (per-type) form
constexpr int kSasaMaxAtoms = 1 << 28; // the cell arrays hold 4 n + 4097 ints

// Geometry of one call, formed on the GPU from the atoms (sasa_geom_kernel,
// sasa_plan_kernel; zero on entry) and read by the cell-list and occlusion
// kernels, which do nothing when `bad` is set.
struct SasaGeom {
    unsigned lo_key[3];  // complemented ordered keys of the box minima
    unsigned hi_key[3];  // ordered keys of the box maxima
    unsigned amax_key;   // bits of the largest |coordinate|
    unsigned rmax_key;   // bits of the largest radius (unit form)
    unsigned present[kSasaMaxTypes / 32]; // types present (typed form)
    unsigned bad;        // a non-finite position, a bad radius or type
    // the cell grid (sasa_plan_kernel)
    int dims[3];
    int n_cells;
    float lo[3];
    float margin;
    double inv_cell;
};

// Cell list built on the GPU from the atoms in caller order.
struct SasaCellArgs {
    const float4 *atoms_in;   // [n_atoms] caller order: x, y, z, w (type bits or unused)
    const float *radii_in;    // [n_atoms] per-atom radii (unit form) or nullptr (typed form)
    const float *type_radius; // [n_types] radius of each type (typed form)
    int *cell_count;          // [n_cells + 1]; zero on entry to the bin kernel
    int *cell_start;          // [n_cells + 1] exclusive prefix sum of cell_count
    int *cell_of;             // [n_atoms] cell of each caller-order atom
    int *rank_of;             // [n_atoms] slot inside its cell
    float4 *atoms;            // [n_atoms] cell order: x, y, z, radius
    int *orig_index;          // [n_atoms] caller index of each cell-ordered atom
    int *type_of;             // [n_atoms] type of each cell-ordered atom (typed form)
    int *cell_sorted;         // [n_atoms] cell of each cell-ordered atom
    SasaGeom *geom;
    const float *dot_reach;   // [n_types] largest |d| of each type's table (typed form)
    float unit_reach, probe;  // unit form: reach of a dot is (r + P) * unit_reach
    int n_atoms, n_types;
    int cells_cap;            // cell_count / cell_start hold cells_cap entries (>= 4 n + 4097)
};

// Occlusion pass over the cell-ordered atoms: one warp per atom.
struct SasaArgs {
    const float4 *atoms;      // [n_atoms] cell order: x, y, z, radius
    const int *orig_index;    // [n_atoms] caller index of each cell-ordered atom
    const int *type_of;       // [n_atoms] type (typed form) or nullptr
    const int *cell_id;       // [n_atoms] cell of each cell-ordered atom
    const int *cell_start;    // [n_cells + 1]
    // Dot tables in groups of 32 (spatially compact on the sphere); a dot
    // whose x is not finite is padding.  Unit form: one table of unit
    // directions, dot = unit * (r_i + P); typed form: one pre-scaled table
    // per type, dot = d.
    const float4 *dots;
    const int *group_base;    // [n_types] first group of each type's table
    const int *group_count;   // [n_types] groups of each type's table
    const float *dot_reach;   // [n_types] largest |d| of each type's table (typed form)
    float unit_reach;         // largest |u| of the unit table (unit form)
    int typed;
    unsigned *counts;         // [n_atoms] accessible dots, caller order
    unsigned long long *tests; // optional: occlusion tests to the first occluder
    const SasaGeom *geom;     // cell grid and rounding margin of the call
    int n_atoms;
    float probe;
};

// Geometry (checks, bounding box, cell grid) and the cell list; c.geom,
// c.cell_count are cleared here first.
cudaError_t launch_sasa_cells(const SasaCellArgs &c, cudaStream_t st);
cudaError_t launch_sasa(const SasaArgs &a, cudaStream_t st);

} // namespace rsx
