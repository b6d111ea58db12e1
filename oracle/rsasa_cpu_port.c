/*
 * Port of the reference's CPU dot-sphere SASA -- TEST INFRASTRUCTURE ONLY
 * (see rsx_oracle.h).  Restates rsasa_cpu_alg<float,float>::calc_rsasa
 * (resaxslib/src/rsasa_cpu_alg.cpp:112-185) with its voxel grid
 * (resaxslib/include/bb_grid.hpp:130-266) in C, operation for operation in
 * FP32 (compiled with -ffp-contract=off), so that it can time the reference's
 * CPU path on machines where the compiled reference is absent.  It is
 * bit-identical to the compiled reference on x86 (tests/test_oracle.py).
 *
 * What it keeps from the reference, including its approximations:
 *  - 6 A voxels over the atoms' bounding box; voxel counts ceil(side / 6)
 *    per axis, at least 1; an atom's voxel is floor((v - lo) * (1 / 6)) with
 *    the linear index z*nx*ny + y*nx + x unclamped (bb_grid.hpp:178-187);
 *  - neighbour voxels: the box around atom i grown by r_i + 2P + 1.5 A
 *    (max_radius, rsasa_cpu_alg.cpp:136-140), clamped to the grid, so an
 *    occluder of radius > 1.5 A can be missed;
 *  - two neighbour lists (overlapping spheres first), the occlusion test
 *    (P + r_b)^2 - |c - p_b|^2 > 0.0001 in FP32 (rsasa_cpu_alg.cpp:62-69);
 *  - rsasa = accessible dots / dots of the atom (float division).
 * Atoms are split over threads (the reference is single threaded; every
 * atom's result is independent of the others).
 */
#include "rsx_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

static int port_threads(int n)
{
    if (n > 0)
        return n;
    long c = sysconf(_SC_NPROCESSORS_ONLN);
    return c > 0 ? (int)c : 1;
}

typedef struct {
    const float *atoms;     /* [n][4] */
    int n;
    const float *radius;    /* per atom */
    /* dots: typed (pre-scaled per type, CSR) or unit (scaled per atom) */
    const float *tdots;     /* [*][4] */
    const int *tstart;      /* [n_types + 1] */
    const float *unit;      /* [n_unit][3] */
    int n_unit;
    float probe;
    /* grid */
    float lo[3], rside;
    int nv[3];
    long n_vox;
    int *vox_start, *vox_items;
    float *out_rsasa;
    unsigned *out_counts;
    int next;
    pthread_mutex_t mu;
} port_job;

static unsigned body_type_bits(const float *atoms, int i)
{
    unsigned t;
    memcpy(&t, &atoms[4 * i + 3], 4);
    return t;
}

/* get_virtual_index (bb_grid.hpp:175-180) */
static void virtual_index(const port_job *J, const float p[3], int v[3])
{
    for (int a = 0; a < 3; ++a) {
        const float d = (p[a] - J->lo[a]) * J->rside;
        v[a] = (int)floorf(d);
    }
}

/* get_nearest_bounded_index (bb_grid.hpp:165-173) */
static void bounded_index(const port_job *J, const float p[3], int v[3])
{
    virtual_index(J, p, v);
    for (int a = 0; a < 3; ++a) {
        if (v[a] < 0)
            v[a] = 0;
        if (v[a] > J->nv[a] - 1)
            v[a] = J->nv[a] - 1;
    }
}

static long linear_index(const port_job *J, const int v[3])
{
    return (long)v[2] * J->nv[0] * J->nv[1] + (long)v[1] * J->nv[0] + v[0];
}

static float dist2_f(const float *a, const float *b)
{
    const float xd = a[0] - b[0];
    const float yd = a[1] - b[1];
    const float zd = a[2] - b[2];
    const float xx = xd * xd;
    const float yy = yd * yd;
    const float zz = zd * zd;
    return (xx + yy) + zz;
}

/* is_intersecting (rsasa_cpu_alg.cpp:62-69): the float difference compared
 * with the double literal 0.0001, which for a float operand is the same as
 * comparing with 0.0001f */
static int intersecting(const float c[3], const float *b, float probe, float rb)
{
    const float s = probe + rb;
    const float sum_r2 = s * s;
    const float d2 = dist2_f(c, b);
    const float diff = sum_r2 - d2;
    return (double)diff > 0.0001;
}

static void *port_worker(void *arg)
{
    port_job *J = (port_job *)arg;
    int cap = 256;
    int *nb1 = (int *)malloc(sizeof(int) * cap), *nb2 = (int *)malloc(sizeof(int) * cap);
    for (;;) {
        pthread_mutex_lock(&J->mu);
        const int i = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (i >= J->n)
            break;
        const float *pi = &J->atoms[4 * i];
        const float atom_radius = J->radius[i];
        const float radius = atom_radius + 2 * J->probe + 1.5f;
        float lc[3], uc[3];
        for (int a = 0; a < 3; ++a) {
            lc[a] = pi[a] + (-radius);
            uc[a] = pi[a] + radius;
        }
        int li[3], ui[3];
        bounded_index(J, lc, li);
        bounded_index(J, uc, ui);
        int n1 = 0, n2 = 0;
        for (int z = li[2]; z <= ui[2]; ++z)
            for (int y = li[1]; y <= ui[1]; ++y)
                for (int x = li[0]; x <= ui[0]; ++x) {
                    const int v[3] = {x, y, z};
                    const long c = linear_index(J, v);
                    for (int s = J->vox_start[c]; s < J->vox_start[c + 1]; ++s) {
                        const int b = J->vox_items[s];
                        const float rs1 = atom_radius + J->radius[b];
                        const float rs2 = rs1 + 2 * J->probe;
                        const float d2 = dist2_f(pi, &J->atoms[4 * b]);
                        if (n1 >= cap || n2 >= cap) {
                            cap *= 2;
                            nb1 = (int *)realloc(nb1, sizeof(int) * cap);
                            nb2 = (int *)realloc(nb2, sizeof(int) * cap);
                        }
                        if (d2 < rs1 * rs1)
                            nb1[n1++] = b;
                        else if (d2 < rs2 * rs2)
                            nb2[n2++] = b;
                    }
                }
        int n_dots, dot_num = 0;
        const float *tdots = NULL;
        float ext = 0.f;
        if (J->tdots) {
            const unsigned t = body_type_bits(J->atoms, i);
            tdots = &J->tdots[4 * (size_t)J->tstart[t]];
            n_dots = J->tstart[t + 1] - J->tstart[t];
        } else {
            n_dots = J->n_unit;
            ext = atom_radius + J->probe;
        }
        for (int k = 0; k < n_dots; ++k) {
            float sdot[3], c[3];
            for (int a = 0; a < 3; ++a)
                sdot[a] = tdots ? tdots[4 * k + a] : J->unit[3 * k + a] * ext;
            for (int a = 0; a < 3; ++a)
                c[a] = sdot[a] + pi[a];
            int hit = 0;
            for (int s = 0; s < n1 && !hit; ++s)
                hit = intersecting(c, &J->atoms[4 * nb1[s]], J->probe, J->radius[nb1[s]]);
            for (int s = 0; s < n2 && !hit; ++s)
                hit = intersecting(c, &J->atoms[4 * nb2[s]], J->probe, J->radius[nb2[s]]);
            if (!hit)
                ++dot_num;
        }
        if (J->out_rsasa)
            J->out_rsasa[i] = (float)dot_num / (float)n_dots;
        if (J->out_counts)
            J->out_counts[i] = (unsigned)dot_num;
    }
    free(nb1);
    free(nb2);
    return NULL;
}

static int port_run(port_job *J, int n_threads)
{
    const int n = J->n;
    if (n <= 0)
        return 0;
    /* bounding_box_3d(atoms) (bb_grid.hpp:95-116) and the voxel counts
     * get_ns1 (:134-140) */
    float hi[3];
    for (int a = 0; a < 3; ++a) {
        J->lo[a] = 3.402823466e38f;
        hi[a] = -3.402823466e38f;
    }
    for (int i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            const float v = J->atoms[4 * i + a];
            J->lo[a] = v < J->lo[a] ? v : J->lo[a];
            hi[a] = v > hi[a] ? v : hi[a];
        }
    const float side = 6.0f;
    J->rside = 1 / side;
    J->n_vox = 1;
    for (int a = 0; a < 3; ++a) {
        const float box_side = hi[a] - J->lo[a];
        const float d = box_side / side;
        const float cd = ceilf(d);
        J->nv[a] = (int)cd > 1 ? (int)cd : 1;
        J->n_vox *= J->nv[a];
    }
    J->vox_start = (int *)calloc((size_t)J->n_vox + 1, sizeof(int));
    J->vox_items = (int *)malloc(sizeof(int) * (size_t)n);
    long *lin = (long *)malloc(sizeof(long) * (size_t)n);
    if (!J->vox_start || !J->vox_items || !lin) {
        free(J->vox_start);
        free(J->vox_items);
        free(lin);
        return -2;
    }
    for (int i = 0; i < n; ++i) {
        int v[3];
        virtual_index(J, &J->atoms[4 * i], v);
        long c = linear_index(J, v);
        /* an index past the grid is undefined behaviour in the reference;
         * it is kept inside here */
        if (c < 0)
            c = 0;
        if (c >= J->n_vox)
            c = J->n_vox - 1;
        lin[i] = c;
        J->vox_start[c + 1]++;
    }
    for (long c = 0; c < J->n_vox; ++c)
        J->vox_start[c + 1] += J->vox_start[c];
    int *fill = (int *)malloc(sizeof(int) * (size_t)J->n_vox);
    memcpy(fill, J->vox_start, sizeof(int) * (size_t)J->n_vox);
    for (int i = 0; i < n; ++i) /* insertion order, as grid[index].push_back(i) */
        J->vox_items[fill[lin[i]]++] = i;
    free(fill);
    free(lin);
    J->next = 0;
    pthread_mutex_init(&J->mu, NULL);
    const int nt = port_threads(n_threads);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nt);
    for (int t = 0; t < nt; ++t)
        pthread_create(&th[t], NULL, port_worker, J);
    for (int t = 0; t < nt; ++t)
        pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&J->mu);
    free(J->vox_start);
    free(J->vox_items);
    return 0;
}

int orc_refport_rsasa_typed(const float *atoms, int n_atoms, const float *type_radii,
                            int n_types, const float *dots_xyzw, const int *dot_start,
                            float probe, float *out_rsasa, int n_threads)
{
    float *radius = (float *)malloc(sizeof(float) * (size_t)(n_atoms > 0 ? n_atoms : 1));
    for (int i = 0; i < n_atoms; ++i) {
        const unsigned t = body_type_bits(atoms, i);
        if ((int)t >= n_types) {
            free(radius);
            return -1;
        }
        radius[i] = type_radii[t]; /* get_radii (rsasa_cpu_alg.cpp:99-110) */
    }
    port_job J;
    memset(&J, 0, sizeof J);
    J.atoms = atoms;
    J.n = n_atoms;
    J.radius = radius;
    J.tdots = dots_xyzw;
    J.tstart = dot_start;
    J.probe = probe;
    J.out_rsasa = out_rsasa;
    const int rc = port_run(&J, n_threads);
    free(radius);
    return rc;
}

int orc_refport_rsasa_unit(const float *atoms, int n_atoms, const float *radii,
                           const float *unit_dots, int n_dots, float probe,
                           unsigned *out_counts, int n_threads)
{
    port_job J;
    memset(&J, 0, sizeof J);
    J.atoms = atoms;
    J.n = n_atoms;
    J.radius = radii;
    J.unit = unit_dots;
    J.n_unit = n_dots;
    J.probe = probe;
    J.out_counts = out_counts;
    return port_run(&J, n_threads);
}
