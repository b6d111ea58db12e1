/*
 * CPU oracle for the dot-sphere SASA counts -- TEST INFRASTRUCTURE ONLY
 * (see rsx_oracle.h).  Compiled with -ffp-contract=off so that every
 * multiply and add below rounds to FP32 on its own, as the occlusion test of
 * resaxslib/src/rsasa_dot_spheres.cl:94-163 is specified here.
 */
#include "rsx_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

static int pick_threads(int n)
{
    if (n > 0)
        return n;
    long c = sysconf(_SC_NPROCESSORS_ONLN);
    return c > 0 ? (int)c : 1;
}

/* Fibonacci sphere, rsasa_algorithm.cpp:96-116 with n = n_dots/2.  The
 * reference computes in FLT_T = float: theta = 2*pi_f*i/phi, sphi = i/n,
 * cphi = (float)(sqrt((n+i)*(n-i))/n) in double, x = cphi*sin(theta)*ext,
 * y = cphi*cos(theta)*ext, z = sphi*ext.  With ext = 1 the products below are
 * the unit factors; the caller multiplies by ext in FP32 (same rounding as
 * the reference's left-to-right product). */
void orc_fibonacci_unit_dots(int n_dots, float *out_xyz)
{
    const int n = n_dots / 2;
    const float phi = (1.0f + sqrtf(5.0f)) / 2.0f;
    const float pi_f = (float)3.14159265358979323846;
    int k = 0;
    for (int i = -(n - 1); i <= n; ++i) {
        const float theta = 2 * pi_f * (float)i / phi;
        const float sphi = (float)i / (float)n;
        const float cphi = (float)(sqrt((double)((n + i) * (n - i))) / n);
        out_xyz[3 * k + 0] = cphi * sinf(theta);
        out_xyz[3 * k + 1] = cphi * cosf(theta);
        out_xyz[3 * k + 2] = sphi;
        ++k;
    }
}

typedef struct {
    const float *atoms, *radii, *unit;
    int n, nd;
    float probe;
    unsigned *counts;
    int use_cells;
    /* cell list */
    float lo[3], cell;
    int dims[3];
    int *cell_start, *cell_items;
    int next;
    pthread_mutex_t mu;
} sasa_job;

static int occluded(const float sd[3], const float *b, float rb, float probe)
{
    const float e = probe + rb;
    const float w = e * e;
    const float dx = sd[0] - b[0];
    const float dy = sd[1] - b[1];
    const float dz = sd[2] - b[2];
    const float xx = dx * dx;
    const float yy = dy * dy;
    const float zz = dz * dz;
    const float dist2 = (xx + yy) + zz;
    const float diff = w - dist2;
    return diff > 0.0001f;
}

static void atom_dot(const sasa_job *J, int i, int k, float sd[3])
{
    const float *p = &J->atoms[4 * i];
    const float ext = J->radii[i] + J->probe;
    for (int c = 0; c < 3; ++c) {
        const float d = J->unit[3 * k + c] * ext;
        sd[c] = d + p[c];
    }
}

static void cell_of(const sasa_job *J, const float *p, int c[3])
{
    for (int a = 0; a < 3; ++a) {
        int v = (int)floorf((p[a] - J->lo[a]) / J->cell);
        if (v < 0)
            v = 0;
        if (v >= J->dims[a])
            v = J->dims[a] - 1;
        c[a] = v;
    }
}

static void *sasa_worker(void *arg)
{
    sasa_job *J = (sasa_job *)arg;
    int *nb = (int *)malloc(sizeof(int) * (size_t)J->n);
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int i = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (i >= J->n)
            break;
        int n_nb = 0;
        if (J->use_cells) {
            int c[3];
            cell_of(J, &J->atoms[4 * i], c);
            for (int x = c[0] - 1; x <= c[0] + 1; ++x)
                for (int y = c[1] - 1; y <= c[1] + 1; ++y)
                    for (int z = c[2] - 1; z <= c[2] + 1; ++z) {
                        if (x < 0 || y < 0 || z < 0 || x >= J->dims[0] || y >= J->dims[1] ||
                            z >= J->dims[2])
                            continue;
                        int cid = (x * J->dims[1] + y) * J->dims[2] + z;
                        for (int s = J->cell_start[cid]; s < J->cell_start[cid + 1]; ++s)
                            nb[n_nb++] = J->cell_items[s];
                    }
        } else {
            for (int b = 0; b < J->n; ++b)
                nb[n_nb++] = b;
        }
        unsigned cnt = 0;
        for (int k = 0; k < J->nd; ++k) {
            float sd[3];
            atom_dot(J, i, k, sd);
            int occ = 0;
            for (int s = 0; s < n_nb && !occ; ++s) {
                int b = nb[s];
                occ = occluded(sd, &J->atoms[4 * b], J->radii[b], J->probe);
            }
            cnt += occ ? 0u : 1u;
        }
        J->counts[i] = cnt;
    }
    free(nb);
    return NULL;
}

void orc_sasa_counts(const float *atoms, const float *radii, int n_atoms,
                     const float *unit_dots, int n_dots, float probe,
                     unsigned *counts, int use_cells, int n_threads)
{
    sasa_job J;
    memset(&J, 0, sizeof J);
    J.atoms = atoms;
    J.radii = radii;
    J.unit = unit_dots;
    J.n = n_atoms;
    J.nd = n_dots;
    J.probe = probe;
    J.counts = counts;
    J.use_cells = use_cells;
    J.next = 0;
    pthread_mutex_init(&J.mu, NULL);
    if (use_cells && n_atoms > 0) {
        float hi[3], rmax = 0.0f;
        for (int a = 0; a < 3; ++a)
            J.lo[a] = hi[a] = atoms[a];
        for (int i = 0; i < n_atoms; ++i) {
            for (int a = 0; a < 3; ++a) {
                float v = atoms[4 * i + a];
                if (v < J.lo[a])
                    J.lo[a] = v;
                if (v > hi[a])
                    hi[a] = v;
            }
            if (radii[i] > rmax)
                rmax = radii[i];
        }
        /* any occluder of a dot of i lies within r_i + r_b + 2P <= 2 rmax + 2P
         * of atom i; a cell this wide plus its 26 neighbours covers it. */
        J.cell = 2.0f * rmax + 2.0f * probe + 0.01f;
        long total = 1;
        for (int a = 0; a < 3; ++a) {
            J.dims[a] = (int)floorf((hi[a] - J.lo[a]) / J.cell) + 1;
            total *= J.dims[a];
        }
        J.cell_start = (int *)calloc((size_t)total + 1, sizeof(int));
        J.cell_items = (int *)malloc(sizeof(int) * (size_t)n_atoms);
        int *cid = (int *)malloc(sizeof(int) * (size_t)n_atoms);
        for (int i = 0; i < n_atoms; ++i) {
            int c[3];
            cell_of(&J, &atoms[4 * i], c);
            cid[i] = (c[0] * J.dims[1] + c[1]) * J.dims[2] + c[2];
            J.cell_start[cid[i] + 1]++;
        }
        for (long c = 0; c < total; ++c)
            J.cell_start[c + 1] += J.cell_start[c];
        int *fill = (int *)malloc(sizeof(int) * (size_t)total);
        memcpy(fill, J.cell_start, sizeof(int) * (size_t)total);
        for (int i = 0; i < n_atoms; ++i)
            J.cell_items[fill[cid[i]]++] = i;
        free(fill);
        free(cid);
    }
    int nt = pick_threads(n_threads);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nt);
    for (int t = 0; t < nt; ++t)
        pthread_create(&th[t], NULL, sasa_worker, &J);
    for (int t = 0; t < nt; ++t)
        pthread_join(th[t], NULL);
    free(th);
    free(J.cell_start);
    free(J.cell_items);
    pthread_mutex_destroy(&J.mu);
}

/* ---- typed dot maps: pre-scaled dots per atom type ---------------------- */

typedef struct {
    const float *atoms, *type_radii, *dot_map;
    int n, n_types, stride;
    float probe;
    const float *reach;    /* per atom: max |dot| of its type + P + margin */
    unsigned *counts;
    float lo[3], cell;
    int dims[3];
    int *cell_start, *cell_items;
    float rmax;
    int next;
    pthread_mutex_t mu;
} typed_job;

static unsigned atom_type(const float *atoms, int i)
{
    unsigned t;
    memcpy(&t, &atoms[4 * i + 3], 4);
    return t;
}

static void typed_cell_of(const typed_job *J, const float *p, int c[3])
{
    for (int a = 0; a < 3; ++a) {
        int v = (int)floorf((p[a] - J->lo[a]) / J->cell);
        if (v < 0)
            v = 0;
        if (v >= J->dims[a])
            v = J->dims[a] - 1;
        c[a] = v;
    }
}

static void *typed_worker(void *arg)
{
    typed_job *J = (typed_job *)arg;
    int *nb = (int *)malloc(sizeof(int) * (size_t)(J->n > 0 ? J->n : 1));
    for (;;) {
        pthread_mutex_lock(&J->mu);
        const int i = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (i >= J->n)
            break;
        const float *pi = &J->atoms[4 * i];
        int n_nb = 0, c[3];
        typed_cell_of(J, pi, c);
        for (int x = c[0] - 1; x <= c[0] + 1; ++x)
            for (int y = c[1] - 1; y <= c[1] + 1; ++y)
                for (int z = c[2] - 1; z <= c[2] + 1; ++z) {
                    if (x < 0 || y < 0 || z < 0 || x >= J->dims[0] || y >= J->dims[1] ||
                        z >= J->dims[2])
                        continue;
                    const int cid = (x * J->dims[1] + y) * J->dims[2] + z;
                    for (int s = J->cell_start[cid]; s < J->cell_start[cid + 1]; ++s)
                        nb[n_nb++] = J->cell_items[s];
                }
        const unsigned t = atom_type(J->atoms, i);
        const float *dots = &J->dot_map[4 * (size_t)t * J->stride];
        unsigned cnt = 0;
        for (int k = 0; k < J->stride; ++k) {
            if (!isfinite(dots[4 * k]))
                continue; /* padding: not a dot */
            float sd[3];
            for (int a = 0; a < 3; ++a)
                sd[a] = dots[4 * k + a] + pi[a];
            int occ = 0;
            for (int s = 0; s < n_nb && !occ; ++s) {
                const int b = nb[s];
                occ = occluded(sd, &J->atoms[4 * b],
                               J->type_radii[atom_type(J->atoms, b)], J->probe);
            }
            cnt += occ ? 0u : 1u;
        }
        J->counts[i] = cnt;
    }
    free(nb);
    return NULL;
}

int orc_sasa_counts_typed(const float *atoms, int n_atoms, const float *type_radii,
                          int n_types, const float *dot_map, int stride, float probe,
                          unsigned *counts, int n_threads)
{
    if (n_atoms <= 0)
        return 0;
    typed_job J;
    memset(&J, 0, sizeof J);
    J.atoms = atoms;
    J.type_radii = type_radii;
    J.dot_map = dot_map;
    J.n = n_atoms;
    J.n_types = n_types;
    J.stride = stride;
    J.probe = probe;
    J.counts = counts;
    /* largest dot distance over the types, largest radius over the atoms */
    float ext = 0.0f, hi[3], rmax = 0.0f;
    for (int t = 0; t < n_types; ++t)
        for (int k = 0; k < stride; ++k) {
            const float *d = &dot_map[4 * ((size_t)t * stride + k)];
            if (!isfinite(d[0]))
                continue;
            const double r = sqrt((double)d[0] * d[0] + (double)d[1] * d[1] + (double)d[2] * d[2]);
            if (r > ext)
                ext = (float)r;
        }
    float amax = 0.0f;
    for (int a = 0; a < 3; ++a)
        J.lo[a] = hi[a] = atoms[a];
    for (int i = 0; i < n_atoms; ++i) {
        const unsigned t = atom_type(atoms, i);
        if ((int)t >= n_types)
            return -1;
        for (int a = 0; a < 3; ++a) {
            const float v = atoms[4 * i + a];
            if (!isfinite(v))
                return -1;
            if (v < J.lo[a])
                J.lo[a] = v;
            if (v > hi[a])
                hi[a] = v;
            if (fabsf(v) > amax)
                amax = fabsf(v);
        }
        if (type_radii[t] > rmax)
            rmax = type_radii[t];
    }
    /* an occluder b of a dot of atom i lies within |dot| + P + r_b of atom i
     * (plus the rounding of the dot's position) */
    J.cell = ext + probe + rmax + 0.01f + 8e-6f * amax;
    long total = 1;
    for (int a = 0; a < 3; ++a) {
        J.dims[a] = (int)floorf((hi[a] - J.lo[a]) / J.cell) + 1;
        total *= J.dims[a];
    }
    J.cell_start = (int *)calloc((size_t)total + 1, sizeof(int));
    J.cell_items = (int *)malloc(sizeof(int) * (size_t)n_atoms);
    int *cid = (int *)malloc(sizeof(int) * (size_t)n_atoms);
    for (int i = 0; i < n_atoms; ++i) {
        int c[3];
        typed_cell_of(&J, &atoms[4 * i], c);
        cid[i] = (c[0] * J.dims[1] + c[1]) * J.dims[2] + c[2];
        J.cell_start[cid[i] + 1]++;
    }
    for (long c = 0; c < total; ++c)
        J.cell_start[c + 1] += J.cell_start[c];
    int *fill = (int *)malloc(sizeof(int) * (size_t)total);
    memcpy(fill, J.cell_start, sizeof(int) * (size_t)total);
    for (int i = 0; i < n_atoms; ++i)
        J.cell_items[fill[cid[i]]++] = i;
    free(fill);
    free(cid);
    pthread_mutex_init(&J.mu, NULL);
    const int nt = pick_threads(n_threads);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nt);
    for (int t = 0; t < nt; ++t)
        pthread_create(&th[t], NULL, typed_worker, &J);
    for (int t = 0; t < nt; ++t)
        pthread_join(th[t], NULL);
    free(th);
    free(J.cell_start);
    free(J.cell_items);
    pthread_mutex_destroy(&J.mu);
    return 0;
}
