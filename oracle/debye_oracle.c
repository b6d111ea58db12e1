/*
 * CPU oracle for the Debye sum -- TEST INFRASTRUCTURE ONLY (see rsx_oracle.h).
 * Restates resaxslib/src/host_debye.cpp:54-109 in FP64, plus its gradient.
 */
#include "rsx_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

static unsigned body_type(const float *bodies, int i)
{
    unsigned t;
    memcpy(&t, &bodies[4 * i + 3], sizeof t); /* utils.hpp:61-66 */
    return t;
}

static int pick_threads(int n)
{
    if (n > 0)
        return n;
    long c = sysconf(_SC_NPROCESSORS_ONLN);
    return c > 0 ? (int)c : 1;
}

/* effective factor, gpu_saxs_pt_wf.cl:130-138 (in FP64) */
static double eff_factor(const float *ff, int n_factors, int k, unsigned t,
                         const float *rsasa, double ww, int water_index, int i)
{
    double f = ff[(size_t)k * n_factors + t];
    if (rsasa)
        f += (double)rsasa[i] * ((double)ff[(size_t)k * n_factors + water_index] * ww);
    return f;
}

/* ---------------- direct FP64 Debye, parallel over rows ---------------- */

typedef struct {
    const double *q;
    int n_q;
    const float *bodies;
    int n;
    const double *f; /* [n_q][n] effective factors */
    int next_row;    /* shared work counter (guarded by mu) */
    pthread_mutex_t mu;
    double *acc; /* [n_threads][n_q] */
} debye_job;

typedef struct {
    debye_job *job;
    int tid;
} debye_arg;

static int grab_rows(pthread_mutex_t *mu, int *next, int limit, int chunk, int *begin)
{
    pthread_mutex_lock(mu);
    int b = *next;
    int e = b + chunk > limit ? limit : b + chunk;
    *next = e;
    pthread_mutex_unlock(mu);
    *begin = b;
    return e;
}

static void *debye_worker(void *p)
{
    debye_arg *a = (debye_arg *)p;
    debye_job *J = a->job;
    double *acc = J->acc + (size_t)a->tid * J->n_q;
    double *inner = (double *)calloc((size_t)J->n_q, sizeof(double));
    for (;;) {
        int b;
        int e = grab_rows(&J->mu, &J->next_row, J->n, 16, &b);
        if (b >= e)
            break;
        for (int y = b; y < e; ++y) {
            const float *py = &J->bodies[4 * y];
            for (int k = 0; k < J->n_q; ++k)
                inner[k] = 0.0;
            for (int x = 0; x < y; ++x) {
                const float *px = &J->bodies[4 * x];
                double dx = (double)px[0] - py[0];
                double dy = (double)px[1] - py[1];
                double dz = (double)px[2] - py[2];
                double r = sqrt(dx * dx + dy * dy + dz * dz);
                for (int k = 0; k < J->n_q; ++k) {
                    double qr = J->q[k] * r;
                    double s = (qr == 0.0) ? 1.0 : sin(qr) / qr;
                    inner[k] += J->f[(size_t)k * J->n + x] * s;
                }
            }
            for (int k = 0; k < J->n_q; ++k)
                acc[k] += inner[k] * J->f[(size_t)k * J->n + y];
        }
    }
    free(inner);
    return NULL;
}

void orc_debye_f64_libm(const double *q, int n_q, const float *bodies, int n_bodies,
                        const float *ff, int n_factors, const float *rsasa,
                        double water_weight, int water_index, double *out_iq,
                        int n_threads)
{
    int nt = pick_threads(n_threads);
    double *f = (double *)malloc(sizeof(double) * (size_t)n_q * n_bodies);
    for (int k = 0; k < n_q; ++k)
        for (int i = 0; i < n_bodies; ++i)
            f[(size_t)k * n_bodies + i] = eff_factor(ff, n_factors, k, body_type(bodies, i),
                                                     rsasa, water_weight, water_index, i);
    debye_job J;
    J.q = q;
    J.n_q = n_q;
    J.bodies = bodies;
    J.n = n_bodies;
    J.f = f;
    J.next_row = 0;
    pthread_mutex_init(&J.mu, NULL);
    J.acc = (double *)calloc((size_t)nt * n_q, sizeof(double));
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nt);
    debye_arg *args = (debye_arg *)malloc(sizeof(debye_arg) * nt);
    for (int t = 0; t < nt; ++t) {
        args[t].job = &J;
        args[t].tid = t;
        pthread_create(&th[t], NULL, debye_worker, &args[t]);
    }
    for (int t = 0; t < nt; ++t)
        pthread_join(th[t], NULL);
    for (int k = 0; k < n_q; ++k) {
        double cross = 0.0, self = 0.0;
        for (int t = 0; t < nt; ++t)
            cross += J.acc[(size_t)t * n_q + k];
        for (int i = 0; i < n_bodies; ++i) {
            double fi = f[(size_t)k * n_bodies + i];
            self += fi * fi; /* autologous terms, host_debye.cpp:85 */
        }
        out_iq[k] = 2.0 * cross + self; /* host_debye.cpp:106-107 */
    }
    pthread_mutex_destroy(&J.mu);
    free(J.acc);
    free(th);
    free(args);
    free(f);
}


/* ------------- direct FP64 Debye with the oracle's own sine -------------- */

/* FP64 sine for the oracle, written for it: Cody & Waite reduction by pi/2
 * (pi/2 = C1 + C2 + C3, C1 and C2 with 32 significant bits so n*C1, n*C2 are
 * exact for |n| < 2^21), then the Taylor series of sin / cos on |r| <= pi/4
 * (to r^17 / r^18: truncation below 1e-19).  Branch-free so that the loops
 * below vectorise. */
#define ORC_C1 0x1.921fb54400000p+0
#define ORC_C2 0x1.0b4611a600000p-34
#define ORC_C3 0x1.3198a2e037073p-69
#define ORC_2PI_INV 0.6366197723675814

static inline double orc_sin(double x)
{
    double n = __builtin_nearbyint(x * ORC_2PI_INV);
    double r = ((x - n * ORC_C1) - n * ORC_C2) - n * ORC_C3;
    double r2 = r * r;
    double ps = 1.0 / 355687428096000.0; /* 1/17! */
    ps = ps * r2 - 1.0 / 1307674368000.0;
    ps = ps * r2 + 1.0 / 6227020800.0;
    ps = ps * r2 - 1.0 / 39916800.0;
    ps = ps * r2 + 1.0 / 362880.0;
    ps = ps * r2 - 1.0 / 5040.0;
    ps = ps * r2 + 1.0 / 120.0;
    ps = ps * r2 - 1.0 / 6.0;
    double sv = r + r * r2 * ps;
    double pc = -1.0 / 6402373705728000.0; /* -1/18! */
    pc = pc * r2 + 1.0 / 20922789888000.0;
    pc = pc * r2 - 1.0 / 87178291200.0;
    pc = pc * r2 + 1.0 / 479001600.0;
    pc = pc * r2 - 1.0 / 3628800.0;
    pc = pc * r2 + 1.0 / 40320.0;
    pc = pc * r2 - 1.0 / 720.0;
    pc = pc * r2 + 1.0 / 24.0;
    pc = pc * r2 - 0.5;
    double cv = 1.0 + r2 * pc;
    long long qn = (long long)n;
    double v = (qn & 1) ? cv : sv;
    return (qn & 2) ? -v : v;
}

double orc_sin_probe(double x) { return orc_sin(x); }

/* The same sine in a form gcc vectorises on any target: reduction modulo
 * 2*pi (the pi/2 split times 4, exact) with the 1.5*2^52 rounding constant,
 * then the odd Taylor series of sin on |r| <= pi up to r^33 (truncation
 * pi^35/35! < 1e-22).  No quadrant logic, no floor, no integer conversion. */
static inline double orc_sin_v(double x)
{
    const double magic = 0x1.8p52;
    const double inv2pi = 0.15915494309189535;
    double n = (x * inv2pi + magic) - magic;
    double r = ((x - n * (4.0 * ORC_C1)) - n * (4.0 * ORC_C2)) - n * (4.0 * ORC_C3);
    double r2 = r * r;
    double p = 1.0 / 8.683317618811886e36;    /* 1/33! */
    p = p * r2 - 1.0 / 8.222838654177922e33;  /* 1/31! */
    p = p * r2 + 1.0 / 8.841761993739702e30;  /* 1/29! */
    p = p * r2 - 1.0 / 1.0888869450418352e28; /* 1/27! */
    p = p * r2 + 1.0 / 1.5511210043330986e25; /* 1/25! */
    p = p * r2 - 1.0 / 2.585201673888498e22;  /* 1/23! */
    p = p * r2 + 1.0 / 5.109094217170944e19;  /* 1/21! */
    p = p * r2 - 1.0 / 1.21645100408832e17;   /* 1/19! */
    p = p * r2 + 1.0 / 355687428096000.0;     /* 1/17! */
    p = p * r2 - 1.0 / 1307674368000.0;
    p = p * r2 + 1.0 / 6227020800.0;
    p = p * r2 - 1.0 / 39916800.0;
    p = p * r2 + 1.0 / 362880.0;
    p = p * r2 - 1.0 / 5040.0;
    p = p * r2 + 1.0 / 120.0;
    p = p * r2 - 1.0 / 6.0;
    return r + r * r2 * p;
}

typedef struct {
    const double *q;
    int n_q;
    const float *bodies;
    int n;
    const double *f; /* [n_q][n] */
    int next_row;
    pthread_mutex_t mu;
    double *acc; /* [n_threads][n_q] */
} fast_job;

typedef struct {
    fast_job *job;
    int tid;
} fast_arg;

static void *fast_worker(void *p)
{
    fast_arg *a = (fast_arg *)p;
    fast_job *J = a->job;
    const int n = J->n;
    double *acc = J->acc + (size_t)a->tid * J->n_q;
    double *r = (double *)malloc(sizeof(double) * (size_t)(n + 1));
    double *t = (double *)malloc(sizeof(double) * (size_t)(n + 1));
    for (;;) {
        int b;
        int e = grab_rows(&J->mu, &J->next_row, J->n, 8, &b);
        if (b >= e)
            break;
        for (int y = b; y < e; ++y) {
            const float *py = &J->bodies[4 * y];
            const double yx = py[0], yy = py[1], yz = py[2];
            for (int x = 0; x < y; ++x) {
                const float *px = &J->bodies[4 * x];
                double dx = (double)px[0] - yx, dy = (double)px[1] - yy, dz = (double)px[2] - yz;
                r[x] = sqrt(dx * dx + dy * dy + dz * dz);
            }
            for (int k = 0; k < J->n_q; ++k) {
                const double qk = J->q[k];
                const double *fk = J->f + (size_t)k * n;
                for (int x = 0; x < y; ++x) {
                    double qr = qk * r[x];
                    double z = (qr == 0.0) ? 1.0 : 0.0;
                    double sn = orc_sin_v(qr);
                    t[x] = fk[x] * ((sn + z) / (qr + z)); /* sinc, = 1 at qr = 0 */
                }
                double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
                int x = 0;
                for (; x + 3 < y; x += 4) {
                    s0 += t[x];
                    s1 += t[x + 1];
                    s2 += t[x + 2];
                    s3 += t[x + 3];
                }
                for (; x < y; ++x)
                    s0 += t[x];
                acc[k] += ((s0 + s1) + (s2 + s3)) * fk[y];
            }
        }
    }
    free(r);
    free(t);
    return NULL;
}

void orc_debye_f64(const double *q, int n_q, const float *bodies, int n_bodies,
                   const float *ff, int n_factors, const float *rsasa,
                   double water_weight, int water_index, double *out_iq,
                   int n_threads)
{
    int nt = pick_threads(n_threads);
    double *f = (double *)malloc(sizeof(double) * (size_t)n_q * (n_bodies > 0 ? n_bodies : 1));
    for (int k = 0; k < n_q; ++k)
        for (int i = 0; i < n_bodies; ++i)
            f[(size_t)k * n_bodies + i] = eff_factor(ff, n_factors, k, body_type(bodies, i),
                                                     rsasa, water_weight, water_index, i);
    fast_job J;
    J.q = q;
    J.n_q = n_q;
    J.bodies = bodies;
    J.n = n_bodies;
    J.f = f;
    J.next_row = 0;
    pthread_mutex_init(&J.mu, NULL);
    J.acc = (double *)calloc((size_t)nt * n_q, sizeof(double));
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nt);
    fast_arg *args = (fast_arg *)malloc(sizeof(fast_arg) * nt);
    for (int t = 0; t < nt; ++t) {
        args[t].job = &J;
        args[t].tid = t;
        pthread_create(&th[t], NULL, fast_worker, &args[t]);
    }
    for (int t = 0; t < nt; ++t)
        pthread_join(th[t], NULL);
    for (int k = 0; k < n_q; ++k) {
        double cross = 0.0, self = 0.0;
        for (int t = 0; t < nt; ++t)
            cross += J.acc[(size_t)t * n_q + k];
        for (int i = 0; i < n_bodies; ++i) {
            double fi = f[(size_t)k * n_bodies + i];
            self += fi * fi;
        }
        out_iq[k] = 2.0 * cross + self;
    }
    pthread_mutex_destroy(&J.mu);
    free(J.acc);
    free(th);
    free(args);
    free(f);
}

/* ------------- FP64 rotation form for a uniform q grid ------------------ */

/* sin and cos of x with the oracle's reduction and series, branch-free (the
 * quadrant selects compile to blends) so that loops over pairs vectorise. */
static inline void orc_sincos(double x, double *s, double *c)
{
    const double magic = 0x1.8p52;
    double n = (x * ORC_2PI_INV + magic) - magic;
    double r = ((x - n * ORC_C1) - n * ORC_C2) - n * ORC_C3;
    double r2 = r * r;
    double ps = 1.0 / 355687428096000.0;
    ps = ps * r2 - 1.0 / 1307674368000.0;
    ps = ps * r2 + 1.0 / 6227020800.0;
    ps = ps * r2 - 1.0 / 39916800.0;
    ps = ps * r2 + 1.0 / 362880.0;
    ps = ps * r2 - 1.0 / 5040.0;
    ps = ps * r2 + 1.0 / 120.0;
    ps = ps * r2 - 1.0 / 6.0;
    double sv = r + r * r2 * ps;
    double pc = -1.0 / 6402373705728000.0;
    pc = pc * r2 + 1.0 / 20922789888000.0;
    pc = pc * r2 - 1.0 / 87178291200.0;
    pc = pc * r2 + 1.0 / 479001600.0;
    pc = pc * r2 - 1.0 / 3628800.0;
    pc = pc * r2 + 1.0 / 40320.0;
    pc = pc * r2 - 1.0 / 720.0;
    pc = pc * r2 + 1.0 / 24.0;
    pc = pc * r2 - 0.5;
    double cv = 1.0 + r2 * pc;
    long long qn = (long long)n;
    double odd = (double)(qn & 1);
    double sgn_s = 1.0 - (double)(qn & 2);          /* quadrants 2,3: -sin */
    double sgn_c = 1.0 - (double)((qn + 1) & 2);    /* quadrants 1,2: -cos */
    *s = sgn_s * (odd * cv + (1.0 - odd) * sv);
    *c = sgn_c * (odd * sv + (1.0 - odd) * cv);
}

typedef struct {
    double q0, dq;
    int n_q;
    const float *bodies;
    int n;
    const float *ff;
    int n_factors;
    int next_row;
    pthread_mutex_t mu;
    double *acc; /* [n_threads][n_q] */
} uni_job;

typedef struct {
    uni_job *job;
    int tid;
} uni_arg;

static void *uni_worker(void *p)
{
    uni_arg *a = (uni_arg *)p;
    uni_job *J = a->job;
    const int nq = J->n_q, n = J->n;
    double *acc = J->acc + (size_t)a->tid * nq;
    double *s = (double *)malloc(sizeof(double) * (size_t)(n + 1));
    double *c = (double *)malloc(sizeof(double) * (size_t)(n + 1));
    double *sd = (double *)malloc(sizeof(double) * (size_t)(n + 1));
    double *cd = (double *)malloc(sizeof(double) * (size_t)(n + 1));
    double *w = (double *)malloc(sizeof(double) * (size_t)(n + 1));
    double *fx = (double *)malloc(sizeof(double) * (size_t)(n + 1));
    unsigned *tx = (unsigned *)malloc(sizeof(unsigned) * (size_t)(n + 1));
    for (int x = 0; x < n; ++x)
        tx[x] = body_type(J->bodies, x);
    for (;;) {
        int b;
        int e = grab_rows(&J->mu, &J->next_row, J->n, 8, &b);
        if (b >= e)
            break;
        for (int y = b; y < e; ++y) {
            const float *py = &J->bodies[4 * y];
            const double yx = py[0], yy = py[1], yz = py[2];
            for (int x = 0; x < y; ++x) {
                const float *px = &J->bodies[4 * x];
                double dx = (double)px[0] - yx, dy = (double)px[1] - yy, dz = (double)px[2] - yz;
                double r = sqrt(dx * dx + dy * dy + dz * dz);
                /* coincident bodies: sinc = 1 for every q (handled by the
                 * r -> tiny limit of sin(q r)/(q r)) */
                r = r > 1e-12 ? r : 1e-12;
                double s0, c0, s1, c1;
                orc_sincos(J->q0 * r, &s0, &c0);
                orc_sincos(J->dq * r, &s1, &c1);
                double ir = 1.0 / r;
                s[x] = s0 * ir;
                c[x] = c0 * ir;
                sd[x] = s1;
                cd[x] = c1;
            }
            const unsigned ty = body_type(J->bodies, y);
            for (int k = 0; k < nq; ++k) {
                const double qk = J->q0 + k * J->dq;
                const float *row = J->ff + (size_t)k * J->n_factors;
                for (int x = 0; x < y; ++x)
                    fx[x] = row[tx[x]];
                double s0 = 0, s1 = 0;
                int x = 0;
                for (; x + 1 < y; x += 2) {
                    s0 += fx[x] * s[x];
                    s1 += fx[x + 1] * s[x + 1];
                }
                for (; x < y; ++x)
                    s0 += fx[x] * s[x];
                double inner = s0 + s1;
                if (qk == 0.0) { /* sinc = 1 */
                    double t = 0;
                    for (int z = 0; z < y; ++z)
                        t += fx[z];
                    inner = t;
                } else {
                    inner /= qk;
                }
                acc[k] += inner * row[ty];
                for (int z = 0; z < y; ++z) {
                    double s2 = s[z] * cd[z] + c[z] * sd[z];
                    double c2 = c[z] * cd[z] - s[z] * sd[z];
                    s[z] = s2;
                    c[z] = c2;
                }
            }
            (void)w;
        }
    }
    free(s);
    free(c);
    free(sd);
    free(cd);
    free(w);
    free(fx);
    free(tx);
    return NULL;
}

void orc_debye_f64_uniform(double q0, double dq, int n_q, const float *bodies,
                           int n_bodies, const float *ff_rows, int n_factors,
                           double *out_iq, int n_threads)
{
    int nt = pick_threads(n_threads);
    uni_job J;
    J.q0 = q0;
    J.dq = dq;
    J.n_q = n_q;
    J.bodies = bodies;
    J.n = n_bodies;
    J.ff = ff_rows;
    J.n_factors = n_factors;
    J.next_row = 0;
    pthread_mutex_init(&J.mu, NULL);
    J.acc = (double *)calloc((size_t)nt * n_q, sizeof(double));
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nt);
    uni_arg *args = (uni_arg *)malloc(sizeof(uni_arg) * nt);
    for (int t = 0; t < nt; ++t) {
        args[t].job = &J;
        args[t].tid = t;
        pthread_create(&th[t], NULL, uni_worker, &args[t]);
    }
    for (int t = 0; t < nt; ++t)
        pthread_join(th[t], NULL);
    for (int k = 0; k < n_q; ++k) {
        double cross = 0.0, self = 0.0;
        for (int t = 0; t < nt; ++t)
            cross += J.acc[(size_t)t * n_q + k];
        for (int i = 0; i < n_bodies; ++i) {
            double fi = ff_rows[(size_t)k * n_factors + body_type(bodies, i)];
            self += fi * fi;
        }
        out_iq[k] = 2.0 * cross + self;
    }
    pthread_mutex_destroy(&J.mu);
    free(J.acc);
    free(th);
    free(args);
}

/* ------------------------- FP64 gradient -------------------------------- */

typedef struct {
    const double *q, *w;
    int n_q;
    const float *bodies;
    int n;
    const double *f; /* [n_q][n] */
    int next_row;
    pthread_mutex_t mu;
    double *grad;
    const int *rows;  /* NULL: every body; else grad row r belongs to body rows[r] */
    int n_rows;
} grad_job;

typedef struct {
    grad_job *job;
} grad_arg;

static void *grad_worker(void *p)
{
    grad_job *J = ((grad_arg *)p)->job;
    const int limit = J->rows ? J->n_rows : J->n;
    for (;;) {
        int b;
        int e = grab_rows(&J->mu, &J->next_row, limit, J->rows ? 1 : 8, &b);
        if (b >= e)
            break;
        for (int row = b; row < e; ++row) {
            const int i = J->rows ? J->rows[row] : row;
            const float *pi = &J->bodies[4 * i];
            double g[3] = {0.0, 0.0, 0.0};
            for (int j = 0; j < J->n; ++j) {
                if (j == i)
                    continue;
                const float *pj = &J->bodies[4 * j];
                double d[3] = {(double)pi[0] - pj[0], (double)pi[1] - pj[1],
                               (double)pi[2] - pj[2]};
                double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                double r = sqrt(r2);
                if (r == 0.0)
                    continue; /* derivative of sinc at 0 is 0 */
                double G = 0.0;
                for (int k = 0; k < J->n_q; ++k) {
                    double qk = J->q[k];
                    if (qk == 0.0)
                        continue;
                    double x = qk * r;
                    double dsinc = cos(x) - sin(x) / x; /* x * d sinc/dx */
                    G += J->w[k] * J->f[(size_t)k * J->n + i] * J->f[(size_t)k * J->n + j] * dsinc;
                }
                G *= 2.0 / r2;
                g[0] += G * d[0];
                g[1] += G * d[1];
                g[2] += G * d[2];
            }
            J->grad[3 * row + 0] = g[0];
            J->grad[3 * row + 1] = g[1];
            J->grad[3 * row + 2] = g[2];
        }
    }
    return NULL;
}

static void grad_run(const double *q, int n_q, const double *w_q, const float *bodies,
                     int n_bodies, const float *ff, int n_factors, const float *rsasa,
                     double water_weight, int water_index, const int *rows, int n_rows,
                     double *grad, int n_threads)
{
    int nt = pick_threads(n_threads);
    double *f = (double *)malloc(sizeof(double) * (size_t)n_q * n_bodies);
    for (int k = 0; k < n_q; ++k)
        for (int i = 0; i < n_bodies; ++i)
            f[(size_t)k * n_bodies + i] = eff_factor(ff, n_factors, k, body_type(bodies, i),
                                                     rsasa, water_weight, water_index, i);
    grad_job J;
    J.q = q;
    J.w = w_q;
    J.n_q = n_q;
    J.bodies = bodies;
    J.n = n_bodies;
    J.f = f;
    J.next_row = 0;
    J.grad = grad;
    J.rows = rows;
    J.n_rows = n_rows;
    pthread_mutex_init(&J.mu, NULL);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nt);
    grad_arg *args = (grad_arg *)malloc(sizeof(grad_arg) * nt);
    for (int t = 0; t < nt; ++t) {
        args[t].job = &J;
        pthread_create(&th[t], NULL, grad_worker, &args[t]);
    }
    for (int t = 0; t < nt; ++t)
        pthread_join(th[t], NULL);
    pthread_mutex_destroy(&J.mu);
    free(th);
    free(args);
    free(f);
}

void orc_debye_grad_f64(const double *q, int n_q, const double *w_q,
                        const float *bodies, int n_bodies, const float *ff,
                        int n_factors, const float *rsasa, double water_weight,
                        int water_index, double *grad, int n_threads)
{
    grad_run(q, n_q, w_q, bodies, n_bodies, ff, n_factors, rsasa, water_weight, water_index,
             NULL, 0, grad, n_threads);
}

void orc_debye_grad_rows_f64(const double *q, int n_q, const double *w_q,
                             const float *bodies, int n_bodies, const float *ff,
                             int n_factors, const int *rows, int n_rows, double *grad,
                             int n_threads)
{
    grad_run(q, n_q, w_q, bodies, n_bodies, ff, n_factors, NULL, 0.0, 0, rows, n_rows, grad,
             n_threads);
}

/* Central differences of L = sum_q w_q I(q) along single coordinates: only
 * the pairs of the moved body change, so
 *   L(x+) - L(x-) = sum_q w_q 2 f_i(q) sum_{j != i} f_j(q)
 *                   [sinc(q |p_j - p_i(x+)|) - sinc(q |p_j - p_i(x-)|)]
 * (host_debye.cpp:74-108 restricted to row i), in FP64 with libm sin. */
typedef struct {
    const double *q, *w;
    int n_q;
    const float *bodies;
    int n;
    const double *f;
    const int *atom, *axis;
    const float *plus, *minus;
    int n_coords, next;
    pthread_mutex_t mu;
    double *out;
} fd_job;

static void *fd_worker(void *p)
{
    fd_job *J = (fd_job *)p;
    for (;;) {
        int c;
        pthread_mutex_lock(&J->mu);
        c = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (c >= J->n_coords)
            break;
        const int i = J->atom[c], ax = J->axis[c];
        double pp[3], pm[3];
        for (int a = 0; a < 3; ++a)
            pp[a] = pm[a] = J->bodies[4 * i + a];
        pp[ax] = J->plus[c];
        pm[ax] = J->minus[c];
        double dl = 0.0;
        for (int j = 0; j < J->n; ++j) {
            if (j == i)
                continue;
            const float *pj = &J->bodies[4 * j];
            double a2 = 0.0, b2 = 0.0;
            for (int a = 0; a < 3; ++a) {
                const double da = pp[a] - pj[a], db = pm[a] - pj[a];
                a2 += da * da;
                b2 += db * db;
            }
            const double ra = sqrt(a2), rb = sqrt(b2);
            double s = 0.0;
            for (int k = 0; k < J->n_q; ++k) {
                const double qk = J->q[k];
                const double xa = qk * ra, xb = qk * rb;
                const double sa = xa == 0.0 ? 1.0 : sin(xa) / xa;
                const double sb = xb == 0.0 ? 1.0 : sin(xb) / xb;
                s += J->w[k] * J->f[(size_t)k * J->n + i] * J->f[(size_t)k * J->n + j] * (sa - sb);
            }
            dl += 2.0 * s;
        }
        J->out[c] = dl / ((double)J->plus[c] - (double)J->minus[c]);
    }
    return NULL;
}

void orc_debye_fd_f64(const double *q, int n_q, const double *w_q, const float *bodies,
                      int n_bodies, const float *ff, int n_factors, const int *atom,
                      const int *axis, const float *plus, const float *minus, int n_coords,
                      double *out, int n_threads)
{
    int nt = pick_threads(n_threads);
    double *f = (double *)malloc(sizeof(double) * (size_t)n_q * n_bodies);
    for (int k = 0; k < n_q; ++k)
        for (int i = 0; i < n_bodies; ++i)
            f[(size_t)k * n_bodies + i] = ff[(size_t)k * n_factors + body_type(bodies, i)];
    fd_job J;
    J.q = q;
    J.w = w_q;
    J.n_q = n_q;
    J.bodies = bodies;
    J.n = n_bodies;
    J.f = f;
    J.atom = atom;
    J.axis = axis;
    J.plus = plus;
    J.minus = minus;
    J.n_coords = n_coords;
    J.next = 0;
    J.out = out;
    pthread_mutex_init(&J.mu, NULL);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nt);
    for (int t = 0; t < nt; ++t)
        pthread_create(&th[t], NULL, fd_worker, &J);
    for (int t = 0; t < nt; ++t)
        pthread_join(th[t], NULL);
    pthread_mutex_destroy(&J.mu);
    free(th);
    free(f);
}

/* ------------- reference-faithful port of host_debye -------------------- */

/* distance<double>(a, b): host_debye.cpp:36-42 */
static double port_distance(const float *a, const float *b)
{
    double dx = (double)a[0] - b[0];
    double dy = (double)a[1] - b[1];
    double dz = (double)a[2] - b[2];
    return sqrt(dx * dx + dy * dy + dz * dz);
}

static void port_q_range(const float *v_q, int k0, int k1, int n_bodies,
                         const double *r, const float *factors, float *out_v_iq)
{
    for (int k = k0; k < k1; k++) {
        double q = v_q[k];
        double Iq = 0;
        const float *Fq = &factors[(size_t)k * n_bodies];
        double auto_Iq = 0;
        for (int y = 0; y < n_bodies; y++) {
            double Fqy = Fq[y];
            auto_Iq += Fqy * Fqy;
            double inner_sum = 0;
            for (int x = 0; x < y; x++) {
                double v1 = 1;
                if (q != 0) {
                    double qr = q * r[(size_t)y * n_bodies + x];
                    v1 = sin(qr) / qr; /* utils.hpp sinc */
                }
                inner_sum += Fq[x] * v1;
            }
            Iq += inner_sum * Fqy;
        }
        out_v_iq[k] = (float)(Iq * 2 + auto_Iq);
    }
}

static double *port_matrix(const float *v_bodies, int n_bodies)
{
    double *r = (double *)malloc(sizeof(double) * (size_t)n_bodies * n_bodies);
    if (!r)
        return NULL;
    for (int y = 1; y < n_bodies; y++)
        for (int x = 0; x < y; x++)
            r[(size_t)y * n_bodies + x] = port_distance(&v_bodies[4 * x], &v_bodies[4 * y]);
    return r;
}

static float *port_factors(const float *v_bodies, int n_bodies, int n_q,
                           const float *t_factors, int n_factors)
{
    float *factors = (float *)malloc(sizeof(float) * (size_t)n_q * n_bodies);
    for (int k = 0; k < n_q; k++)
        for (int i = 0; i < n_bodies; i++)
            factors[(size_t)k * n_bodies + i] =
                t_factors[(size_t)k * n_factors + body_type(v_bodies, i)];
    return factors;
}

void orc_refport_host_debye(const float *v_q, int n_q, const float *v_bodies,
                            int n_bodies, const float *t_factors, int n_factors,
                            float *out_v_iq)
{
    double *r = port_matrix(v_bodies, n_bodies);
    float *factors = port_factors(v_bodies, n_bodies, n_q, t_factors, n_factors);
    port_q_range(v_q, 0, n_q, n_bodies, r, factors, out_v_iq);
    free(factors);
    free(r);
}

typedef struct {
    const float *v_q;
    int k0, k1, n;
    const double *r;
    const float *factors;
    float *out;
} port_arg;

static void *port_worker(void *p)
{
    port_arg *a = (port_arg *)p;
    port_q_range(a->v_q, a->k0, a->k1, a->n, a->r, a->factors, a->out);
    return NULL;
}

#include <time.h>
static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

double orc_refport_host_debye_mt(const float *v_q, int n_q, const float *v_bodies,
                                 int n_bodies, const float *t_factors,
                                 int n_factors, float *out_v_iq, int n_threads)
{
    int nt = pick_threads(n_threads);
    if (nt > n_q)
        nt = n_q;
    double t0 = now_s();
    double *r = port_matrix(v_bodies, n_bodies);
    double t_matrix = now_s() - t0;
    float *factors = port_factors(v_bodies, n_bodies, n_q, t_factors, n_factors);
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nt);
    port_arg *args = (port_arg *)malloc(sizeof(port_arg) * nt);
    for (int t = 0; t < nt; ++t) {
        args[t].v_q = v_q;
        args[t].k0 = (int)((long)n_q * t / nt);
        args[t].k1 = (int)((long)n_q * (t + 1) / nt);
        args[t].n = n_bodies;
        args[t].r = r;
        args[t].factors = factors;
        args[t].out = out_v_iq;
        pthread_create(&th[t], NULL, port_worker, &args[t]);
    }
    for (int t = 0; t < nt; ++t)
        pthread_join(th[t], NULL);
    free(th);
    free(args);
    free(factors);
    free(r);
    return t_matrix;
}

/* ---- the same loop over a sample of rows of the lower triangle ---------- */

typedef struct {
    const float *v_q;
    int k0, k1, n, n_rows;
    const int *rows;
    const double *r;       /* [n_rows][n]: row y's distances to x < y */
    const float *factors;  /* [n_q][n] */
    double *out;           /* [n_q] */
} rows_arg;

/* host_debye.cpp:74-104 for the rows y in `rows` only: the inner sum over
 * x < y, multiplied by F_q(y) and added to the partial, in the order and
 * mixed float/double arithmetic of the reference (auto terms and the final
 * "2 * Iq + auto" belong to the whole curve and are left out). */
static void *rows_worker(void *p)
{
    rows_arg *a = (rows_arg *)p;
    for (int k = a->k0; k < a->k1; k++) {
        double q = a->v_q[k];
        double Iq = 0;
        const float *Fq = &a->factors[(size_t)k * a->n];
        for (int s = 0; s < a->n_rows; s++) {
            const int y = a->rows[s];
            const double *ry = &a->r[(size_t)s * a->n];
            double Fqy = Fq[y];
            double inner_sum = 0;
            for (int x = 0; x < y; x++) {
                double v1 = 1;
                if (q != 0) {
                    double qr = q * ry[x];
                    v1 = sin(qr) / qr;
                }
                inner_sum += Fq[x] * v1;
            }
            Iq += inner_sum * Fqy;
        }
        a->out[k] = Iq;
    }
    return NULL;
}

int orc_refport_host_debye_rows(const float *v_q, int n_q, const float *v_bodies,
                                int n_bodies, const float *t_factors, int n_factors,
                                const int *rows, int n_rows, double *out_partial,
                                int n_threads)
{
    for (int s = 0; s < n_rows; s++)
        if (rows[s] < 0 || rows[s] >= n_bodies)
            return -1;
    int nt = pick_threads(n_threads);
    if (nt > n_q)
        nt = n_q;
    /* the distance rows, as host_debye.cpp:58-61 fills its matrix */
    double *r = (double *)malloc(sizeof(double) * (size_t)n_rows * (n_bodies > 0 ? n_bodies : 1));
    float *factors = port_factors(v_bodies, n_bodies, n_q, t_factors, n_factors);
    if (!r || !factors) {
        free(r);
        free(factors);
        return -2;
    }
    for (int s = 0; s < n_rows; s++) {
        const int y = rows[s];
        for (int x = 0; x < y; x++)
            r[(size_t)s * n_bodies + x] = port_distance(&v_bodies[4 * x], &v_bodies[4 * y]);
    }
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nt);
    rows_arg *args = (rows_arg *)malloc(sizeof(rows_arg) * nt);
    for (int t = 0; t < nt; ++t) {
        args[t].v_q = v_q;
        args[t].k0 = (int)((long)n_q * t / nt);
        args[t].k1 = (int)((long)n_q * (t + 1) / nt);
        args[t].n = n_bodies;
        args[t].n_rows = n_rows;
        args[t].rows = rows;
        args[t].r = r;
        args[t].factors = factors;
        args[t].out = out_partial;
        pthread_create(&th[t], NULL, rows_worker, &args[t]);
    }
    for (int t = 0; t < nt; ++t)
        pthread_join(th[t], NULL);
    free(th);
    free(args);
    free(factors);
    free(r);
    return 0;
}
