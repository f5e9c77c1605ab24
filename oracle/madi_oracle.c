/*
 * madi_oracle.c -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * CPU restatement of the reference MADI hot path (jadenfigger/Custom_MADI), used
 * only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
 * checker.  The product path (custom_madi_gb300) never calls it.
 *
 *   oracle_classify_kd     madi/walker_gpu.py:222-335 (stackless KD nearest +
 *                          adaptive ball d1 + 2 alpha_1; = Ensemble.classify_cpu,
 *                          madi/ensemble.py:213-256)
 *   oracle_classify_brute  all-seed SI Eq. S2 evaluation
 *                          (tests/physics_audit/test_geometry_diagnostics.py:119-140)
 *   oracle_walk            _walk_cpu transition, madi/walker_gpu.py:698-840, in
 *                          separately rounded fp64 (build with -ffp-contract=off);
 *                          periodic wrap and Philox draws are the GB300 extensions
 *   oracle_reduce          _reduce_cpu, madi/walker_gpu.py:954-968
 *   oracle_philox          Philox4x32-10 (Salmon et al., SC'11)
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int n_seeds;
    const double* seeds;      /* [n][3] */
    const double* annulus;    /* [n] */
    const int32_t* cell;      /* [n] base cell id (NULL = identity) */
    const int32_t* kd_seed;
    const int32_t* kd_left;
    const int32_t* kd_right;
    const int32_t* kd_parent;
    const int8_t* kd_axis;
    double L, source_lo, source_hi;
    int periodic;
    int has_cells;
} oracle_geom;

typedef struct {
    int n_walkers, n_steps, steps_per_h, n_grid;
    double sigma, ts, pp;
    int rng;                  /* 0 = Philox draws, 1 = replay stream */
    uint32_t key0, key1, walker_base;
    const double* init;       /* [n][3] */
    const double* incr;       /* [n_steps][n][3] */
    const double* unif;       /* [n_steps][n] */
    double* Y;                /* optional [n][n_grid][3] */
    int8_t* inside_trace;     /* optional [n][n_grid] */
    int n_pairs, n_b, n_dirs;
    const int32_t *jd, *jD, *js;
    const double* coef;       /* [n_pairs * n_b] */
    const double* dirs;       /* [n_dirs][3] */
    double* cos_sum;          /* optional [n_pairs * n_b * n_dirs] */
    double* sin_sum;
    int64_t* occupancy;       /* [n_grid] */
    int64_t counters[8];      /* walkers, escaped, classifier_error, full, -, -, accept, reject */
    int n_threads;
} oracle_walk_args;

/* ---------------------------------------------------------------- Philox */
typedef struct { uint32_t v[4]; } u4;

static u4 philox10(u4 c, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c.v[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c.v[2];
        u4 o;
        o.v[0] = (uint32_t)(p1 >> 32) ^ c.v[1] ^ k0;
        o.v[1] = (uint32_t)p1;
        o.v[2] = (uint32_t)(p0 >> 32) ^ c.v[3] ^ k1;
        o.v[3] = (uint32_t)p0;
        c = o;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

void oracle_philox(const uint32_t* ctr, uint32_t k0, uint32_t k1, uint32_t* out) {
    u4 c = {{ctr[0], ctr[1], ctr[2], ctr[3]}};
    u4 r = philox10(c, k0, k1);
    memcpy(out, r.v, 16);
}

/* ------------------------------------------------------------ classifier */
static double sq3(double x, double y, double z) { return x * x + y * y + z * z; }

static int kd_nearest(const oracle_geom* g, const double* p, double* d2o) {
    int node = 0, from = -1, best = -1;
    double bd = INFINITY;
    while (node >= 0) {
        int sid = g->kd_seed[node], ax = g->kd_axis[node];
        const double* c = g->seeds + 3 * (size_t)sid;
        double delta = p[ax] - c[ax];
        int l = g->kd_left[node], r = g->kd_right[node], up = g->kd_parent[node];
        int nr = delta <= 0.0 ? l : r, fr = delta <= 0.0 ? r : l, next;
        if (from == up) {
            double d2 = sq3(p[0] - c[0], p[1] - c[1], p[2] - c[2]);
            if (d2 < bd) { bd = d2; best = sid; }
            if (nr >= 0) next = nr;
            else if (fr >= 0 && delta * delta < bd) next = fr;
            else next = up;
        } else if (from == nr && fr >= 0 && delta * delta < bd) {
            next = fr;
        } else {
            next = up;
        }
        from = node;
        node = next;
    }
    *d2o = bd;
    return best;
}

/* returns 0 ok, -1 error; seed1 = nearest seed index */
static int classify_kd(const oracle_geom* g, const double* p, int* seed1, int* inside) {
    double d1sq;
    int s1 = kd_nearest(g, p, &d1sq);
    if (s1 < 0) return -1;
    const double* c1 = g->seeds + 3 * (size_t)s1;
    double a1 = g->annulus[s1];
    double rad = sqrt(d1sq) + 2.0 * a1;
    double rad2 = rad * rad;
    int node = 0, from = -1;
    *seed1 = s1;
    *inside = 1;
    while (node >= 0) {
        int sid = g->kd_seed[node], ax = g->kd_axis[node];
        const double* c = g->seeds + 3 * (size_t)sid;
        double delta = p[ax] - c[ax];
        int l = g->kd_left[node], r = g->kd_right[node], up = g->kd_parent[node];
        int nr = delta <= 0.0 ? l : r, fr = delta <= 0.0 ? r : l, next;
        int far_ok = fr >= 0 && delta * delta <= rad2;
        if (from == up) {
            double d2 = sq3(p[0] - c[0], p[1] - c[1], p[2] - c[2]);
            if (sid != s1 && d2 <= rad2) {
                double sep = sqrt(sq3(c[0] - c1[0], c[1] - c1[1], c[2] - c1[2]));
                if (sep <= 0.0) return -1;
                double margin = (d2 - d1sq) / (2.0 * sep);
                if (margin < a1) { *inside = 0; return 0; }
            }
            next = nr >= 0 ? nr : (far_ok ? fr : up);
        } else if (from == nr && far_ok) {
            next = fr;
        } else {
            next = up;
        }
        from = node;
        node = next;
    }
    return 0;
}

static int cell_of(const oracle_geom* g, int s) { return g->cell ? g->cell[s] : s; }

void oracle_classify_kd(const oracle_geom* g, int64_t n, const double* pts, int32_t* cell, uint8_t* inside) {
    for (int64_t i = 0; i < n; ++i) {
        int s = 0, in = 0;
        if (classify_kd(g, pts + 3 * i, &s, &in) != 0) { cell[i] = -1; inside[i] = 0; continue; }
        cell[i] = cell_of(g, s);
        inside[i] = (uint8_t)in;
    }
}

void oracle_classify_brute(const oracle_geom* g, int64_t n, const double* pts, int32_t* cell, uint8_t* inside) {
    for (int64_t i = 0; i < n; ++i) {
        const double* p = pts + 3 * i;
        int s1 = 0;
        double b = INFINITY;
        for (int j = 0; j < g->n_seeds; ++j) {
            const double* c = g->seeds + 3 * (size_t)j;
            double d2 = sq3(c[0] - p[0], c[1] - p[1], c[2] - p[2]);
            if (d2 < b) { b = d2; s1 = j; }
        }
        const double* c1 = g->seeds + 3 * (size_t)s1;
        int in = 1;
        for (int j = 0; j < g->n_seeds && in; ++j) {
            if (j == s1) continue;
            const double* c = g->seeds + 3 * (size_t)j;
            double d2 = sq3(c[0] - p[0], c[1] - p[1], c[2] - p[2]);
            double sep = sqrt(sq3(c[0] - c1[0], c[1] - c1[1], c[2] - c1[2]));
            if ((d2 - b) / (2.0 * sep) < g->annulus[s1]) in = 0;
        }
        cell[i] = cell_of(g, s1);
        inside[i] = (uint8_t)in;
    }
}

/* ------------------------------------------------------------------ walk */
typedef struct {
    const oracle_geom* g;
    oracle_walk_args* a;
    int w0, w1;
    double* cs;
    double* ss;
    int64_t* occ;
    int64_t cnt[8];
} job_t;

static void normals_for_step(const oracle_walk_args* a, uint32_t widx, int step, double* n3, uint32_t* word) {
    uint32_t pair = (uint32_t)step >> 1;
    u4 ra = philox10((u4){{widx, pair, 0u, 0u}}, a->key0, a->key1);
    u4 rb = philox10((u4){{widx, pair, 1u, 0u}}, a->key0, a->key1);
    double g[6];
    uint32_t w[6] = {ra.v[0], ra.v[1], ra.v[2], ra.v[3], rb.v[0], rb.v[1]};
    for (int k = 0; k < 3; ++k) {
        double u1 = (double)w[2 * k] * 2.3283064365386963e-10 + 1.1641532182693481e-10;
        double u2 = (double)(w[2 * k + 1] >> 8) * 5.9604644775390625e-08;
        double r = sqrt(-2.0 * log(u1));
        g[2 * k] = r * cos(6.283185307179586 * u2);
        g[2 * k + 1] = r * sin(6.283185307179586 * u2);
    }
    if ((step & 1) == 0) {
        n3[0] = g[0]; n3[1] = g[1]; n3[2] = g[2];
        *word = rb.v[2];
    } else {
        n3[0] = g[3]; n3[1] = g[4]; n3[2] = g[5];
        *word = rb.v[3];
    }
}

static void* walk_range(void* arg) {
    job_t* J = (job_t*)arg;
    const oracle_geom* g = J->g;
    oracle_walk_args* a = J->a;
    const int n = a->n_walkers, G = a->n_grid;
    const double L = g->L, half_L = L / 2.0, ts = a->ts, pp = a->pp;
    const int fused = a->cos_sum != NULL;
    const int n_out = a->n_pairs * a->n_b * a->n_dirs;
    double* Ysnap = (double*)calloc((size_t)G * 3, sizeof(double));
    double* dM = (double*)calloc((size_t)(a->n_pairs > 0 ? a->n_pairs : 1) * 3, sizeof(double));
    const uint64_t thr1 = (uint64_t)ldexp(pp, 64) , thr2 = (uint64_t)ldexp(pp * pp, 64);
    for (int w = J->w0; w < J->w1; ++w) {
        const uint32_t widx = a->walker_base + (uint32_t)w;
        double p[3];
        if (a->rng == 1) {
            p[0] = a->init[3 * (size_t)w]; p[1] = a->init[3 * (size_t)w + 1]; p[2] = a->init[3 * (size_t)w + 2];
        } else {
            u4 r = philox10((u4){{widx, 0u, 0u, 1u}}, a->key0, a->key1);
            double span = g->source_hi - g->source_lo;
            for (int k = 0; k < 3; ++k) p[k] = g->source_lo + span * ((double)r.v[k] * 2.3283064365386963e-10);
            if (g->periodic)
                for (int k = 0; k < 3; ++k) if (p[k] >= L) p[k] = 0.0;
        }
        int cell = 0, inside = 0, escaped = 0, cerr = 0, img[3] = {0, 0, 0};
        if (g->has_cells) {
            int s = 0;
            if (classify_kd(g, p, &s, &inside) != 0) cerr = 1;
            cell = cell_of(g, s);
            J->cnt[3]++;
        }
        double prev[3] = {p[0] - half_L, p[1] - half_L, p[2] - half_L};
        double Y[3] = {0.0, 0.0, 0.0};
        memset(Ysnap, 0, sizeof(double) * (size_t)G * 3);
        if (a->inside_trace) a->inside_trace[(size_t)w * G] = (int8_t)inside;
        if (inside) J->occ[0]++;
        for (int step = 0; step < a->n_steps; ++step) {
            if (!escaped && !cerr) {
                double inc[3], u = 0.0;
                uint32_t word = 0;
                if (a->rng == 1) {
                    size_t o = (size_t)step * n + w;
                    inc[0] = a->incr[3 * o]; inc[1] = a->incr[3 * o + 1]; inc[2] = a->incr[3 * o + 2];
                    u = a->unif[o];
                } else {
                    normals_for_step(a, widx, step, inc, &word);
                    for (int k = 0; k < 3; ++k) inc[k] *= a->sigma;
                }
                double q[3] = {p[0] + inc[0], p[1] + inc[1], p[2] + inc[2]};
                int qimg[3] = {img[0], img[1], img[2]};
                int ok = 1;
                if (g->periodic) {
                    for (int k = 0; k < 3; ++k) {
                        if (q[k] < 0.0) { q[k] = q[k] + L; qimg[k]--; }
                        if (q[k] >= L) { q[k] = q[k] - L; qimg[k]++; }
                    }
                } else if (q[0] < 0.0 || q[0] >= L || q[1] < 0.0 || q[1] >= L || q[2] < 0.0 || q[2] >= L) {
                    escaped = 1;
                    ok = 0;
                }
                if (ok) {
                    int ncell = 0, nin = 0;
                    if (g->has_cells) {
                        int s = 0;
                        if (classify_kd(g, q, &s, &nin) != 0) cerr = 1;
                        ncell = cell_of(g, s);
                        J->cnt[3]++;
                    }
                    if (!cerr) {
                        int m = 0;
                        if (inside && !nin) m = 1;
                        else if (!inside && nin) m = 1;
                        else if (inside && nin && cell != ncell) m = 2;
                        int accept = 1;
                        if (m > 0 && pp < 1.0) {
                            if (a->rng == 1) {
                                accept = !(u >= (m == 1 ? pp : pp * pp));
                            } else {
                                uint64_t thr = m == 1 ? thr1 : thr2;
                                uint32_t th = (uint32_t)(thr >> 32);
                                if (word != th) accept = word < th;
                                else {
                                    u4 rc = philox10((u4){{widx, (uint32_t)step, 2u, 0u}}, a->key0, a->key1);
                                    accept = rc.v[0] < (uint32_t)thr;
                                }
                            }
                            if (accept) J->cnt[6]++; else J->cnt[7]++;
                        }
                        if (accept) {
                            for (int k = 0; k < 3; ++k) { p[k] = q[k]; img[k] = qimg[k]; }
                            cell = ncell;
                            inside = nin;
                        }
                        for (int k = 0; k < 3; ++k) {
                            double cur = p[k] - half_L;
                            if (g->periodic) cur = cur + (double)img[k] * L;
                            Y[k] += 0.5 * (prev[k] + cur) * ts;
                            prev[k] = cur;
                        }
                    }
                }
            }
            int si = step + 1;
            if (si % a->steps_per_h == 0) {
                int j = si / a->steps_per_h;
                for (int k = 0; k < 3; ++k) Ysnap[3 * j + k] = Y[k];
                if (a->inside_trace) a->inside_trace[(size_t)w * G + j] = (int8_t)inside;
                if (inside) J->occ[j]++;
            }
        }
        J->cnt[0]++;
        if (escaped) J->cnt[1]++;
        if (cerr) J->cnt[2]++;
        if (a->Y) memcpy(a->Y + (size_t)w * G * 3, Ysnap, sizeof(double) * (size_t)G * 3);
        if (fused && !escaped && !cerr) {
            for (int q = 0; q < a->n_pairs; ++q)
                for (int k = 0; k < 3; ++k)
                    dM[3 * q + k] = Ysnap[3 * a->jd[q] + k] + Ysnap[3 * a->jD[q] + k] - Ysnap[3 * a->js[q] + k];
            for (int q = 0; q < a->n_pairs; ++q)
                for (int u = 0; u < a->n_dirs; ++u) {
                    const double* e = a->dirs + 3 * u;
                    double proj = e[0] * dM[3 * q] + e[1] * dM[3 * q + 1] + e[2] * dM[3 * q + 2];
                    for (int b = 0; b < a->n_b; ++b) {
                        double ph = a->coef[q * a->n_b + b] * proj;
                        int o = (q * a->n_b + b) * a->n_dirs + u;
                        J->cs[o] += cos(ph);
                        J->ss[o] += sin(ph);
                    }
                }
        }
    }
    (void)n_out;
    free(Ysnap);
    free(dM);
    return NULL;
}

int oracle_walk(const oracle_geom* g, oracle_walk_args* a) {
    int T = a->n_threads > 0 ? a->n_threads : 1;
    if (T > a->n_walkers) T = a->n_walkers > 0 ? a->n_walkers : 1;
    const int n_out = a->n_pairs * a->n_b * a->n_dirs;
    job_t* jobs = (job_t*)calloc((size_t)T, sizeof(job_t));
    pthread_t* th = (pthread_t*)calloc((size_t)T, sizeof(pthread_t));
    for (int t = 0; t < T; ++t) {
        jobs[t].g = g;
        jobs[t].a = a;
        jobs[t].w0 = (int)((int64_t)a->n_walkers * t / T);
        jobs[t].w1 = (int)((int64_t)a->n_walkers * (t + 1) / T);
        jobs[t].cs = (double*)calloc((size_t)(n_out > 0 ? n_out : 1), sizeof(double));
        jobs[t].ss = (double*)calloc((size_t)(n_out > 0 ? n_out : 1), sizeof(double));
        jobs[t].occ = (int64_t*)calloc((size_t)a->n_grid, sizeof(int64_t));
    }
    for (int t = 1; t < T; ++t) pthread_create(&th[t], NULL, walk_range, &jobs[t]);
    walk_range(&jobs[0]);
    for (int t = 1; t < T; ++t) pthread_join(th[t], NULL);
    memset(a->counters, 0, sizeof(a->counters));
    for (int t = 0; t < T; ++t) {
        for (int k = 0; k < 8; ++k) a->counters[k] += jobs[t].cnt[k];
        for (int j = 0; j < a->n_grid; ++j) if (a->occupancy) a->occupancy[j] += jobs[t].occ[j];
        if (a->cos_sum)
            for (int o = 0; o < n_out; ++o) { a->cos_sum[o] += jobs[t].cs[o]; a->sin_sum[o] += jobs[t].ss[o]; }
        free(jobs[t].cs); free(jobs[t].ss); free(jobs[t].occ);
    }
    free(jobs);
    free(th);
    return 0;
}

void oracle_reduce(const double* Y, int64_t n, int n_grid, const int32_t* jd, const int32_t* jD,
                   const int32_t* js, const double* coef, int n_cols, double* cos_sum, double* sin_sum) {
    for (int c = 0; c < n_cols; ++c) {
        double cs = 0.0, ss = 0.0;
        for (int64_t w = 0; w < n; ++w)
            for (int k = 0; k < 3; ++k) {
                const double* y = Y + (size_t)w * n_grid * 3;
                double dm = y[3 * jd[c] + k] + y[3 * jD[c] + k] - y[3 * js[c] + k];
                double ph = coef[c] * dm;
                cs += cos(ph);
                ss += sin(ph);
            }
        cos_sum[c] = cs;
        sin_sum[c] = ss;
    }
}
