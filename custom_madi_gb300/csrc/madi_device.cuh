// Device building blocks of the GB300 MADI walker: counter-based RNG, the
// geometry view, and three classifiers of the SI Eq. S2 contracted-Voronoi rule
// (point p, nearest seed c1, per-seed annulus alpha): p is intracellular iff for
// every other seed cj the signed distance of p to the c1|cj bisector plane,
//     m_j(p) = (|p - cj|^2 - |p - c1|^2) / (2 |c1 - cj|),
// is at least alpha_1 (madi/ensemble.py:213-256, madi/walker_gpu.py:272-335).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/madi_gb300.h"

#define MADI_DEV __device__ __forceinline__

namespace madi {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies on a 4-word counter
// under a 2-word key, key bumped by the Weyl constants between rounds.
// ---------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };

MADI_DEV U4 philox10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// Two independent N(0,1) from two words (Box-Muller).  u1 in (0, 1], u2 in [0, 1).
MADI_DEV void box_muller(uint32_t a, uint32_t b, float& g0, float& g1) {
    const float u1 = fmaf((float)a, 2.3283064365386963e-10f, 1.1641532182693481e-10f);
    const float u2 = (float)(b >> 8) * 5.9604644775390625e-08f;
    const float r = sqrtf(-2.0f * __logf(u1));
    float s, c;
    __sincosf(6.283185307179586f * u2, &s, &c);
    g0 = r * c;
    g1 = r * s;
}

// ---------------------------------------------------------------------------
// Geometry view.  `base` is either shared memory (staged) or the global stage
// buffer; both carry the layout of madi_geometry (include/madi_gb300.h).
// ---------------------------------------------------------------------------
struct Geo {
    const float4* seed;         // x, y, z (fp32), alpha (fp32)
    const int32_t* cell;
    const uint32_t* off;
    const void* ids;
    const double* f64;          // [n][4] in global memory
    const int32_t *kd_seed, *kd_left, *kd_right, *kd_parent;
    const int8_t* kd_axis;
    int ids_u32;
    int G;
    float inv_h;
    float L;
    float cap;
    float cerr;                 // |fp32 seed - exact seed| per axis
    int n_seeds;
    // cell facet table (n_cells = 0: none)
    const float4* ccen;         // [n_cells] base seed x, y, z, alpha
    int fstride;                // facet slots per cell (multiple of 32)
    const float4* fpl;          // [n_cells][fstride] unit normal, offset
    const int32_t* fnbr;        // [n_cells][fstride] cell across the facet
    int n_cells;
    float ftol;                 // fp32 error of a facet margin, without the |w| term
};

MADI_DEV Geo make_geo(const madi_geometry& g, const unsigned char* base) {
    Geo v;
    v.seed = reinterpret_cast<const float4*>(base);
    v.cell = reinterpret_cast<const int32_t*>(base + g.off_cell);
    v.off = reinterpret_cast<const uint32_t*>(base + g.off_grid_offset);
    v.ids = base + g.off_grid_ids;
    v.f64 = g.seed_f64;
    v.kd_seed = g.kd_seed; v.kd_left = g.kd_left; v.kd_right = g.kd_right;
    v.kd_parent = g.kd_parent; v.kd_axis = g.kd_axis;
    v.ids_u32 = g.ids_u32;
    v.G = g.grid_n;
    v.inv_h = (float)(1.0 / g.grid_h);
    v.L = (float)g.L;
    v.cap = (float)g.safe_cap;
    v.cerr = (float)g.coord_err;
    v.n_seeds = g.n_seeds;
    v.ccen = reinterpret_cast<const float4*>(base + g.off_cell_center);
    v.fstride = (int)g.facet_stride;
    v.fpl = reinterpret_cast<const float4*>(base + g.off_facet_plane);
    v.fnbr = reinterpret_cast<const int32_t*>(base + g.off_facet_nbr);
    v.n_cells = g.n_cells;
    v.ftol = (float)g.facet_tol;
    return v;
}

MADI_DEV int cand_id(const Geo& g, uint32_t k) {
    return g.ids_u32 ? (int)reinterpret_cast<const uint32_t*>(g.ids)[k]
                     : (int)reinterpret_cast<const uint16_t*>(g.ids)[k];
}

MADI_DEV int voxel_of(const Geo& g, float px, float py, float pz) {
    int ix = (int)(px * g.inv_h), iy = (int)(py * g.inv_h), iz = (int)(pz * g.inv_h);
    ix = min(max(ix, 0), g.G - 1);
    iy = min(max(iy, 0), g.G - 1);
    iz = min(max(iz, 0), g.G - 1);
    return (iz * g.G + iy) * g.G + ix;
}

MADI_DEV int cell_of(const Geo& g, int seed) { return g.cell[seed]; }

enum { CLS_OK = 0, CLS_FALLBACK = 1, CLS_ERROR = 2, CLS_NOT_NEAREST = 3 };

#define MADI_EPS21 4.76837158203125e-07f   // 2^-21
#define MADI_EPS19 1.9073486328125e-06f    // 2^-19

// ---------------------------------------------------------------------------
// fp32 voxel-grid classifier.
//
// For nearest seed c1 the shifted-facet margin of p w.r.t. seed cj is the signed
// distance of p to their bisector plane,  m_j = u.(cj + c1 - 2p) / (2|u|),
// u = cj - c1, and p is intracellular iff m_j >= alpha_1 for every j.  The fp32
// value carries the error bound
//   tol_j = 2 [ e (1 + |w|/|u|) + 2^-21 (|p-c1| + |p-cj| + |w| + |m_j|) ],
// w = 2p - cj - c1, e the per-axis fp32 seed rounding; decisions inside the
// band go to the fp64 rule (CLS_FALLBACK).  The same pass proves nearestness:
// m_j < 0 means cj is closer than c1 (CLS_NOT_NEAREST).
//
// rsafe receives a proven lower bound on the distance from p to the nearest
// point whose label differs (capped at g.cap):
//   inside : min_j (m_j - alpha_1)                   (distance to the shrunk facets)
//   outside: min( alpha_1 - min_j m_j,               (distance to the own shrunk cell)
//                 min_{i != 1} (m_i + alpha_i) )      (distance to any other shrunk cell)
// Seeds absent from the voxel list have m > alpha_max + cap, so they cannot lower it.
// ---------------------------------------------------------------------------
MADI_DEV int margins_pass(const Geo& g, float px, float py, float pz, uint32_t b, uint32_t e, int bi,
                          int& inside, float& rsafe) {
    const float4 h1 = g.seed[bi];
    const float a1 = h1.w;
    const float bx = px - h1.x, by = py - h1.y, bz = pz - h1.z;
    const float t0 = g.cerr + MADI_EPS21 * 3.0f * (fabsf(bx) + fabsf(by) + fabsf(bz));
    bool out_sure = false, amb = false, found = false, tie = false;
    float r_in = 3.0e38f, r_other = 3.0e38f, m_min_up = 3.0e38f;
    for (uint32_t k = b; k < e; ++k) {
        const int id = cand_id(g, k);
        if (id == bi) { found = true; continue; }
        const float4 h = g.seed[id];
        const float ux = h.x - h1.x, uy = h.y - h1.y, uz = h.z - h1.z;
        const float wx = (px - h.x) + bx, wy = (py - h.y) + by, wz = (pz - h.z) + bz;
        const float num = -fmaf(ux, wx, fmaf(uy, wy, uz * wz));
        const float rs = rsqrtf(fmaf(ux, ux, fmaf(uy, uy, uz * uz)));
        const float m = 0.5f * num * rs;
        const float wl = fabsf(wx) + fabsf(wy) + fabsf(wz);
        const float tol = 2.0f * (t0 + wl * fmaf(g.cerr, rs, 2.0f * MADI_EPS21) + MADI_EPS21 * (fabsf(m) + a1 + h.w));
        if (m < -tol) return CLS_NOT_NEAREST;
        const float dm = m - a1;
        out_sure |= dm < -tol;
        amb |= fabsf(dm) <= tol;
        r_in = fminf(r_in, dm - tol);
        m_min_up = fminf(m_min_up, m + tol);
        r_other = fminf(r_other, m - tol + h.w);
        tie |= m <= tol;                     // nearest seed not decided in fp32
    }
    if (!found) return CLS_NOT_NEAREST;
    if (tie) return CLS_FALLBACK;
    if (out_sure) {
        inside = 0;
        const float r = fminf(a1 * (1.0f - MADI_EPS19) - m_min_up, r_other);
        rsafe = fminf(fmaxf(r, 0.0f), g.cap);
        return CLS_OK;
    }
    if (amb) return CLS_FALLBACK;
    inside = 1;
    rsafe = fminf(fmaxf(r_in, 0.0f), g.cap);
    return CLS_OK;
}

// guess: the nearest seed of a nearby earlier point (or -1).  One pass when the
// guess is still nearest, else a nearest search over the list and a second pass.
MADI_DEV int classify_f32(const Geo& g, float px, float py, float pz, int guess,
                          int& seed1, int& inside, float& rsafe) {
    const int v = voxel_of(g, px, py, pz);
    const uint32_t b = g.off[v], e = g.off[v + 1];
    if (b >= e) return CLS_ERROR;
    if (guess >= 0) {
        const int st = margins_pass(g, px, py, pz, b, e, guess, inside, rsafe);
        if (st != CLS_NOT_NEAREST) { seed1 = guess; return st; }
    }
    float best = 3.0e38f, second = 3.0e38f;
    int bi = -1;
    for (uint32_t k = b; k < e; ++k) {
        const int id = cand_id(g, k);
        const float4 h = g.seed[id];
        const float ax = px - h.x, ay = py - h.y, az = pz - h.z;
        const float d2 = fmaf(ax, ax, fmaf(ay, ay, az * az));
        if (d2 < best) { second = best; best = d2; bi = id; }
        else if (d2 < second) { second = d2; }
    }
    if (second - best <= MADI_EPS19 * second + 8.0f * g.cerr * sqrtf(second)) return CLS_FALLBACK;
    seed1 = bi;
    const int st = margins_pass(g, px, py, pz, b, e, bi, inside, rsafe);
    return st == CLS_NOT_NEAREST ? CLS_FALLBACK : st;
}

// ---------------------------------------------------------------------------
// Warp-cooperative form of classify_f32: the 32 lanes of a warp classify ONE
// point together, lane l taking candidates b + l, b + l + 32, ... of its voxel
// list, and combine with warp reductions.  Same arithmetic per candidate and
// the same decisions as the per-lane form; every lane returns the same result.
// Called in warp-uniform control flow only.
// ---------------------------------------------------------------------------
#define MADI_FULL 0xffffffffu

// Order-preserving int image of a float, for integer warp min-reductions.
MADI_DEV int f2o(float f) { const int i = __float_as_int(f); return i >= 0 ? i : i ^ 0x7FFFFFFF; }
MADI_DEV float o2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }
MADI_DEV float warp_minf(float v) { return o2f(__reduce_min_sync(MADI_FULL, f2o(v))); }

// Warp-cooperative margins pass for seed bi over the candidate list [b, e):
// the lanes split the candidates, then vote.  Same decisions and error bands
// as margins_pass.
MADI_DEV int coop_margins(const Geo& g, float px, float py, float pz, uint32_t b, uint32_t e, int bi, int lane,
                          int& inside) {
    const float4 h1 = g.seed[bi];
    const float a1 = h1.w;
    const float bx = px - h1.x, by = py - h1.y, bz = pz - h1.z;
    const float t0 = g.cerr + MADI_EPS21 * 3.0f * (fabsf(bx) + fabsf(by) + fabsf(bz));
    bool not_near = false, out_sure = false, amb = false, found = false, tie = false;
    for (uint32_t k = b + lane; k < e; k += 32) {
        const int id = cand_id(g, k);
        if (id == bi) { found = true; continue; }
        const float4 h = g.seed[id];
        const float ux = h.x - h1.x, uy = h.y - h1.y, uz = h.z - h1.z;
        const float wx = (px - h.x) + bx, wy = (py - h.y) + by, wz = (pz - h.z) + bz;
        const float num = -fmaf(ux, wx, fmaf(uy, wy, uz * wz));
        const float rs = rsqrtf(fmaf(ux, ux, fmaf(uy, uy, uz * uz)));
        const float m = 0.5f * num * rs;
        const float wl = fabsf(wx) + fabsf(wy) + fabsf(wz);
        const float tol = 2.0f * (t0 + wl * fmaf(g.cerr, rs, 2.0f * MADI_EPS21) + MADI_EPS21 * (fabsf(m) + a1 + h.w));
        const float dm = m - a1;
        not_near |= m < -tol;
        out_sure |= dm < -tol;
        amb |= fabsf(dm) <= tol;
        tie |= m <= tol;
    }
    if (__any_sync(MADI_FULL, not_near) || !__any_sync(MADI_FULL, found)) return CLS_NOT_NEAREST;
    if (__any_sync(MADI_FULL, tie)) return CLS_FALLBACK;
    const bool outside = __any_sync(MADI_FULL, out_sure);
    if (!outside && __any_sync(MADI_FULL, amb)) return CLS_FALLBACK;
    inside = outside ? 0 : 1;
    return CLS_OK;
}

MADI_DEV int coop_nearest(const Geo& g, float px, float py, float pz, uint32_t b, uint32_t e, int lane, int& bi) {
    float best = 3.0e38f, second = 3.0e38f;
    int id_best = -1;
    for (uint32_t k = b + lane; k < e; k += 32) {
        const int id = cand_id(g, k);
        const float4 h = g.seed[id];
        const float ax = px - h.x, ay = py - h.y, az = pz - h.z;
        const float d2 = fmaf(ax, ax, fmaf(ay, ay, az * az));
        if (d2 < best) { second = best; best = d2; id_best = id; }
        else if (d2 < second) { second = d2; }
    }
    // d2 >= 0, so the float bit patterns order like unsigned integers.
    const unsigned key = __float_as_uint(best);
    const unsigned kmin = __reduce_min_sync(MADI_FULL, key);
    const unsigned who = __ballot_sync(MADI_FULL, key == kmin);
    const int src = __ffs(who) - 1;
    bi = __shfl_sync(MADI_FULL, id_best, src);
    const float sec = lane == src ? second : best;
    const float smin = __uint_as_float(__reduce_min_sync(MADI_FULL, __float_as_uint(sec)));
    const float bmin = __uint_as_float(kmin);
    if (__popc(who) > 1 || smin - bmin <= MADI_EPS19 * smin + 8.0f * g.cerr * sqrtf(smin)) return CLS_FALLBACK;
    return CLS_OK;
}

// Classify point p cooperatively; guess = a seed likely to be nearest or -1.
MADI_DEV int coop_classify(const Geo& g, float px, float py, float pz, int guess, int lane, int& seed1, int& inside) {
    const int v = voxel_of(g, px, py, pz);
    const uint32_t b = g.off[v], e = g.off[v + 1];
    if (b >= e) return CLS_ERROR;
    if (guess >= 0) {
        const int st = coop_margins(g, px, py, pz, b, e, guess, lane, inside);
        if (st != CLS_NOT_NEAREST) { seed1 = guess; return st; }
    }
    int bi = 0;
    const int st = coop_nearest(g, px, py, pz, b, e, lane, bi);
    if (st != CLS_OK) return st;
    seed1 = bi;
    const int st2 = coop_margins(g, px, py, pz, b, e, bi, lane, inside);
    return st2 == CLS_NOT_NEAREST ? CLS_FALLBACK : st2;
}

// ---------------------------------------------------------------------------
// Facet-plane labels.  For q in the Voronoi cell of base seed c the margins
// to all other seeds are bounded below by the distances to the cell's own
// facet planes, m_k(q) = h_k - n_k.w with w = q - c (periodic: the nearest
// image), so the cell's facet list alone decides the SI Eq. S2 label:
//   min_k m_k > T and min_k m_k - alpha_c > T   -> intracellular, cell c
//   min_k m_k > T and min_k m_k - alpha_c < -T  -> extracellular, Voronoi cell c
//   min_k m_k < -T                              -> q is in another cell
// T bounds the fp32 error of m_k (seed rounding, stored n and h, the
// subtraction and wrap of w, three fused multiply-adds):
//   |m - m_exact| <= 2 e + 2^-21 (h + |w|_1 + L),   e = per-axis seed error,
// taken twice; ftol holds the part without |w|_1.
// ---------------------------------------------------------------------------
enum { FACET_OUT = 0, FACET_IN = 1, FACET_LEFT = -1, FACET_BAND = -2 };

MADI_DEV float facet_m(const float4 f, float wx, float wy, float wz) {
    return fmaf(-f.z, wz, fmaf(-f.y, wy, fmaf(-f.x, wx, f.w)));
}

// Result of a full facet pass: the three facets of smallest margin (slots
// k1..k3), the smallest margin m1, a lower bound m4 on every other facet's
// margin, the cell across the most violated facet, the point w relative to the
// cell centre cc, and the error bound T at w.
struct FacetTop {
    float m1, m4;
    uint32_t k1, k2, k3;
    int nb1;                    // cell across the facet of margin m1
    float wx, wy, wz, T;
    float4 cc;
};

// ---------------------------------------------------------------------------
// fp64 rule on the voxel candidate list: nearest seed, then every seed within
// d1 + 2 alpha_1 must satisfy m_j >= alpha_1 (madi/walker_gpu.py:284-335).  No
// fused multiply-add, matching the separately rounded numpy expressions.
// ---------------------------------------------------------------------------
MADI_DEV double dsq3(double x, double y, double z) {
    return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}

MADI_DEV int classify_list_f64(const Geo& g, double px, double py, double pz,
                               int& seed1, int& inside) {
    const float fx = (float)px, fy = (float)py, fz = (float)pz;
    const int v = voxel_of(g, fx, fy, fz);
    const uint32_t b = g.off[v], e = g.off[v + 1];
    if (b >= e) return CLS_ERROR;
    double best = 1.0e300;
    int bi = -1;
    for (uint32_t k = b; k < e; ++k) {
        const int id = cand_id(g, k);
        const double* c = g.f64 + 4 * (size_t)id;
        const double d2 = dsq3(__dsub_rn(px, c[0]), __dsub_rn(py, c[1]), __dsub_rn(pz, c[2]));
        if (d2 < best || (d2 == best && id < bi)) { best = d2; bi = id; }
    }
    const double* c1 = g.f64 + 4 * (size_t)bi;
    const double a1 = c1[3];
    const double rad = __dadd_rn(sqrt(best), __dmul_rn(2.0, a1));
    const double rad2 = __dmul_rn(rad, rad);
    inside = 1;
    for (uint32_t k = b; k < e; ++k) {
        const int id = cand_id(g, k);
        if (id == bi) continue;
        const double* c = g.f64 + 4 * (size_t)id;
        const double d2 = dsq3(__dsub_rn(px, c[0]), __dsub_rn(py, c[1]), __dsub_rn(pz, c[2]));
        if (!(d2 <= rad2)) continue;
        const double sep = sqrt(dsq3(__dsub_rn(c[0], c1[0]), __dsub_rn(c[1], c1[1]), __dsub_rn(c[2], c1[2])));
        if (sep <= 0.0) return CLS_ERROR;
        const double margin = __ddiv_rn(__dsub_rn(d2, best), __dmul_rn(2.0, sep));
        if (margin < a1) { inside = 0; break; }
    }
    seed1 = bi;
    return CLS_OK;
}

// ---------------------------------------------------------------------------
// fp64 stackless KD traversal with parent links (exact nearest, then the exact
// ball d1 + 2 alpha_1): the reference device rule of madi/walker_gpu.py:222-335.
// The tree and seeds live in global memory.
// ---------------------------------------------------------------------------
MADI_DEV double coord(double x, double y, double z, int axis) {
    return axis == 0 ? x : (axis == 1 ? y : z);
}

MADI_DEV int kd_nearest_f64(const Geo& g, double px, double py, double pz, double& d2_out) {
    int node = 0, from = -1, best_seed = -1;
    double best = 1.0e300;
    while (node >= 0) {
        const int sid = g.kd_seed[node];
        const int axis = g.kd_axis[node];
        const double* c = g.f64 + 4 * (size_t)sid;
        const double delta = __dsub_rn(coord(px, py, pz, axis), c[axis]);
        const int left = g.kd_left[node], right = g.kd_right[node], up = g.kd_parent[node];
        const int near_c = delta <= 0.0 ? left : right;
        const int far_c = delta <= 0.0 ? right : left;
        int next;
        if (from == up) {
            const double d2 = dsq3(__dsub_rn(px, c[0]), __dsub_rn(py, c[1]), __dsub_rn(pz, c[2]));
            if (d2 < best) { best = d2; best_seed = sid; }
            if (near_c >= 0) next = near_c;
            else if (far_c >= 0 && __dmul_rn(delta, delta) < best) next = far_c;
            else next = up;
        } else if (from == near_c && far_c >= 0 && __dmul_rn(delta, delta) < best) {
            next = far_c;
        } else {
            next = up;
        }
        from = node;
        node = next;
    }
    d2_out = best;
    return best_seed;
}

MADI_DEV int classify_kd_f64(const Geo& g, double px, double py, double pz, int& seed1, int& inside) {
    double d1sq;
    const int s1 = kd_nearest_f64(g, px, py, pz, d1sq);
    if (s1 < 0) return CLS_ERROR;
    const double* c1 = g.f64 + 4 * (size_t)s1;
    const double a1 = c1[3];
    const double rad = __dadd_rn(sqrt(d1sq), __dmul_rn(2.0, a1));
    const double rad2 = __dmul_rn(rad, rad);
    int node = 0, from = -1;
    seed1 = s1;
    inside = 1;
    while (node >= 0) {
        const int sid = g.kd_seed[node];
        const int axis = g.kd_axis[node];
        const double* c = g.f64 + 4 * (size_t)sid;
        const double delta = __dsub_rn(coord(px, py, pz, axis), c[axis]);
        const int left = g.kd_left[node], right = g.kd_right[node], up = g.kd_parent[node];
        const int near_c = delta <= 0.0 ? left : right;
        const int far_c = delta <= 0.0 ? right : left;
        const bool far_ok = far_c >= 0 && __dmul_rn(delta, delta) <= rad2;
        int next;
        if (from == up) {
            const double d2 = dsq3(__dsub_rn(px, c[0]), __dsub_rn(py, c[1]), __dsub_rn(pz, c[2]));
            if (sid != s1 && d2 <= rad2) {
                const double sep = sqrt(dsq3(__dsub_rn(c[0], c1[0]), __dsub_rn(c[1], c1[1]),
                                             __dsub_rn(c[2], c1[2])));
                if (sep <= 0.0) return CLS_ERROR;
                const double margin = __ddiv_rn(__dsub_rn(d2, d1sq), __dmul_rn(2.0, sep));
                if (margin < a1) { inside = 0; return CLS_OK; }
            }
            next = near_c >= 0 ? near_c : (far_ok ? far_c : up);
        } else if (from == near_c && far_ok) {
            next = far_c;
        } else {
            next = up;
        }
        from = node;
        node = next;
    }
    return CLS_OK;
}

// Index of the job owning work tile `t` (jobs sorted by tile_begin).
MADI_DEV int find_job(const madi_walk_job* jobs, int n_jobs, int t) {
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].tile_begin <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

}  // namespace madi
