// GB300 walker: one persistent launch walks every (ensemble, p_p) job of a
// batch.  Work unit = a tile of `tile_walkers` walkers (one per thread) of one
// job; CTAs pull tiles from a device counter and stage the tile's geometry
// (seeds, voxel candidate lists, cell facet table) into shared memory when it
// changes and fits.
//
// Per step and walker (fp32 state, madi/walker_gpu.py:574-655 transition):
//   propose x' = x + N(0, sigma^2 I)  (Philox4x32-10 + Box-Muller),
//   boundary: fatal escape (SI) or periodic wrap,
//   classify x' (the walker's label cache of three facet planes, else a
//   warp-cooperative pass over its cell's facets, else the voxel-grid rule,
//   else fp64),
//   m = endpoint membrane count, accept iff U64 < pp^m * 2^64, else revert,
//   Y'(t) = int_0^t (x - x0) dt by the step trapezoid (fp32 within one storage
//   interval, fp64 across intervals).
// At the end the phase epilogue forms dM = Y(delta) + Y(Delta) - Y(Delta+delta)
// per pair and axis and sums cos / sin(coef * u.dM) over the tile in exact
// 64-bit fixed point.
#include <cstdio>
#include <cstring>
#include <cmath>
#include "madi_device.cuh"
#include "madi_host.h"

namespace madi {

// Per Y grid point: coefficient k_p in {-1, 0, 1, 2} of Y(t_j) in the pair-p
// moment dM_p = Y(delta) + Y(Delta) - Y(Delta + delta), packed 2 bits per pair.
struct Snap { uint32_t code, any; };
MADI_DEV float snap_coef(uint32_t code, int p) { return (float)((int)((code >> (2 * p)) & 3u) - 1); }

// Y relative to x0 -> the reference's origin L/2 (madi/walker_gpu.py:562-564).
MADI_DEV double y_ref(double yrel, double x0, double half_L, double t) {
    return yrel + (x0 - half_L) * t;
}

// Shared-memory blocks of one CTA besides the staged geometry.
struct TileShared {
    long long* acc;       // [2 n_out] fixed-point cos / sin sums of the tile
    unsigned int* occ;    // [n_grid] inside counts
    const Snap* snap;     // [n_grid] moment coefficients
    double* auxd;         // [3][blockDim.x] Y' at the last storage point (fp64)
    float* auxf;          // [3 + 3 NP][blockDim.x] interval-start displacement, moments dM
    float4* fc;           // [5][blockDim.x] per-walker label cache (two facet planes + sphere)
    uint32_t* auxc;       // [3][blockDim.x] rare counters: fp64 fallbacks, accepted, rejected crossings
};

// Per-walker state touched once per storage interval lives in shared memory
// (structure of arrays, one column per thread) to keep the step loop in registers.
#define AUX_Y(k) ts.auxd[(k) * blockDim.x + threadIdx.x]
#define AUX_A(k) ts.auxf[(k) * blockDim.x + threadIdx.x]
#define AUX_M(p, k) ts.auxf[(3 + 3 * (p) + (k)) * blockDim.x + threadIdx.x]
#define AUX_C(k) ts.auxc[(k) * blockDim.x + threadIdx.x]
#define FC(k) ts.fc[(k) * blockDim.x + threadIdx.x]

// Per-walker label cache, built at a point q0 of cell c by a full facet pass
// (facets k1, k2, k3 of smallest margin, every other facet's margin >= m4 as
// computed; error bound T0 at q0):
//   FC(0..2) = facets k1, k2, k3 (n, h);   FC(3) = (w0, R^2);
//   FC(4) = (c, alpha_c + Tm);   FC(5) = (alpha_c - Tm, Tm, c, cell across k1),
// Tm = 3 T0.  Every other facet k has exact m_k(q0) >= m4 - T0 and is
// 1-Lipschitz, so for |w - w0| < R = m4 - alpha_c - 8 T0 it stays above
// alpha_c + T(q) (T(q) <= Tm there, and the w rounding of both points adds at
// most T(q) + T0): for q in the Voronoi cell of c (all cached margins > Tm)
// the label follows from the three cached margins alone, by the facet-plane
// rule.
// A point across a cached facet goes to a full pass (the facet list of c does
// not bound the seeds beyond it), started in the cell across k1 when k1 is
// the facet crossed.
constexpr int FC_BYTES_PER_WALKER = 6 * 16;

// Writes the cache of the walker in thread `w` (this CTA) from a full pass;
// p1..p3 are the records of facets k1..k3.
MADI_DEV void fc_build(const TileShared& ts, int w, const FacetTop& t, int c, float L, const float4& p1,
                       const float4& p2, const float4& p3) {
    const float Tm = 3.0f * t.T;
    const float R = fminf(t.m4 - t.cc.w - 8.0f * t.T, L);
    float4* f = ts.fc + w;
    const int n = blockDim.x;
    f[0] = p1;
    f[n] = p2;
    f[2 * n] = p3;
    f[3 * n] = make_float4(t.wx, t.wy, t.wz, R > 0.f ? R * R * (1.0f - MADI_EPS19) : 0.f);
    f[4 * n] = make_float4(t.cc.x, t.cc.y, t.cc.z, t.cc.w + Tm);
    f[5 * n] = make_float4(t.cc.w - Tm, Tm, __int_as_float(c), __int_as_float(t.nb1));
}

// Order-preserving 32-bit key of a facet margin: the float's bits mapped to
// unsigned order, the low KEY_BITS replaced by the facet's slot.  Dropping
// those mantissa bits rounds the margin down (towards -inf) by at most
// 2^(KEY_BITS - 23) relative; key_floor() returns that lower bound.
constexpr int KEY_BITS = 6;                      // slots per cell <= 64
constexpr uint32_t KEY_SLOT = (1u << KEY_BITS) - 1u;

MADI_DEV uint32_t margin_key(float m, uint32_t slot) {
    const uint32_t b = __float_as_uint(m);
    const uint32_t u = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
    return (u & ~KEY_SLOT) | slot;
}

MADI_DEV float key_floor(uint32_t key) {
    const uint32_t u = key & ~KEY_SLOT;
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

MADI_DEV void cx(uint32_t& a, uint32_t& b) {
    const uint32_t lo = min(a, b), hi = max(a, b);
    a = lo; b = hi;
}

// ascending sort of four keys
MADI_DEV void sort4(uint32_t& a, uint32_t& b, uint32_t& c, uint32_t& d) {
    cx(a, b); cx(c, d); cx(a, c); cx(b, d); cx(b, c);
}

// the four smallest of two ascending quadruples, ascending, into (a0..a3)
MADI_DEV void merge4(uint32_t& a0, uint32_t& a1, uint32_t& a2, uint32_t& a3, uint32_t b0, uint32_t b1,
                     uint32_t b2, uint32_t b3) {
    a0 = min(a0, b3); a1 = min(a1, b2); a2 = min(a2, b1); a3 = min(a3, b0);   // bitonic
    cx(a0, a2); cx(a1, a3); cx(a0, a1); cx(a2, a3);
}

// Full facet passes for the lanes with `need`, warp-cooperatively: a group of
// FG lanes takes one walker, splits its cell's facet slots (FU loads per lane
// in flight, coalesced), keeps each lane's four smallest margin keys with
// sorting networks and merges the group's in log2(FG) butterfly rounds.  The
// three smallest keys name the cached facets, whose margins are recomputed
// exactly (the true smallest margin is among them unless four margins lie
// within 2^-17 relative of each other, which the widened band covers); the
// fourth key bounds every other facet from below.  The group decides by the
// facet-plane rule and its first lane writes the walker's label cache.  A walker
// whose point lies across a facet is queued again from the cell beyond the
// most violated facet (at most three moves).  Called by all 32 lanes; `start`
// is each walker's first cell.  Returns FACET_IN / FACET_OUT with cell_q
// set, or a negative code when the voxel-grid classifier has to decide.
constexpr int FG = 4;
constexpr int FU = 8;

template <bool PERIODIC>
MADI_DEV int coop_facets(const Geo& g, const TileShared& ts, bool need, float qx, float qy, float qz, int start,
                         int lane, int& cell_q) {
    const int gid = lane / FG, sub = lane % FG;
    const int warp0 = threadIdx.x & ~31;
    const int S = g.fstride;
    int my_cell = start, hops = 0, r_mine = FACET_BAND;
    bool pend = need;
    unsigned pending = __ballot_sync(MADI_FULL, pend);
    while (pending) {
        const unsigned src = __fns(pending, 0, gid + 1);      // walker of this group, ~0u if none
        const bool act = src < 32u;
        const int s = act ? (int)src : 0;
        const float sx = __shfl_sync(MADI_FULL, qx, s);
        const float sy = __shfl_sync(MADI_FULL, qy, s);
        const float sz = __shfl_sync(MADI_FULL, qz, s);
        const int sc = __shfl_sync(MADI_FULL, my_cell, s);
        const uint32_t base = (uint32_t)sc * (uint32_t)S;
        float4 cc = make_float4(0.f, 0.f, 0.f, 0.f);
        float wx = 0.f, wy = 0.f, wz = 0.f;
        uint32_t q0 = 0xffffffffu, q1 = 0xffffffffu, q2 = 0xffffffffu, q3 = 0xffffffffu;
        if (act) {
            // the cell record and the cell's slots depend only on sc: one round trip
            cc = g.ccen[sc];
            for (int k0 = sub; k0 < S; k0 += FG * FU) {
                float4 f[FU];
#pragma unroll
                for (int i = 0; i < FU; ++i) f[i] = g.fpl[base + k0 + FG * i];
                wx = sx - cc.x; wy = sy - cc.y; wz = sz - cc.z;
                if (PERIODIC) {
                    const float hl = 0.5f * g.L;
                    wx = wx > hl ? wx - g.L : (wx < -hl ? wx + g.L : wx);
                    wy = wy > hl ? wy - g.L : (wy < -hl ? wy + g.L : wy);
                    wz = wz > hl ? wz - g.L : (wz < -hl ? wz + g.L : wz);
                }
                uint32_t k[FU];
#pragma unroll
                for (int i = 0; i < FU; ++i) k[i] = margin_key(facet_m(f[i], wx, wy, wz), (uint32_t)(k0 + FG * i));
                sort4(k[0], k[1], k[2], k[3]);
                sort4(k[4], k[5], k[6], k[7]);
                merge4(k[0], k[1], k[2], k[3], k[4], k[5], k[6], k[7]);
                merge4(q0, q1, q2, q3, k[0], k[1], k[2], k[3]);
            }
        }
#pragma unroll
        for (int o = 1; o < FG; o <<= 1) {
            const uint32_t b0 = __shfl_xor_sync(MADI_FULL, q0, o);
            const uint32_t b1 = __shfl_xor_sync(MADI_FULL, q1, o);
            const uint32_t b2 = __shfl_xor_sync(MADI_FULL, q2, o);
            const uint32_t b3 = __shfl_xor_sync(MADI_FULL, q3, o);
            merge4(q0, q1, q2, q3, b0, b1, b2, b3);
        }
        int r = FACET_BAND, nb = -1;
        if (act) {
            FacetTop t;
            t.k1 = base + (q0 & KEY_SLOT);
            t.k2 = base + (q1 & KEY_SLOT);
            t.k3 = base + (q2 & KEY_SLOT);
            t.m4 = key_floor(q3);
            // the three candidates' records and neighbours, loaded together (L1)
            const float4 p1 = g.fpl[t.k1], p2 = g.fpl[t.k2], p3 = g.fpl[t.k3];
            const int n1 = g.fnbr[t.k1], n2 = g.fnbr[t.k2], n3 = g.fnbr[t.k3];
            const float e1 = facet_m(p1, wx, wy, wz);
            const float e2 = facet_m(p2, wx, wy, wz);
            const float e3 = facet_m(p3, wx, wy, wz);
            const float m1 = fminf(e1, fminf(e2, e3));
            t.m1 = m1;
            t.wx = wx; t.wy = wy; t.wz = wz; t.cc = cc;
            t.T = fmaf(2.0f * MADI_EPS21, fabsf(wx) + fabsf(wy) + fabsf(wz), g.ftol) + 7.62939453125e-6f * fabsf(m1);
            t.nb1 = e1 <= e2 ? (e1 <= e3 ? n1 : n3) : (e2 <= e3 ? n2 : n3);
            if (m1 > t.T) {
                const float dd = m1 - cc.w;
                r = dd > t.T ? FACET_IN : (dd < -t.T ? FACET_OUT : FACET_BAND);
            } else if (m1 < -t.T) {
                r = FACET_LEFT;
                nb = t.nb1;
            }
            if (sub == 0 && r >= 0) fc_build(ts, warp0 + s, t, sc, g.L, p1, p2, p3);
        }
        // each pending walker reads its group's verdict (group = its rank among the pending)
        const int rank = __popc(pending & ((1u << lane) - 1u));
        const bool mine = pend && rank < 32 / FG;
        const int leader = (mine ? rank : 0) * FG;
        const int rl = __shfl_sync(MADI_FULL, r, leader);
        const int nbl = __shfl_sync(MADI_FULL, nb, leader);
        if (mine) {
            if (rl == FACET_LEFT && nbl >= 0 && hops < 3) { my_cell = nbl; ++hops; }
            else { r_mine = rl; pend = false; }
        }
        pending = __ballot_sync(MADI_FULL, pend);
    }
    __syncwarp();
    cell_q = my_cell;
    return r_mine;
}

// Walk one tile (blockDim.x walkers of one job) on geometry view g.
template <int OUT, bool PERIODIC, int NP>
__device__ __forceinline__ void walk_tile(const madi_walk_desc& d, const madi_walk_job& job,
                                          const madi_geometry& gd, const Geo& g, int local, const TileShared& ts) {
    const int lane = threadIdx.x & 31;
    const bool active = local < job.n_walkers;
    const uint32_t widx = job.walker_base + (uint32_t)local;
    const float L = (float)gd.L;
    const float sigma = (float)d.sigma;
    const bool cells = gd.has_cells != 0;
    const bool stream = d.rng == MADI_RNG_STREAM;

    // ---- initial position (Omega_src cube; the whole box when periodic) ----
    float px = 0.f, py = 0.f, pz = 0.f;
    if (active) {
        double x0, y0, z0;
        if (stream) {
            x0 = d.init[3 * (size_t)local + 0];
            y0 = d.init[3 * (size_t)local + 1];
            z0 = d.init[3 * (size_t)local + 2];
        } else {
            const U4 r = philox10(U4{widx, 0u, 0u, 1u}, job.key0, job.key1);
            const double span = gd.source_hi - gd.source_lo;
            x0 = gd.source_lo + span * ((double)r.x * 2.3283064365386963e-10);
            y0 = gd.source_lo + span * ((double)r.y * 2.3283064365386963e-10);
            z0 = gd.source_lo + span * ((double)r.z * 2.3283064365386963e-10);
        }
        px = (float)x0; py = (float)y0; pz = (float)z0;
        if (PERIODIC) {
            if (px >= L) px = 0.f;
            if (py >= L) py = 0.f;
            if (pz >= L) pz = 0.f;
        }
    }
    const float x0f = px, y0f = py, z0f = pz;
    // ---- state ----
    float dx = 0.f, dy = 0.f, dz = 0.f;           // unwrapped displacement from x0
    int cell = 0, inside = 0;                     // Voronoi cell of the position and its label
    const bool facets = cells && g.n_cells > 0;
    bool dead = !active;
    bool frozen = !active;
    uint32_t n_full = 0, n_t1 = 0, n_fp = 0, escaped = 0, cerr = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) { AUX_Y(k) = 0.0; AUX_A(k) = 0.f; AUX_C(k) = 0u; }
#pragma unroll
    for (int p = 0; p < NP; ++p) { AUX_M(p, 0) = 0.f; AUX_M(p, 1) = 0.f; AUX_M(p, 2) = 0.f; }
    FC(0) = make_float4(0.f, 0.f, 0.f, 3.0e38f);  // empty label cache
    FC(3) = make_float4(0.f, 0.f, 0.f, 0.f);
    FC(4) = make_float4(0.f, 0.f, 0.f, 0.f);
    FC(5) = make_float4(0.f, 0.f, __int_as_float(-1), __int_as_float(-1));
    if (cells) {
        int my_st = CLS_OK, my_s1 = 0, my_in = 0;
        for (unsigned pend = __ballot_sync(MADI_FULL, active); pend; pend &= pend - 1) {
            const int src = __ffs(pend) - 1;
            const float sx = __shfl_sync(MADI_FULL, px, src);
            const float sy = __shfl_sync(MADI_FULL, py, src);
            const float sz = __shfl_sync(MADI_FULL, pz, src);
            int s1 = 0, in = 0;
            const int st = coop_classify(g, sx, sy, sz, -1, lane, s1, in);
            if (lane == src) { my_st = st; my_s1 = s1; my_in = in; }
        }
        __syncwarp();
        if (active) {
            if (my_st == CLS_FALLBACK) {
                my_st = classify_list_f64(g, px, py, pz, my_s1, my_in);
                ++AUX_C(0);
            }
            if (my_st != CLS_OK) { cerr = 1; dead = true; }
            else { cell = cell_of(g, my_s1); inside = my_in; }
            ++n_full;
        }
    }
    float Sx = 0.f, Sy = 0.f, Sz = 0.f;           // sum of displacements in this interval
    const size_t row = (size_t)job.y_row + (size_t)local;
    if (OUT == MADI_OUT_Y && active) {
        d.Y[(row * d.n_grid) * 3 + 0] = 0.0;
        d.Y[(row * d.n_grid) * 3 + 1] = 0.0;
        d.Y[(row * d.n_grid) * 3 + 2] = 0.0;
        d.inside_trace[row * d.n_grid] = (int8_t)inside;
    }
    {
        const unsigned b = __ballot_sync(0xffffffffu, active && inside);
        if (lane == 0 && b) atomicAdd(&ts.occ[0], (unsigned)__popc(b));
    }
    const bool always = job.pp >= 1.0;
    const uint32_t th1 = (uint32_t)(job.thr1 >> 32), th2 = (uint32_t)(job.thr2 >> 32);
    float g3 = 0.f, g4 = 0.f, g5 = 0.f;
    uint32_t acc_word_odd = 0;
    int h_left = d.steps_per_h;
    int jgrid = 0;
    for (int step = 0; step < d.n_steps; ++step) {
        // ---- random numbers: one Philox call per step on average ----
        float nx, ny, nz;
        uint32_t word = 0;
        double ustream = 0.0;
        if (stream) {
            if (!dead) {
                const size_t o = ((size_t)step * job.n_walkers + local);
                nx = (float)d.incr[3 * o + 0];
                ny = (float)d.incr[3 * o + 1];
                nz = (float)d.incr[3 * o + 2];
                ustream = d.unif[o];
            } else { nx = ny = nz = 0.f; }
        } else if ((step & 1) == 0) {
            const uint32_t pair = (uint32_t)step >> 1;
            const U4 ra = philox10(U4{widx, pair, 0u, 0u}, job.key0, job.key1);
            const U4 rb = philox10(U4{widx, pair, 1u, 0u}, job.key0, job.key1);
            float g0, g1, g2;
            box_muller(ra.x, ra.y, g0, g1);
            box_muller(ra.z, ra.w, g2, g3);
            box_muller(rb.x, rb.y, g4, g5);
            nx = g0 * sigma; ny = g1 * sigma; nz = g2 * sigma;
            word = rb.z;
            acc_word_odd = rb.w;
        } else {
            nx = g3 * sigma; ny = g4 * sigma; nz = g5 * sigma;
            word = acc_word_odd;
        }
        // ---- proposal and boundary ----
        float qx = px, qy = py, qz = pz;
        bool ok = false;
        if (!dead) {
            qx = px + nx; qy = py + ny; qz = pz + nz;
            ok = true;
            if (PERIODIC) {
                if (qx < 0.f) qx += L;
                if (qx >= L) qx -= L;
                if (qy < 0.f) qy += L;
                if (qy >= L) qy -= L;
                if (qz < 0.f) qz += L;
                if (qz >= L) qz -= L;
            } else if (qx < 0.f || qx >= L || qy < 0.f || qy >= L || qz < 0.f || qz >= L) {
                ok = false;
                escaped = 1;
                dead = true;
            }
        }
        const float ex = dx + nx, ey = dy + ny, ez = dz + nz;
        // ---- label from the facet planes of the current cell (and its neighbours) ----
        bool t1 = false;
        int t1_in = 0, t1_cell = cell;
        int start = cell;
        if (ok && facets) {
            // inside the cached sphere three planes decide
            const float4 sp = FC(3), ce = FC(4), f1 = FC(0), th = FC(5);
            float wx = qx - ce.x, wy = qy - ce.y, wz = qz - ce.z;
            if (PERIODIC) {
                const float hl = 0.5f * L;
                wx = wx > hl ? wx - L : (wx < -hl ? wx + L : wx);
                wy = wy > hl ? wy - L : (wy < -hl ? wy + L : wy);
                wz = wz > hl ? wz - L : (wz < -hl ? wz + L : wz);
            }
            const float m1 = facet_m(f1, wx, wy, wz);
            const float ux = wx - sp.x, uy = wy - sp.y, uz = wz - sp.z;
            if (fmaf(ux, ux, fmaf(uy, uy, uz * uz)) < sp.w) {
                const float4 f2 = FC(1), f3 = FC(2);
                const float mm = fminf(m1, fminf(facet_m(f2, wx, wy, wz), facet_m(f3, wx, wy, wz)));
                if (mm > ce.w) { t1 = true; t1_in = 1; t1_cell = __float_as_int(th.z); }
                else if (mm > th.y && mm < th.x) { t1 = true; t1_in = 0; t1_cell = __float_as_int(th.z); }
            }
            // across the cached cell's nearest facet (an exact plane of it): start
            // the full pass in the cell beyond
            const int nb1 = __float_as_int(th.w);
            if (!t1 && m1 < -th.y && nb1 >= 0) start = nb1;
        }
        // ---- cache misses: cooperative full facet passes, which rebuild the caches ----
        const bool miss = ok && facets && !t1;
        n_fp += miss ? 1u : 0u;
        if (__any_sync(MADI_FULL, miss)) {
            int cq = start;
            const int r = coop_facets<PERIODIC>(g, ts, miss, qx, qy, qz, start, lane, cq);
            if (miss && r >= 0) { t1 = true; t1_in = r; t1_cell = cq; }
        }
        // ---- full classifications of this step, one warp-cooperative pass each ----
        const bool need = ok && cells && !t1;
        int my_st = CLS_OK, my_s1 = 0, my_in = 0;
        for (unsigned pend = __ballot_sync(MADI_FULL, need); pend; pend &= pend - 1) {
            const int src = __ffs(pend) - 1;
            const float sx = __shfl_sync(MADI_FULL, qx, src);
            const float sy = __shfl_sync(MADI_FULL, qy, src);
            const float sz = __shfl_sync(MADI_FULL, qz, src);
            const int sg = __shfl_sync(MADI_FULL, cell, src);
            int s1 = 0, in = 0;
            const int st = coop_classify(g, sx, sy, sz, sg, lane, s1, in);
            if (lane == src) { my_st = st; my_s1 = s1; my_in = in; }
        }
        __syncwarp();
        if (ok) {
            int ncell = 0, nin = 0;
            if (t1) {
                ncell = t1_cell; nin = t1_in; ++n_t1;
            } else if (need) {
                if (my_st == CLS_FALLBACK) {
                    my_st = classify_list_f64(g, qx, qy, qz, my_s1, my_in);
                    ++AUX_C(0);
                }
                ++n_full;
                if (my_st != CLS_OK) { cerr = 1; dead = true; }
                else { ncell = cell_of(g, my_s1); nin = my_in; }
            }
            if (!dead) {
                int m = 0;
                if (inside != nin) m = 1;
                else if (inside && nin && cell != ncell) m = 2;
                bool accept = true;
                if (m > 0 && !always) {
                    if (stream) {
                        accept = ustream < (m == 1 ? job.pp : job.pp * job.pp);
                    } else {
                        const uint32_t th = m == 1 ? th1 : th2;
                        if (word != th) {
                            accept = word < th;
                        } else {
                            const uint64_t thr = m == 1 ? job.thr1 : job.thr2;
                            const U4 rc = philox10(U4{widx, (uint32_t)step, 2u, 0u}, job.key0, job.key1);
                            accept = rc.x < (uint32_t)thr;
                        }
                    }
                    ++AUX_C(accept ? 1 : 2);
                }
                if (accept) {
                    px = qx; py = qy; pz = qz;
                    dx = ex; dy = ey; dz = ez;
                    cell = ncell; inside = nin;
                }
            }
        }
        if (!dead) {
            Sx += dx; Sy += dy; Sz += dz;
        } else if (!frozen) {
            // Walker stopped (fatal escape or classifier failure): close its
            // trapezoid at the last accepted step and add nothing after.
            frozen = true;
            AUX_Y(0) += d.ts * ((double)Sx + 0.5 * ((double)AUX_A(0) - (double)dx));
            AUX_Y(1) += d.ts * ((double)Sy + 0.5 * ((double)AUX_A(1) - (double)dy));
            AUX_Y(2) += d.ts * ((double)Sz + 0.5 * ((double)AUX_A(2) - (double)dz));
            Sx = Sy = Sz = 0.f;
            AUX_A(0) = dx; AUX_A(1) = dy; AUX_A(2) = dz;
        }
        if (--h_left == 0) {
            h_left = d.steps_per_h;
            ++jgrid;
            const double tsd = d.ts;
            const double Yx = AUX_Y(0) + tsd * ((double)Sx + 0.5 * ((double)AUX_A(0) - (double)dx));
            const double Yy = AUX_Y(1) + tsd * ((double)Sy + 0.5 * ((double)AUX_A(1) - (double)dy));
            const double Yz = AUX_Y(2) + tsd * ((double)Sz + 0.5 * ((double)AUX_A(2) - (double)dz));
            AUX_Y(0) = Yx; AUX_Y(1) = Yy; AUX_Y(2) = Yz;
            Sx = Sy = Sz = 0.f;
            AUX_A(0) = dx; AUX_A(1) = dy; AUX_A(2) = dz;
            if (OUT == MADI_OUT_Y) {
                if (active) {
                    const double t = (double)jgrid * d.steps_per_h * tsd;
                    const double half_L = 0.5 * gd.L;
                    double* yo = d.Y + (row * d.n_grid + jgrid) * 3;
                    yo[0] = y_ref(Yx, x0f, half_L, t);
                    yo[1] = y_ref(Yy, y0f, half_L, t);
                    yo[2] = y_ref(Yz, z0f, half_L, t);
                    d.inside_trace[row * d.n_grid + jgrid] = (int8_t)inside;
                }
            } else {
                const Snap sn = ts.snap[jgrid];
                if (sn.any) {
                    const float fx = (float)Yx, fy = (float)Yy, fz = (float)Yz;
#pragma unroll
                    for (int p = 0; p < NP; ++p) {
                        const float k = snap_coef(sn.code, p);
                        if (k != 0.f) {
                            AUX_M(p, 0) = fmaf(k, fx, AUX_M(p, 0));
                            AUX_M(p, 1) = fmaf(k, fy, AUX_M(p, 1));
                            AUX_M(p, 2) = fmaf(k, fz, AUX_M(p, 2));
                        }
                    }
                }
            }
            const unsigned b = __ballot_sync(0xffffffffu, active && inside);
            if (lane == 0 && b) atomicAdd(&ts.occ[jgrid], (unsigned)__popc(b));
        }
    }
    // ---- phase epilogue: per (pair, dir, b) warp sums -> fixed point ----
    if (OUT == MADI_OUT_FUSED) {
        const bool live = active && !escaped && !cerr;
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            if (p >= d.n_pairs) break;
            const float mx = AUX_M(p, 0), my = AUX_M(p, 1), mz = AUX_M(p, 2);
            for (int u = 0; u < d.n_dirs; ++u) {
                const float proj = fmaf(d.dirs[3 * u], mx, fmaf(d.dirs[3 * u + 1], my, d.dirs[3 * u + 2] * mz));
                for (int bb = 0; bb < d.n_b; ++bb) {
                    float c = 0.f, s = 0.f;
                    if (live) sincosf(d.coef[p * d.n_b + bb] * proj, &s, &c);
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        c += __shfl_xor_sync(0xffffffffu, c, o);
                        s += __shfl_xor_sync(0xffffffffu, s, o);
                    }
                    if (lane == 0) {
                        const int idx = ((p * d.n_b + bb) * d.n_dirs + u) * 2;
                        atomicAdd(reinterpret_cast<unsigned long long*>(&ts.acc[idx]),
                                  (unsigned long long)__float2ll_rn(c * 4294967296.0f));
                        atomicAdd(reinterpret_cast<unsigned long long*>(&ts.acc[idx + 1]),
                                  (unsigned long long)__float2ll_rn(s * 4294967296.0f));
                    }
                }
            }
        }
    }
    // ---- counters ----
    {
        uint64_t* cnt = d.counters + (size_t)job.slot * MADI_CNT_N;
        const uint32_t v0 = __reduce_add_sync(0xffffffffu, active ? 1u : 0u);
        const uint32_t v1 = __reduce_add_sync(0xffffffffu, escaped);
        const uint32_t v2 = __reduce_add_sync(0xffffffffu, cerr);
        const uint32_t v3 = __reduce_add_sync(0xffffffffu, n_full);
        const uint32_t v4 = __reduce_add_sync(0xffffffffu, n_t1);
        const uint32_t v5 = __reduce_add_sync(0xffffffffu, AUX_C(0));
        const uint32_t v6 = __reduce_add_sync(0xffffffffu, AUX_C(1));
        const uint32_t v7 = __reduce_add_sync(0xffffffffu, AUX_C(2));
        const uint32_t v8 = __reduce_add_sync(0xffffffffu, n_fp);
        if (lane == 0) {
            unsigned long long* c = reinterpret_cast<unsigned long long*>(cnt);
            if (v0) atomicAdd(&c[0], (unsigned long long)v0);
            if (v1) atomicAdd(&c[1], (unsigned long long)v1);
            if (v2) atomicAdd(&c[2], (unsigned long long)v2);
            if (v3) atomicAdd(&c[3], (unsigned long long)v3);
            if (v4) atomicAdd(&c[4], (unsigned long long)v4);
            if (v5) atomicAdd(&c[5], (unsigned long long)v5);
            if (v6) atomicAdd(&c[6], (unsigned long long)v6);
            if (v7) atomicAdd(&c[7], (unsigned long long)v7);
            if (v8) atomicAdd(&c[MADI_CNT_FACET_PASS], (unsigned long long)v8);
        }
    }
}

template <int OUT, bool PERIODIC, int NP, int MINB>
__global__ void __launch_bounds__(256, MINB) walk_f32_kernel(const madi_walk_desc d) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_item;
    const int nthr = blockDim.x;
    const int tid = threadIdx.x;
    const int n_out = d.n_pairs * d.n_b * d.n_dirs;
    // Dynamic shared memory: [stage][acc int64 x 2 n_out][occ u32 x n_grid][snap x n_grid]
    unsigned char* stage = smem;
    TileShared ts;
    ts.acc = reinterpret_cast<long long*>(smem + d.stage_smem);
    ts.occ = reinterpret_cast<unsigned int*>(ts.acc + 2 * n_out);
    Snap* snap = reinterpret_cast<Snap*>(ts.occ + d.n_grid);
    ts.snap = snap;
    unsigned char* aux = smem + d.stage_smem + 16 * n_out + 12 * ((d.n_grid + 3) & ~3);
    ts.auxd = reinterpret_cast<double*>(aux);
    ts.fc = reinterpret_cast<float4*>(aux + 24 * nthr);
    ts.auxf = reinterpret_cast<float*>(aux + (24 + FC_BYTES_PER_WALKER) * nthr);
    ts.auxc = reinterpret_cast<uint32_t*>(ts.auxf + (3 + 3 * NP) * nthr);

    for (int j = tid; j < d.n_grid; j += nthr) {
        uint32_t code = 0, any = 0;
        for (int p = 0; p < MADI_MAX_PAIRS; ++p) {
            int k = 0;
            if (p < d.n_pairs) k = (d.pair_jd[p] == j) + (d.pair_jD[p] == j) - (d.pair_js[p] == j);
            code |= (uint32_t)(k + 1) << (2 * p);
            any |= k != 0;
        }
        snap[j] = Snap{code, any};
    }
    int cur_geom = -1;
    int first = 1;
    for (;;) {
        __syncthreads();
        if (tid == 0) {
            if (d.grid_blocks > 0) s_item = (int)atomicAdd(d.work_counter, 1u);
            else s_item = first ? (int)blockIdx.x : d.n_tiles;
        }
        first = 0;
        for (int i = tid; i < 2 * n_out; i += nthr) ts.acc[i] = 0;
        for (int j = tid; j < d.n_grid; j += nthr) ts.occ[j] = 0;
        __syncthreads();
        const int item = s_item;
        if (item >= d.n_tiles) break;
        const int jn = find_job(d.jobs, d.n_jobs, item);
        const madi_walk_job job = d.jobs[jn];
        const madi_geometry gd = d.geoms[job.geom];
        const int local = (item - job.tile_begin) * nthr + tid;
        const bool here = d.stage_smem > 0 && (int)gd.stage_bytes <= d.stage_smem;
        if (here) {
            if (job.geom != cur_geom) {
                const uint4* src = reinterpret_cast<const uint4*>(gd.stage);
                uint4* dst = reinterpret_cast<uint4*>(stage);
                for (uint32_t i = tid; i < gd.stage_bytes / 16u; i += nthr) dst[i] = src[i];
                cur_geom = job.geom;
                __syncthreads();
            }
            walk_tile<OUT, PERIODIC, NP>(d, job, gd, make_geo(gd, stage), local, ts);
        } else {
            walk_tile<OUT, PERIODIC, NP>(d, job, gd, make_geo(gd, reinterpret_cast<const unsigned char*>(gd.stage)),
                                         local, ts);
        }
        __syncthreads();
        if (OUT == MADI_OUT_FUSED) {
            long long* out = reinterpret_cast<long long*>(d.accum) + (size_t)job.slot * 2 * n_out;
            for (int i = tid; i < 2 * n_out; i += nthr)
                if (ts.acc[i]) atomicAdd(reinterpret_cast<unsigned long long*>(&out[i]), (unsigned long long)ts.acc[i]);
        }
        uint64_t* occ_out = d.occupancy + (size_t)job.slot * d.n_grid;
        for (int j = tid; j < d.n_grid; j += nthr)
            if (ts.occ[j]) atomicAdd(reinterpret_cast<unsigned long long*>(&occ_out[j]), (unsigned long long)ts.occ[j]);
    }
}

// ---------------------------------------------------------------------------
// fp64 walker (madi/walker_gpu.py:520-585 design and :698-840 arithmetic:
// separately rounded fp64, reference origin L/2, exact KD rule at every step,
// Y stored).  One thread per walker of jobs[0]; it replays a fixed random
// stream (golden check) or walks the fp32 walker's Philox numbers.
// ---------------------------------------------------------------------------
// Normals of step `step` of walker widx from the Philox stream of the fp32
// walker, in fp64 (Box-Muller: u1 = (w + 1/2) 2^-32, u2 = (w' >> 8) 2^-24), and
// the step's acceptance word: the fp32 walker's random numbers, evaluated in
// the reference's precision.
MADI_DEV void normals_f64(uint32_t widx, int step, uint32_t k0, uint32_t k1, double (&n)[3], uint32_t& word) {
    const uint32_t pair = (uint32_t)step >> 1;
    const U4 ra = philox10(U4{widx, pair, 0u, 0u}, k0, k1);
    const U4 rb = philox10(U4{widx, pair, 1u, 0u}, k0, k1);
    const uint32_t wd[6] = {ra.x, ra.y, ra.z, ra.w, rb.x, rb.y};
    double gv[6];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double u1 = __dadd_rn(__dmul_rn((double)wd[2 * k], 2.3283064365386963e-10), 1.1641532182693481e-10);
        const double u2 = __dmul_rn((double)(wd[2 * k + 1] >> 8), 5.9604644775390625e-08);
        const double r = sqrt(__dmul_rn(-2.0, log(u1)));
        double sn, cs;
        sincos(__dmul_rn(6.283185307179586, u2), &sn, &cs);
        gv[2 * k] = __dmul_rn(r, cs);
        gv[2 * k + 1] = __dmul_rn(r, sn);
    }
    const bool odd = (step & 1) != 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) n[k] = odd ? gv[3 + k] : gv[k];
    word = (step & 1) ? rb.w : rb.z;
}

__global__ void __launch_bounds__(128) walk_f64_kernel(const madi_walk_desc d) {
    const madi_walk_job job = d.jobs[0];
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= job.n_walkers) return;
    const madi_geometry gd = d.geoms[job.geom];
    const Geo g = make_geo(gd, reinterpret_cast<const unsigned char*>(gd.stage));
    const bool periodic = gd.boundary == MADI_BOUNDARY_PERIODIC;
    const bool cells = gd.has_cells != 0;
    const bool stream = d.rng == MADI_RNG_STREAM;
    const uint32_t widx = job.walker_base + (uint32_t)w;
    const double L = gd.L, half_L = gd.L / 2.0, ts = d.ts, pp = job.pp;
    const size_t row = (size_t)job.y_row + w;
    double px, py, pz;
    if (stream) {
        px = d.init[3 * (size_t)w]; py = d.init[3 * (size_t)w + 1]; pz = d.init[3 * (size_t)w + 2];
    } else {
        const U4 r = philox10(U4{widx, 0u, 0u, 1u}, job.key0, job.key1);
        const double span = gd.source_hi - gd.source_lo;
        px = gd.source_lo + span * ((double)r.x * 2.3283064365386963e-10);
        py = gd.source_lo + span * ((double)r.y * 2.3283064365386963e-10);
        pz = gd.source_lo + span * ((double)r.z * 2.3283064365386963e-10);
        if (periodic) {
            if (px >= L) px = 0.0;
            if (py >= L) py = 0.0;
            if (pz >= L) pz = 0.0;
        }
    }
    int cell = 0, inside = 0, escaped = 0, cerr = 0;
    uint32_t n_acc = 0, n_rej = 0, n_full = 0;
    if (cells) {
        int s1 = 0;
        if (classify_kd_f64(g, px, py, pz, s1, inside) != CLS_OK) cerr = 1;
        cell = g.cell[s1];
        ++n_full;
    }
    int kx = 0, ky = 0, kz = 0;
    double xp = __dsub_rn(px, half_L), yp = __dsub_rn(py, half_L), zp = __dsub_rn(pz, half_L);
    double Yx = 0.0, Yy = 0.0, Yz = 0.0;
    double* Yo = d.Y + row * d.n_grid * 3;
    int8_t* It = d.inside_trace + row * d.n_grid;
    Yo[0] = Yo[1] = Yo[2] = 0.0;
    It[0] = (int8_t)inside;
    for (int step = 0; step < d.n_steps; ++step) {
        if (!escaped && !cerr) {
            double inc[3], u = 0.0;
            uint32_t word = 0;
            if (stream) {
                const size_t o = (size_t)step * job.n_walkers + w;
                inc[0] = d.incr[3 * o]; inc[1] = d.incr[3 * o + 1]; inc[2] = d.incr[3 * o + 2];
                u = d.unif[o];
            } else {
                normals_f64(widx, step, job.key0, job.key1, inc, word);
                inc[0] = __dmul_rn(inc[0], d.sigma); inc[1] = __dmul_rn(inc[1], d.sigma); inc[2] = __dmul_rn(inc[2], d.sigma);
            }
            double qx = __dadd_rn(px, inc[0]), qy = __dadd_rn(py, inc[1]), qz = __dadd_rn(pz, inc[2]);
            int qkx = kx, qky = ky, qkz = kz;
            bool ok = true;
            if (periodic) {
                if (qx < 0.0) { qx = __dadd_rn(qx, L); --qkx; }
                if (qx >= L) { qx = __dsub_rn(qx, L); ++qkx; }
                if (qy < 0.0) { qy = __dadd_rn(qy, L); --qky; }
                if (qy >= L) { qy = __dsub_rn(qy, L); ++qky; }
                if (qz < 0.0) { qz = __dadd_rn(qz, L); --qkz; }
                if (qz >= L) { qz = __dsub_rn(qz, L); ++qkz; }
            } else if (qx < 0.0 || qx >= L || qy < 0.0 || qy >= L || qz < 0.0 || qz >= L) {
                escaped = 1;
                ok = false;
            }
            if (ok) {
                int ncell = 0, nin = 0;
                if (cells) {
                    int s1 = 0;
                    if (classify_kd_f64(g, qx, qy, qz, s1, nin) != CLS_OK) { cerr = 1; }
                    ncell = g.cell[s1];
                    ++n_full;
                }
                if (!cerr) {
                    int m = 0;
                    if (inside && !nin) m = 1;
                    else if (!inside && nin) m = 1;
                    else if (inside && nin && cell != ncell) m = 2;
                    bool accept = true;
                    if (m > 0 && pp < 1.0) {
                        if (stream) {
                            const double thr = m == 1 ? pp : __dmul_rn(pp, pp);
                            accept = !(u >= thr);
                        } else {            // 64-bit uniform against floor(pp^m 2^64), as the fp32 walker
                            const uint64_t thr = m == 1 ? job.thr1 : job.thr2;
                            const uint32_t th = (uint32_t)(thr >> 32);
                            if (word != th) {
                                accept = word < th;
                            } else {
                                const U4 rc = philox10(U4{widx, (uint32_t)step, 2u, 0u}, job.key0, job.key1);
                                accept = rc.x < (uint32_t)thr;
                            }
                        }
                        if (accept) ++n_acc; else ++n_rej;
                    }
                    if (accept) {
                        px = qx; py = qy; pz = qz; kx = qkx; ky = qky; kz = qkz;
                        cell = ncell; inside = nin;
                    }
                    double xn = __dsub_rn(px, half_L), yn = __dsub_rn(py, half_L), zn = __dsub_rn(pz, half_L);
                    if (periodic) {
                        xn = __dadd_rn(xn, __dmul_rn((double)kx, L));
                        yn = __dadd_rn(yn, __dmul_rn((double)ky, L));
                        zn = __dadd_rn(zn, __dmul_rn((double)kz, L));
                    }
                    Yx = __dadd_rn(Yx, __dmul_rn(__dmul_rn(0.5, __dadd_rn(xp, xn)), ts));
                    Yy = __dadd_rn(Yy, __dmul_rn(__dmul_rn(0.5, __dadd_rn(yp, yn)), ts));
                    Yz = __dadd_rn(Yz, __dmul_rn(__dmul_rn(0.5, __dadd_rn(zp, zn)), ts));
                    xp = xn; yp = yn; zp = zn;
                }
            }
        }
        const int si = step + 1;
        if (si % d.steps_per_h == 0) {
            const int j = si / d.steps_per_h;
            Yo[3 * j] = Yx; Yo[3 * j + 1] = Yy; Yo[3 * j + 2] = Yz;
            It[j] = (int8_t)inside;
            if (inside) atomicAdd(reinterpret_cast<unsigned long long*>(&d.occupancy[(size_t)job.slot * d.n_grid + j]), 1ull);
        }
    }
    uint64_t* cnt = d.counters + (size_t)job.slot * MADI_CNT_N;
    atomicAdd(reinterpret_cast<unsigned long long*>(&cnt[MADI_CNT_WALKERS]), 1ull);
    if (escaped) atomicAdd(reinterpret_cast<unsigned long long*>(&cnt[MADI_CNT_ESCAPED]), 1ull);
    if (cerr) atomicAdd(reinterpret_cast<unsigned long long*>(&cnt[MADI_CNT_CLASSIFIER_ERROR]), 1ull);
    atomicAdd(reinterpret_cast<unsigned long long*>(&cnt[MADI_CNT_FULL]), (unsigned long long)n_full);
    atomicAdd(reinterpret_cast<unsigned long long*>(&cnt[MADI_CNT_CROSS_ACCEPT]), (unsigned long long)n_acc);
    atomicAdd(reinterpret_cast<unsigned long long*>(&cnt[MADI_CNT_CROSS_REJECT]), (unsigned long long)n_rej);
    const int8_t i0 = It[0];
    if (i0) atomicAdd(reinterpret_cast<unsigned long long*>(&d.occupancy[(size_t)job.slot * d.n_grid]), 1ull);
}

// ---------------------------------------------------------------------------
// Column reduction from stored Y (replaces _reduce_kernel, madi/walker_gpu.py:
// 658-695, which re-reads Y once per column).  A CTA takes a block of
// REDUCE_THREADS * REDUCE_CPT columns and a range of walkers: walker rows are
// staged in shared memory a few at a time and every thread adds, for its
// columns, cos / sin(coef * dM) over the 3 axes with dM = Y[jd] + Y[jD] - Y[js]
// (the reference's operation order) into fp64 partial sums in a fixed order.
// Each (CTA, column) partial is then rounded once to 2^-32 fixed point and
// added to an int64 accumulator: integer addition is order independent, so the
// sums do not depend on how the grid was scheduled.  Y is read from HBM/L2
// ceil(n_cols / (REDUCE_THREADS * REDUCE_CPT)) times instead of n_cols times.
// ---------------------------------------------------------------------------
constexpr int REDUCE_THREADS = 256;
constexpr int REDUCE_CPT = 4;                                // columns per thread
constexpr int REDUCE_COLS = REDUCE_THREADS * REDUCE_CPT;     // columns per CTA

__global__ void __launch_bounds__(REDUCE_THREADS) reduce_Y_kernel(const double* __restrict__ Y, int64_t n_walkers,
                                                                  int n_grid, int wt, int64_t per_block,
                                                                  const int32_t* __restrict__ jd,
                                                                  const int32_t* __restrict__ jD,
                                                                  const int32_t* __restrict__ js,
                                                                  const double* __restrict__ coef, int n_cols,
                                                                  unsigned long long* accum) {
    extern __shared__ double sy[];                            // [wt][n_grid * 3]
    const int row_len = n_grid * 3;
    int a[REDUCE_CPT], b[REDUCE_CPT], c[REDUCE_CPT];
    double pc[REDUCE_CPT], cs[REDUCE_CPT], sn[REDUCE_CPT];
#pragma unroll
    for (int k = 0; k < REDUCE_CPT; ++k) {
        const int col = blockIdx.x * REDUCE_COLS + k * REDUCE_THREADS + threadIdx.x;
        const bool live = col < n_cols;
        a[k] = live ? 3 * jd[col] : 0;
        b[k] = live ? 3 * jD[col] : 0;
        c[k] = live ? 3 * js[col] : 0;
        pc[k] = live ? coef[col] : 0.0;
        cs[k] = 0.0;
        sn[k] = 0.0;
    }
    const int64_t w0 = (int64_t)blockIdx.y * per_block;
    const int64_t w1 = min(n_walkers, w0 + per_block);
    for (int64_t wb = w0; wb < w1; wb += wt) {
        const int nw = (int)min((int64_t)wt, w1 - wb);
        __syncthreads();
        const double* src = Y + (size_t)wb * row_len;
        for (int i = threadIdx.x; i < nw * row_len; i += REDUCE_THREADS) sy[i] = src[i];
        __syncthreads();
        for (int w = 0; w < nw; ++w) {
            const double* y = sy + w * row_len;
#pragma unroll
            for (int k = 0; k < REDUCE_CPT; ++k) {
#pragma unroll
                for (int ax = 0; ax < 3; ++ax) {
                    const double dm = __dsub_rn(__dadd_rn(y[a[k] + ax], y[b[k] + ax]), y[c[k] + ax]);
                    double s, co;
                    sincos(__dmul_rn(pc[k], dm), &s, &co);
                    cs[k] += co;
                    sn[k] += s;
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < REDUCE_CPT; ++k) {
        const int col = blockIdx.x * REDUCE_COLS + k * REDUCE_THREADS + threadIdx.x;
        if (col < n_cols && w1 > w0) {
            atomicAdd(&accum[col], (unsigned long long)__double2ll_rn(cs[k] * 4294967296.0));
            atomicAdd(&accum[n_cols + col], (unsigned long long)__double2ll_rn(sn[k] * 4294967296.0));
        }
    }
}

__global__ void reduce_Y_finish_kernel(const long long* accum, int n_cols, double* cos_sum, double* sin_sum) {
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= n_cols) return;
    cos_sum[col] = (double)accum[col] * 0x1p-32;
    sin_sum[col] = (double)accum[n_cols + col] * 0x1p-32;
}

}  // namespace madi

using namespace madi;

extern "C" int64_t madi_walk_smem_bytes(int32_t stage_bytes, int32_t tile_walkers, int32_t n_grid) {
    // the fused layout of fused_smem() at the largest output shape (8 pairs)
    const int64_t n_out = (int64_t)MADI_MAX_PAIRS * MADI_MAX_B * MADI_MAX_DIRS;
    return (int64_t)((stage_bytes + 15) & ~15) + 16ll * n_out + 12ll * ((n_grid + 3) & ~3) +
           (24ll + FC_BYTES_PER_WALKER + 4 * (3 + 3 * MADI_MAX_PAIRS) + 12) * tile_walkers;
}

static int64_t fused_smem(const madi_walk_desc* d, int np) {
    const int64_t n_out = (int64_t)d->n_pairs * d->n_b * d->n_dirs;
    return (int64_t)d->stage_smem + 16ll * n_out + 12ll * ((d->n_grid + 3) & ~3) +
           (24 + FC_BYTES_PER_WALKER + 4 * (3 + 3 * np) + 12) * d->tile_walkers;
}

template <int OUT, bool PER, int NP, int MINB>
static madi_status launch_f32(const madi_walk_desc* d, cudaStream_t s) {
    auto k = walk_f32_kernel<OUT, PER, NP, MINB>;
    const int64_t sm = fused_smem(d, NP);
    if (sm > 227 * 1024) return host::fail(MADI_ERR_CAPACITY, "walker shared memory %lld B exceeds 227 KB", (long long)sm);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return host::cuda_fail(e, "cudaFuncSetAttribute(walker)");
    const int blocks = d->grid_blocks > 0 ? d->grid_blocks : d->n_tiles;
    k<<<blocks, d->tile_walkers, (size_t)sm, s>>>(*d);
    e = cudaGetLastError();
    if (e != cudaSuccess) return host::cuda_fail(e, "walker launch");
    return MADI_OK;
}

template <int OUT, bool PER>
static madi_status launch_np(const madi_walk_desc* d, cudaStream_t s) {
    const bool two = d->min_blocks >= 2;
    if (OUT == MADI_OUT_FUSED && d->n_pairs > 4)
        return two ? launch_f32<OUT, PER, 8, 2>(d, s) : launch_f32<OUT, PER, 8, 1>(d, s);
    return two ? launch_f32<OUT, PER, 4, 2>(d, s) : launch_f32<OUT, PER, 4, 1>(d, s);
}

template <int OUT, bool PER>
static const void* kernel_for(const madi_walk_desc* d) {
    const bool two = d->min_blocks >= 2;
    if (OUT == MADI_OUT_FUSED && d->n_pairs > 4)
        return two ? (const void*)walk_f32_kernel<OUT, PER, 8, 2> : (const void*)walk_f32_kernel<OUT, PER, 8, 1>;
    return two ? (const void*)walk_f32_kernel<OUT, PER, 4, 2> : (const void*)walk_f32_kernel<OUT, PER, 4, 1>;
}

extern "C" int32_t madi_walk_blocks_per_sm(const madi_walk_desc* d) {
    if (!d || d->tile_walkers <= 0) return 0;
    const bool per = d->boundary == MADI_BOUNDARY_PERIODIC;
    const void* k = d->out_mode == MADI_OUT_FUSED
        ? (per ? kernel_for<MADI_OUT_FUSED, true>(d) : kernel_for<MADI_OUT_FUSED, false>(d))
        : (per ? kernel_for<MADI_OUT_Y, true>(d) : kernel_for<MADI_OUT_Y, false>(d));
    const bool big = d->out_mode == MADI_OUT_FUSED && d->n_pairs > 4;
    const int64_t sm = fused_smem(d, big ? 8 : 4);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess) return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, d->tile_walkers, (size_t)sm) != cudaSuccess) return 0;
    return n;
}

extern "C" madi_status madi_walk(const madi_walk_desc* d, void* stream) {
    host::clear_error();
    if (!d) return host::fail(MADI_ERR_INVALID, "null walk descriptor");
    if (d->n_jobs <= 0 || d->n_geoms <= 0 || !d->jobs || !d->geoms)
        return host::fail(MADI_ERR_INVALID, "walk needs at least one job and one geometry");
    if (d->n_steps < 0 || d->steps_per_h <= 0 || d->n_grid <= 0 || d->n_grid > MADI_MAX_GRID)
        return host::fail(MADI_ERR_INVALID, "bad step grid (n_steps=%d steps_per_h=%d n_grid=%d)",
                          d->n_steps, d->steps_per_h, d->n_grid);
    if (d->n_steps / d->steps_per_h + 1 > d->n_grid)
        return host::fail(MADI_ERR_INVALID, "n_grid too small for n_steps / steps_per_h");
    if (!d->counters || !d->occupancy) return host::fail(MADI_ERR_INVALID, "counters and occupancy are required");
    if (d->rng == MADI_RNG_STREAM && (!d->init || !d->incr || !d->unif))
        return host::fail(MADI_ERR_INVALID, "stream replay needs init / incr / unif");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (d->precision == 64) {
        if (d->n_jobs != 1) return host::fail(MADI_ERR_UNSUPPORTED, "fp64 walker walks one job");
        if (!d->Y || !d->inside_trace) return host::fail(MADI_ERR_INVALID, "fp64 walker writes Y and inside_trace");
        // The job is read on the device; the host only needs its walker count, passed as n_tiles * 128 bound.
        const int blocks = d->n_tiles;
        walk_f64_kernel<<<blocks, 128, 0, s>>>(*d);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return host::cuda_fail(e, "fp64 walker launch");
        return MADI_OK;
    }
    if (d->precision != 32) return host::fail(MADI_ERR_INVALID, "precision must be 32 or 64");
    if (d->tile_walkers <= 0 || d->tile_walkers > 256 || (d->tile_walkers & 31))
        return host::fail(MADI_ERR_INVALID, "tile_walkers must be a multiple of 32 in [32, 256]");
    if (d->grid_blocks > 0 && !d->work_counter) return host::fail(MADI_ERR_INVALID, "persistent launch needs a zeroed work counter");
    if (d->out_mode == MADI_OUT_FUSED) {
        if (d->n_pairs < 1 || d->n_pairs > MADI_MAX_PAIRS || d->n_b < 1 || d->n_b > MADI_MAX_B ||
            d->n_dirs < 1 || d->n_dirs > MADI_MAX_DIRS)
            return host::fail(MADI_ERR_UNSUPPORTED, "fused epilogue holds <= %d pairs, <= %d b, <= %d dirs",
                              MADI_MAX_PAIRS, MADI_MAX_B, MADI_MAX_DIRS);
        if ((int64_t)d->n_pairs * d->n_b * d->n_dirs > 2048)
            return host::fail(MADI_ERR_UNSUPPORTED, "fused epilogue holds <= 2048 (column, direction) outputs");
        if (!d->accum) return host::fail(MADI_ERR_INVALID, "fused output needs accum");
        for (int p = 0; p < d->n_pairs; ++p)
            if (d->pair_jd[p] < 0 || d->pair_jD[p] < 0 || d->pair_js[p] < 0 || d->pair_jd[p] >= d->n_grid ||
                d->pair_jD[p] >= d->n_grid || d->pair_js[p] >= d->n_grid)
                return host::fail(MADI_ERR_INVALID, "pair grid index out of range");
    } else if (d->out_mode == MADI_OUT_Y) {
        if (!d->Y || !d->inside_trace) return host::fail(MADI_ERR_INVALID, "Y output needs Y and inside_trace");
    } else {
        return host::fail(MADI_ERR_INVALID, "unknown out_mode");
    }
    if (d->stage_smem < 0 || (d->stage_smem & 15)) return host::fail(MADI_ERR_INVALID, "stage_smem must be a multiple of 16");
    const bool per = d->boundary == MADI_BOUNDARY_PERIODIC;
    if (d->out_mode == MADI_OUT_FUSED)
        return per ? launch_np<MADI_OUT_FUSED, true>(d, s) : launch_np<MADI_OUT_FUSED, false>(d, s);
    return per ? launch_np<MADI_OUT_Y, true>(d, s) : launch_np<MADI_OUT_Y, false>(d, s);
}

extern "C" int64_t madi_reduce_Y_scratch_bytes(int32_t n_cols) {
    return n_cols > 0 ? 16ll * n_cols : 0;
}

extern "C" madi_status madi_reduce_Y(const double* Y, int64_t n_walkers, int32_t n_grid, const int32_t* jd,
                                     const int32_t* jD, const int32_t* js, const double* coef, int32_t n_cols,
                                     double* cos_sum, double* sin_sum, void* scratch, int64_t scratch_bytes,
                                     void* stream) {
    host::clear_error();
    if (!Y || !jd || !jD || !js || !coef || !cos_sum || !sin_sum || n_walkers < 0 || n_grid <= 0 ||
        n_grid > MADI_MAX_GRID || n_cols < 0)
        return host::fail(MADI_ERR_INVALID, "bad reduce_Y arguments");
    if (n_cols == 0) return MADI_OK;
    if (!scratch || scratch_bytes < madi_reduce_Y_scratch_bytes(n_cols))
        return host::fail(MADI_ERR_CAPACITY, "reduce_Y: scratch %lld < %lld bytes", (long long)scratch_bytes,
                          (long long)madi_reduce_Y_scratch_bytes(n_cols));
    if ((reinterpret_cast<uintptr_t>(scratch) & 7) != 0) return host::fail(MADI_ERR_INVALID, "reduce_Y: scratch must be 8-byte aligned");
    // the fixed-point column totals hold 3 n_walkers 2^32 < 2^63
    if (n_walkers > 500000000ll) return host::fail(MADI_ERR_UNSUPPORTED, "reduce_Y: at most 5e8 walkers");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    unsigned long long* accum = static_cast<unsigned long long*>(scratch);
    cudaError_t e = cudaMemsetAsync(accum, 0, (size_t)madi_reduce_Y_scratch_bytes(n_cols), s);
    if (e != cudaSuccess) return host::cuda_fail(e, "reduce_Y memset");
    if (n_walkers > 0) {
        // walker rows staged per round: up to 96 KB of shared memory
        const int row_bytes = n_grid * 3 * 8;
        const int wt = std::max(1, std::min(32, (96 * 1024) / row_bytes));
        const size_t smem = (size_t)wt * row_bytes;
        e = cudaFuncSetAttribute(reduce_Y_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return host::cuda_fail(e, "reduce_Y attribute");
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int gx = (n_cols + REDUCE_COLS - 1) / REDUCE_COLS;
        // about 4 CTAs per SM over all column blocks, each walker range a multiple of wt
        const int64_t want = std::max<int64_t>(1, (4ll * sms + gx - 1) / gx);
        int64_t per = (n_walkers + want - 1) / want;
        per = std::max<int64_t>(wt, (per + wt - 1) / wt * wt);
        const int64_t gy = (n_walkers + per - 1) / per;
        if (gy > 65535) return host::fail(MADI_ERR_UNSUPPORTED, "reduce_Y: too many walker blocks");
        reduce_Y_kernel<<<dim3((unsigned)gx, (unsigned)gy), REDUCE_THREADS, smem, s>>>(Y, n_walkers, n_grid, wt, per, jd, jD,
                                                                                       js, coef, n_cols, accum);
        e = cudaGetLastError();
        if (e != cudaSuccess) return host::cuda_fail(e, "reduce_Y launch");
    }
    reduce_Y_finish_kernel<<<(n_cols + 255) / 256, 256, 0, s>>>(reinterpret_cast<const long long*>(accum), n_cols,
                                                                cos_sum, sin_sum);
    e = cudaGetLastError();
    if (e != cudaSuccess) return host::cuda_fail(e, "reduce_Y finish");
    return MADI_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free walk.  The persistent walker needs one zeroed 32-bit tile
// counter besides its inputs and outputs; this entry point keeps it in a
// file-scope device array instead of a caller buffer, so the caller allocates
// nothing for it.  The array is 256 bytes (one word used), lives on every GPU
// that loads this library until the process exits, and is shared by all calls:
// each call clears the word on its own stream before walking, and two calls
// that overlap on the GPU race on it.
// ---------------------------------------------------------------------------
#include <mutex>

#define MADI_WALK_STATIC_SCRATCH_WORDS 64
static __device__ __align__(256) uint32_t g_walk_static_scratch[MADI_WALK_STATIC_SCRATCH_WORDS];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
uint32_t* g_scratch_addr[kMaxDevices] = {};

// Device address of the static scratch on the current device.  The first call
// on a device resolves it with cudaGetSymbolAddress (that device current) and
// caches it.
madi_status static_scratch(uint32_t** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return host::cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return host::fail(MADI_ERR_UNSUPPORTED, "device ordinal %d beyond %d", dev, kMaxDevices);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_walk_static_scratch);
        if (e != cudaSuccess) return host::cuda_fail(e, "cudaGetSymbolAddress(walk scratch)");
        g_scratch_addr[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_scratch_addr[dev];
    return MADI_OK;
}
}  // namespace

extern "C" madi_status madi_walk_batched(const madi_walk_desc* desc, void* stream) {
    host::clear_error();
    if (!desc) return host::fail(MADI_ERR_INVALID, "walk_batched: null descriptor");
    if (desc->precision != 32) return host::fail(MADI_ERR_INVALID, "walk_batched: fp32 walkers only");
    madi_walk_desc d = *desc;
    if (d.grid_blocks <= 0) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int32_t bps = madi_walk_blocks_per_sm(&d);
        if (bps <= 0) return host::fail(MADI_ERR_CUDA, "walk_batched: no resident block fits this descriptor");
        d.grid_blocks = (int32_t)std::min<int64_t>((int64_t)sms * bps, std::max<int64_t>(d.n_tiles, 1));
    }
    return madi_walk(&d, stream);
}

extern "C" madi_status madi_walk_noalloc(const madi_walk_desc* desc, void* stream) {
    host::clear_error();
    if (!desc) return host::fail(MADI_ERR_INVALID, "null walk descriptor");
    const int64_t handed_out = (int64_t)desc->n_tiles + (desc->grid_blocks > 0 ? desc->grid_blocks : 0);
    if (handed_out >= 0x7FFFFFFFll)
        return host::fail(MADI_ERR_CAPACITY,
                          "walk_noalloc: %lld tiles + CTAs exceed the static scratch counter (max %d)",
                          (long long)handed_out, 0x7FFFFFFF - 1);
    uint32_t* counter = nullptr;
    madi_status st = static_scratch(&counter);
    if (st != MADI_OK) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return host::cuda_fail(e, "cudaMemsetAsync(walk scratch)");
    madi_walk_desc d = *desc;
    d.work_counter = counter;
    return madi_walk(&d, stream);
}
