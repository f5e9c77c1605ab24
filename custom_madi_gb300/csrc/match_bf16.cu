// BF16 tensor-core library match (tcgen05 / TMEM), replacing the one-thread-per-
// voxel fp64 scan of _map_kernel_fixed / _map_kernel_free_s0
// (madi/fitters_gpu.py:96-154).
//
// One CTA per SM, persistent over voxel tiles of 128 rows.  The voxels of a
// tile are converted to BF16 in shared memory (K = features padded to 32,
// K-major, no-swizzle UMMA layout); the library, pre-packed once into 8 KB
// tiles of 128 entries in the same layout, streams through four shared stages
// by cp.async.bulk.  Lane 0 of the producer warp issues tcgen05.mma (M=128,
// N=128, K=16, two per tile) into one of four 128-column FP32 TMEM
// accumulators.  Two epilogue warpgroups split each tile's columns: every
// thread owns one voxel row (its TMEM lane) and keeps a top-k of that row over
// its half of the library.
//
// Scores (smaller is better):
//   fixed S0: score_j = |L~_j|^2 - 2 m~.L~_j  (= |m~ - L~_j|^2 - |m~|^2)
//   free  S0: score_j = -(m.r~_j)^2 / |r~_j|^2 when m.r~_j > 0
// with m~ = bf16(m - mu), L~_j = bf16(L_j - mu) (mu the library column mean:
// centring keeps the BF16 products small) and r~_j = bf16(r_j).  For fixed S0
// with F <= 29 the bias is folded into the MMA: three extra K columns carry
// 1 in A and a three-term BF16 split of -|L~_j|^2 / 2 in B, so the accumulator
// is t_j = m~.L~_j - |L~_j|^2 / 2 = -score_j / 2 to fp32 accuracy.
//
// Epilogue per 32-column chunk: the row's 32 keys are staged in shared memory,
// a 32-bit mask marks those under the row's current k-th best, and only the
// marked ones are appended to the row's candidate buffer.  When any lane's
// buffer would overflow, the warp folds all buffers into the sorted register
// top-k with bitonic networks.  Each warpgroup rescores its k candidates in
// fp32 from the fp32 data; the two results are combined (lowest index on ties).
#include <cstdint>
#include <cuda_bf16.h>
#include "madi_device.cuh"
#include "madi_host.h"

namespace madi {
namespace bf16m {

constexpr int TILE_M = 128;                     // voxels per tile (MMA M, TMEM lanes)
constexpr int TILE_N = 128;                     // library entries per tile (MMA N)
constexpr int KPAD = 32;                        // features (+ bias columns) padded to 32
constexpr int BIAS_COLS = 3;                    // folded -|L~|^2/2 as hi + mid + lo BF16
constexpr int CORE = 128;                       // bytes of one 8x8 BF16 core matrix
constexpr int SBO = (KPAD / 8) * CORE;          // 512 B between 8-row groups
constexpr int LBO = CORE;                       // 128 B between K-adjacent core matrices
constexpr int A_BYTES = TILE_M * KPAD * 2;      // 8 KB
constexpr int B_BYTES = TILE_N * KPAD * 2;      // 8 KB
constexpr int AUX_BYTES = TILE_N * 4;           // per-entry |L~|^2 (aux mode) or 1/|r~|^2 (free)
constexpr int STAGES = 4;                       // library tiles in flight
constexpr int ACCS = 4;                         // TMEM accumulators
constexpr int TMEM_COLS = ACCS * TILE_N;        // 512: the whole TMEM of the SM
constexpr int EPI_WG = 2;                       // epilogue warpgroups (column halves)
constexpr int EPI_THREADS = EPI_WG * TILE_M;    // 256
constexpr int EPI_WARPS = EPI_THREADS / 32;     // 8
constexpr int THREADS = EPI_THREADS + 32;       // + producer warp
constexpr int WG_COLS = TILE_N / EPI_WG;        // 64 columns per warpgroup and tile
constexpr int CAP = 64;                         // per-thread candidate buffer entries
constexpr uint32_t SPIN_LIMIT = 1u << 22;       // bounded waits (~0.1-1 s)

enum { MODE_FOLD = 0, MODE_AUX = 1, MODE_FREE = 2 };

// Byte offset of element (row, k) in the no-swizzle K-major canonical layout.
__host__ __device__ __forceinline__ uint32_t canon_off(int row, int k) {
    return (uint32_t)((row >> 3) * SBO + (k >> 3) * LBO + (row & 7) * 16 + (k & 7) * 2);
}

MADI_DEV uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// UMMA shared-memory descriptor: start >> 4, LBO >> 4, SBO >> 4, version 1, no swizzle.
MADI_DEV uint64_t make_sdesc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((LBO >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((SBO >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;                     // descriptor version (sm_100 family)
    return d;                                   // base offset 0, layout type 0 = no swizzle
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major, N = 128, M = 128.
MADI_DEV uint32_t make_idesc() {
    uint32_t d = 0;
    d |= 1u << 4;                               // D format F32
    d |= 1u << 7;                               // A format BF16
    d |= 1u << 10;                              // B format BF16
    d |= (uint32_t)(TILE_N >> 3) << 17;         // N >> 3
    d |= (uint32_t)(TILE_M >> 4) << 24;         // M >> 4
    return d;
}

MADI_DEV void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(bar)), "r"(count) : "memory");
}

MADI_DEV void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_u32(bar)), "r"(bytes) : "memory");
}

MADI_DEV void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(smem_u32(bar)) : "memory");
}

// Bounded parity wait; returns false after SPIN_LIMIT polls.
MADI_DEV bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    for (uint32_t i = 0; i < SPIN_LIMIT; ++i) {
        uint32_t done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                     : "=r"(done) : "r"(a), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

MADI_DEV void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

MADI_DEV void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
MADI_DEV void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

MADI_DEV void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc, uint32_t accumulate) {
    asm volatile("{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                 :: "r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate) : "memory");
}

MADI_DEV void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(smem_u32(bar)) : "memory");
}

// 32 consecutive FP32 columns of this warp's 32 lanes.
MADI_DEV void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                   "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                   "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------------------
// Library packing: fp32 [n_lib][F] -> BF16 canonical tiles, per-entry aux.
// ---------------------------------------------------------------------------
__global__ void column_mean_kernel(const float* lib, int n_lib, int F, float* mu) {
    __shared__ double s[256];
    const int f = blockIdx.x;
    double acc = 0.0;
    for (int i = threadIdx.x; i < n_lib; i += blockDim.x) acc += lib[(size_t)i * F + f];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st) s[threadIdx.x] += s[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) mu[f] = (float)(s[0] / n_lib);
}

__global__ void pack_library_kernel(const float* lib, int n_lib, int F, int n_tiles, int mode, const float* mu,
                                    unsigned char* tiles, float* aux) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)n_tiles * TILE_N) return;
    const int t = (int)(e / TILE_N), n = (int)(e % TILE_N);
    unsigned char* tile = tiles + (size_t)t * B_BYTES;
    const bool live = e < n_lib;
    double q = 0.0;
    for (int k = 0; k < KPAD; ++k) {
        float x = 0.f;
        if (live && k < F) {
            const float v = lib[e * F + k];
            x = mode == MODE_FREE ? v : v - mu[k];
        }
        const __nv_bfloat16 xb = __float2bfloat16_rn(x);
        const double xr = (double)__bfloat162float(xb);
        q += xr * xr;
        *reinterpret_cast<__nv_bfloat16*>(tile + canon_off(n, k)) = xb;
    }
    // The norm is taken of the ROUNDED entry, so the fixed-S0 score is exactly
    // |m~ - L~|^2 - |m~|^2 of the rounded vectors: its error then scales with the
    // residual |m - L| rather than with |m - mu| |L - mu|, and near-ties keep
    // their order (free S0 likewise scores the rounded pair, through 1/|r~|^2).
    if (mode == MODE_FOLD) {
        // -q/2 = hi + mid + lo, each BF16, residual ~2^-25 |q|; padding gets -inf
        const double x = -0.5 * q;
        const __nv_bfloat16 hi = live ? __float2bfloat16_rn((float)x) : __float2bfloat16_rn(-INFINITY);
        const double r1 = live ? x - (double)__bfloat162float(hi) : 0.0;
        const __nv_bfloat16 mid = __float2bfloat16_rn((float)r1);
        const double r2 = r1 - (double)__bfloat162float(mid);
        const __nv_bfloat16 lo = __float2bfloat16_rn((float)r2);
        *reinterpret_cast<__nv_bfloat16*>(tile + canon_off(n, F)) = hi;
        *reinterpret_cast<__nv_bfloat16*>(tile + canon_off(n, F + 1)) = mid;
        *reinterpret_cast<__nv_bfloat16*>(tile + canon_off(n, F + 2)) = lo;
    }
    // Padding entries carry NaN in aux: their score fails every "<" test.
    const float qf = (float)q;
    aux[e] = live ? (mode == MODE_FREE ? 1.f / fmaxf(qf, 1e-30f) : qf) : __int_as_float(0x7fc00000);
}

// ---------------------------------------------------------------------------
// Per-thread top-K: sorted registers + a shared-memory append buffer that is
// merged warp-synchronously by bitonic networks (no serial insertion chains,
// no divergence inside the merge).
// ---------------------------------------------------------------------------
template <int K>
MADI_DEV void cswap(float (&a)[K], int (&ai)[K], int i, int l) {   // ascending at (i, l)
    const bool sw = a[l] < a[i];
    const float x = a[i], y = a[l];
    const int xi = ai[i], yi = ai[l];
    a[i] = sw ? y : x;
    a[l] = sw ? x : y;
    ai[i] = sw ? yi : xi;
    ai[l] = sw ? xi : yi;
}

template <int K>
MADI_DEV void bitonic_sort(float (&a)[K], int (&ai)[K]) {
#pragma unroll
    for (int k = 2; k <= K; k <<= 1)
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
            for (int i = 0; i < K; ++i) {
                const int l = i ^ j;
                if (l > i) {
                    if ((i & k) == 0) cswap<K>(a, ai, i, l);
                    else cswap<K>(a, ai, l, i);
                }
            }
}

// Sorts a bitonic sequence ascending.
template <int K>
MADI_DEV void bitonic_clean(float (&a)[K], int (&ai)[K]) {
#pragma unroll
    for (int j = K >> 1; j > 0; j >>= 1)
#pragma unroll
        for (int i = 0; i < K; ++i) {
            const int l = i ^ j;
            if (l > i) cswap<K>(a, ai, i, l);
        }
}

// Folds this thread's buffered (score, index) entries into ks/kj (ascending)
// K at a time; every lane of the warp takes part.  Buffer entry e of the
// thread lives at buf[e * EPI_THREADS].
template <int K>
MADI_DEV void merge_buffer(float (&ks)[K], int (&kj)[K], float& thr, int& cnt, const float2* buf) {
    const int cmax = __reduce_max_sync(0xffffffffu, cnt);
#pragma unroll 1
    for (int base = 0; base < cmax; base += K) {
        float b[K];
        int bj[K];
#pragma unroll
        for (int i = 0; i < K; ++i) {
            float2 e = make_float2(3.0e38f, 0.f);
            if (base + i < cnt) e = buf[(base + i) * EPI_THREADS];
            b[i] = e.x;
            bj[i] = __float_as_int(e.y);
        }
        bitonic_sort<K>(b, bj);
        // min(ks[i], b[K-1-i]) holds the K smallest of both lists, bitonic
#pragma unroll
        for (int i = 0; i < K; ++i) {
            const float o = b[K - 1 - i];
            if (o < ks[i]) { ks[i] = o; kj[i] = bj[K - 1 - i]; }
        }
        bitonic_clean<K>(ks, kj);
    }
    cnt = 0;
    thr = ks[K - 1];
}

// ---------------------------------------------------------------------------
// Main kernel: warps 0-7 are the epilogue (warpgroup h = warp / 4 takes
// columns [64h, 64h + 64) of every tile; thread tid % 128 = voxel row = TMEM
// lane), lane 0 of warp 8 is the producer (library loads and MMA issue).
// Hand-offs use mbarriers only (every wait bounded):
//   full[s]  / empty[s] : library stage s loaded / consumed by its MMA
//   accf[a]             : accumulator a holds tile scores (and, in the aux and
//                         free modes, the tile's aux row has landed)
//   acce[a]             : the eight epilogue warps are done with accumulator a
//   afull               : the voxel tile (A operand) is written (warpgroup 0)
//   lfull               : warpgroup 1's rescored best per row is written
// Tile sequence g runs over (voxel tile of this CTA, library tile); stage
// g % STAGES, accumulator g % ACCS.  The k-th completion of a barrier is
// waited with parity k & 1.
// ---------------------------------------------------------------------------
struct Smem {
    unsigned char a[A_BYTES];
    unsigned char b[STAGES][B_BYTES];
    float aux[ACCS][TILE_N];
    float4 stage[8][EPI_THREADS];       // the 32 keys of the current chunk, 4 per slot
    float2 buf[CAP][EPI_THREADS];       // candidate buffers (score, index)
    float4 res1[2][TILE_M];             // warpgroup 1 -> 0: (resid, index, s0, -) per row
    uint64_t full[STAGES];
    uint64_t empty[STAGES];
    uint64_t accf[ACCS];
    uint64_t acce[ACCS];
    uint64_t afull;
    uint64_t lfull;
    uint64_t drain;
    uint32_t tmem_base;
    int err;
};

MADI_DEV int err_flag_read(const Smem& S) { return *reinterpret_cast<const volatile int*>(&S.err); }

// Voxel tile -> BF16 canonical A rows (warpgroup 0, each thread its own row),
// then hand the tile to the async proxy and signal the producer.
template <int MODE>
MADI_DEV void write_voxel_tile(Smem& S, const float* __restrict__ meas, const float* __restrict__ mu, int64_t n_vox,
                               int F, int64_t vt, int r, int lane) {
    const int64_t row = vt * TILE_M + r;
    const bool live = row < n_vox;
    for (int kc = 0; kc < KPAD / 8; ++kc) {
        __align__(16) __nv_bfloat16 v8[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int k = kc * 8 + i;
            float x = 0.f;
            if (live && k < F) x = meas[row * F + k] - (MODE == MODE_FREE ? 0.f : __ldg(mu + k));
            if (MODE == MODE_FOLD && k >= F && k < F + BIAS_COLS) x = 1.f;
            v8[i] = __float2bfloat16_rn(x);
        }
        *reinterpret_cast<uint4*>(S.a + canon_off(r, kc * 8)) = *reinterpret_cast<const uint4*>(v8);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // generic -> async proxy
    __syncwarp();
    if (lane == 0) mbar_arrive(&S.afull);
}

template <int MODE>
MADI_DEV void producer(Smem& S, const unsigned char* __restrict__ tiles, const float* __restrict__ aux, int n_tiles,
                       int64_t total, uint32_t tmem) {
    const uint32_t idesc = make_idesc();
    const uint32_t a_base = smem_u32(S.a);
    int64_t gl = 0;                                  // library loads issued
    bool ok = true;
    auto load = [&](int64_t g) -> bool {
        const int st = (int)(g % STAGES);
        if (g >= STAGES && !mbar_wait(&S.empty[st], (uint32_t)((g / STAGES - 1) & 1))) return false;
        mbar_expect_tx(&S.full[st], B_BYTES);
        bulk_g2s(S.b[st], tiles + (size_t)(g % n_tiles) * B_BYTES, B_BYTES, &S.full[st]);
        return true;
    };
    for (; gl < total && gl < STAGES; ++gl)
        if (!load(gl)) { ok = false; break; }
    for (int64_t g = 0; g < total && ok; ++g) {
        const int st = (int)(g % STAGES), acc = (int)(g % ACCS);
        const int tile = (int)(g % n_tiles);
        if (tile == 0 && !mbar_wait(&S.afull, (uint32_t)((g / n_tiles) & 1))) { ok = false; break; }
        if (!mbar_wait(&S.full[st], (uint32_t)((g / STAGES) & 1))) { ok = false; break; }
        if (g >= ACCS && !mbar_wait(&S.acce[acc], (uint32_t)((g / ACCS - 1) & 1))) { ok = false; break; }
        fence_after();
        if (MODE != MODE_FOLD) {
            // the tile's aux row rides on accf[acc] (arrive + tx); the MMA commit is its second arrival
            mbar_expect_tx(&S.accf[acc], AUX_BYTES);
            bulk_g2s(S.aux[acc], aux + (size_t)tile * TILE_N, AUX_BYTES, &S.accf[acc]);
        }
        const uint32_t b_base = smem_u32(S.b[st]);
        const uint32_t d = tmem + (uint32_t)(acc * TILE_N);
        mma_bf16(d, make_sdesc(a_base), make_sdesc(b_base), idesc, 0u);
        mma_bf16(d, make_sdesc(a_base + 2 * LBO), make_sdesc(b_base + 2 * LBO), idesc, 1u);
        mma_commit(&S.empty[st]);
        mma_commit(&S.accf[acc]);
        // refill the stage MMA g-1 used (stays STAGES-1 tiles ahead without
        // waiting on the MMA just issued)
        if (gl < total && gl <= g + STAGES - 1) {
            if (!load(gl)) { ok = false; break; }
            ++gl;
        }
    }
    if (!ok) {
        S.err = 1;
        // let issued copies and MMAs land before TMEM / shared memory go away
        for (int st = 0; st < STAGES; ++st) {
            const int64_t last = gl - 1 - ((gl - 1 - st) % STAGES + STAGES) % STAGES;   // last load into st
            if (last >= 0) mbar_wait(&S.full[st], (uint32_t)((last / STAGES) & 1));
        }
        mma_commit(&S.drain);      // arrives once every earlier MMA is done
        mbar_wait(&S.drain, 0);
    }
}

// fp32 rescore of this thread's k candidates (staged in its buffer) against
// the fp32 data; lowest index on ties.
template <int K, bool FREE>
MADI_DEV void rescore(const float* __restrict__ meas, const float* __restrict__ lib, int64_t row, int n_lib, int F,
                      const float2* mybuf, float& best, int& bj, float& bs0) {
    float m[KPAD];
#pragma unroll
    for (int k = 0; k < KPAD; ++k) m[k] = k < F ? meas[row * F + k] : 0.f;
#pragma unroll 4
    for (int i = 0; i < K; ++i) {
        const float2 cand = mybuf[i * EPI_THREADS];
        const int j = __float_as_int(cand.y);
        if (!(cand.x < 3.0e38f) || j < 0 || j >= n_lib) continue;
        const float* L = lib + (size_t)j * F;
        float lv[KPAD];
#pragma unroll
        for (int k = 0; k < KPAD; ++k) lv[k] = k < F ? __ldg(L + k) : 0.f;
        float dot = 0.f, rr = 0.f;
#pragma unroll
        for (int k = 0; k < KPAD; ++k)
            if (k < F) { dot = fmaf(m[k], lv[k], dot); rr = fmaf(lv[k], lv[k], rr); }
        const float s0 = FREE ? dot / fmaxf(rr, 1e-30f) : 1.f;
        float res = 0.f;
#pragma unroll
        for (int k = 0; k < KPAD; ++k)
            if (k < F) { const float r = m[k] - s0 * lv[k]; res = fmaf(r, r, res); }
        if (FREE && !(dot > 0.f)) res = 3.0e38f;
        if (res < best || (res == best && j < bj)) { best = res; bj = j; bs0 = s0; }
    }
}

template <int K, int MODE>
__global__ void __launch_bounds__(THREADS, 1) match_bf16_kernel(const float* __restrict__ meas, const float* __restrict__ lib,
                                                                int64_t n_vox, int n_lib, int F,
                                                                const unsigned char* __restrict__ tiles,
                                                                const float* __restrict__ aux, const float* __restrict__ mu,
                                                                int n_tiles, int32_t* best_idx, float* best_resid,
                                                                float* best_s0, int* err_flag) {
    static_assert(CAP % K == 0 && CAP >= 32, "buffer holds whole merge batches and a 32-column chunk");
    constexpr bool FREE = MODE == MODE_FREE;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    Smem& S = *reinterpret_cast<Smem*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int i = 0; i < STAGES; ++i) { mbar_init(&S.full[i], 1); mbar_init(&S.empty[i], 1); }
        for (int i = 0; i < ACCS; ++i) {
            mbar_init(&S.accf[i], MODE == MODE_FOLD ? 1 : 2);
            mbar_init(&S.acce[i], EPI_WARPS);
        }
        mbar_init(&S.afull, 4);
        mbar_init(&S.lfull, 4);
        mbar_init(&S.drain, 1);
        S.err = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(&S.tmem_base)), "r"(TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = S.tmem_base;
    const int64_t n_vtiles = (n_vox + TILE_M - 1) / TILE_M;
    const int64_t my_vt = (int64_t)blockIdx.x < n_vtiles ? (n_vtiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;

    if (warp == EPI_WARPS) {
        if (lane == 0) producer<MODE>(S, tiles, aux, n_tiles, my_vt * n_tiles, tmem);
    } else {
        const int wg = warp >> 2;                    // column half
        const int r = tid & (TILE_M - 1);            // voxel row = TMEM lane
        const float2* mybuf = &S.buf[0][tid];
        float2* mybuf_w = &S.buf[0][tid];
        float4* mystage = &S.stage[0][tid];
        const float* mystage_f = reinterpret_cast<const float*>(mystage);
        int64_t g = 0;
        bool ok = true;
        if (wg == 0 && my_vt > 0) write_voxel_tile<MODE>(S, meas, mu, n_vox, F, blockIdx.x, r, lane);
        for (int64_t lv = 0; lv < my_vt && ok; ++lv) {
            const int64_t vt = blockIdx.x + lv * gridDim.x;
            float ks[K];
            int kj[K];
#pragma unroll
            for (int i = 0; i < K; ++i) { ks[i] = 3.0e38f; kj[i] = 0; }
            float thr = 3.0e38f;
            float tthr = -1.5e38f;                   // fold mode: key t hits when t > -thr / 2
            int cnt = 0;
            for (int t = 0; t < n_tiles; ++t, ++g) {
                const int acc = (int)(g % ACCS);
                const bool got_lane = mbar_wait(&S.accf[acc], (uint32_t)((g / ACCS) & 1)) && !err_flag_read(S);
                const bool got = __all_sync(0xffffffffu, got_lane);   // warp-uniform
                if (!got) { S.err = 1; ok = false; break; }
                fence_after();
                const uint32_t taddr = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(acc * TILE_N + wg * WG_COLS);
                const float* ax = S.aux[acc] + wg * WG_COLS;
                const int jb = t * TILE_N + wg * WG_COLS;
#pragma unroll 1
                for (int c = 0; c < WG_COLS; c += 32) {
                    float key[32];
                    tmem_ld32(taddr + (uint32_t)c, key);
                    if (MODE != MODE_FOLD) {
#pragma unroll
                        for (int i = 0; i < 32; i += 4) {
                            const float4 q = *reinterpret_cast<const float4*>(ax + c + i);
                            const float qq[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                const float v = key[i + u];
                                key[i + u] = FREE ? (-v * fabsf(v)) * qq[u] : fmaf(-2.f, v, qq[u]);
                            }
                        }
                    }
#pragma unroll
                    for (int i = 0; i < 32; i += 4)
                        mystage[(i >> 2) * EPI_THREADS] = make_float4(key[i], key[i + 1], key[i + 2], key[i + 3]);
                    // four independent 8-bit masks, then one 32-bit mask
                    uint32_t mk[4] = {0u, 0u, 0u, 0u};
#pragma unroll
                    for (int i = 0; i < 32; ++i) {
                        const bool hit = MODE == MODE_FOLD ? key[i] > tthr : key[i] < thr;
                        if (hit) mk[i >> 3] |= 1u << (i & 7);
                    }
                    uint32_t m = mk[0] | (mk[1] << 8) | (mk[2] << 16) | (mk[3] << 24);
                    const int nh = __popc(m);
                    if (__any_sync(0xffffffffu, cnt + nh > CAP)) {
                        merge_buffer<K>(ks, kj, thr, cnt, mybuf);
                        tthr = -0.5f * thr;
                    }
                    float2* wp = mybuf_w + cnt * EPI_THREADS;
                    const int jc = jb + c;
                    while (m) {
                        const int i = __ffs(m) - 1;
                        m &= m - 1;
                        const float kv = mystage_f[(i >> 2) * (EPI_THREADS * 4) + (i & 3)];
                        *wp = make_float2(MODE == MODE_FOLD ? -2.f * kv : kv, __int_as_float(jc + i));
                        wp += EPI_THREADS;
                    }
                    cnt += nh;
                }
                fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&S.acce[acc]);
            }
            if (!ok) break;
            // every MMA of this voxel tile is complete: the next tile's A may go in now
            if (wg == 0 && lv + 1 < my_vt) write_voxel_tile<MODE>(S, meas, mu, n_vox, F, vt + gridDim.x, r, lane);
            merge_buffer<K>(ks, kj, thr, cnt, mybuf);
            // the (now empty) buffer carries the candidates to the rescore loop, so
            // ks/kj are only ever indexed by constants and stay in registers
#pragma unroll
            for (int i = 0; i < K; ++i) mybuf_w[i * EPI_THREADS] = make_float2(ks[i], __int_as_float(kj[i]));
            const int64_t row = vt * TILE_M + r;
            float best = 3.0e38f, bs0 = 0.f;
            int bj = 0x7FFFFFFF;
            if (row < n_vox) rescore<K, FREE>(meas, lib, row, n_lib, F, mybuf, best, bj, bs0);
            if (wg == 1) {
                S.res1[lv & 1][r] = make_float4(best, __int_as_float(bj), bs0, 0.f);
                __syncwarp();
                if (lane == 0) mbar_arrive(&S.lfull);
            } else {
                const bool got_lane = mbar_wait(&S.lfull, (uint32_t)(lv & 1));
                if (!__all_sync(0xffffffffu, got_lane)) { S.err = 1; ok = false; break; }
                const float4 o = S.res1[lv & 1][r];
                const int j1 = __float_as_int(o.y);
                if (o.x < best || (o.x == best && j1 < bj)) { best = o.x; bj = j1; bs0 = o.z; }
                if (row < n_vox) {
                    best_idx[row] = bj == 0x7FFFFFFF ? 0 : bj;
                    best_resid[row] = best;
                    if (FREE && best_s0) best_s0[row] = bs0;
                }
            }
        }
    }
    // ---- teardown: the producer has drained its copies and MMAs on error ----
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(TMEM_COLS) : "memory");
    }
    if (tid == 0 && S.err) atomicExch(err_flag, 1);
}

}  // namespace bf16m
}  // namespace madi

using namespace madi;
using namespace madi::bf16m;

static int64_t round256(int64_t x) { return (x + 255) & ~int64_t(255); }

int64_t madi_match_bf16_scratch(int64_t n_vox, int32_t n_lib, int32_t n_feat, int32_t topk) {
    (void)n_vox; (void)n_feat; (void)topk;
    const int64_t n_tiles = ((int64_t)n_lib + TILE_N - 1) / TILE_N;
    return round256(n_tiles * B_BYTES) + round256(n_tiles * TILE_N * 4) + round256(KPAD * 4) + 256;
}

// Library column means (fp64 sums), shared with the fp32 fixed-S0 scan.
void madi_match_column_mean(const float* lib, int32_t n_lib, int32_t n_feat, float* mu, cudaStream_t s) {
    column_mean_kernel<<<n_feat, 256, 0, s>>>(lib, n_lib, n_feat, mu);
}

madi_status madi_match_bf16(const madi_match_desc* d, cudaStream_t s) {
    if (d->topk != 8 && d->topk != 16 && d->topk != 32)
        return host::fail(MADI_ERR_UNSUPPORTED, "match bf16: topk must be 8, 16 or 32");
    const int64_t need = madi_match_bf16_scratch(d->n_vox, d->n_lib, d->n_feat, d->topk);
    if (!d->scratch || d->scratch_bytes < need)
        return host::fail(MADI_ERR_CAPACITY, "match bf16: scratch %lld < %lld bytes", (long long)d->scratch_bytes,
                          (long long)need);
    if ((reinterpret_cast<uintptr_t>(d->scratch) & 255) != 0)
        return host::fail(MADI_ERR_INVALID, "match bf16: scratch must be 256-byte aligned");
    const int n_tiles = (d->n_lib + TILE_N - 1) / TILE_N;
    unsigned char* base = static_cast<unsigned char*>(d->scratch);
    unsigned char* tiles = base;
    float* aux = reinterpret_cast<float*>(base + round256((int64_t)n_tiles * B_BYTES));
    float* mu = reinterpret_cast<float*>(base + round256((int64_t)n_tiles * B_BYTES) + round256((int64_t)n_tiles * TILE_N * 4));
    int* err = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(mu) + round256(KPAD * 4));
    const bool free_s0 = d->mode == MADI_MATCH_FREE_S0;
    const int mode = free_s0 ? MODE_FREE : (d->n_feat + BIAS_COLS <= KPAD ? MODE_FOLD : MODE_AUX);
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(int), s);
    if (e != cudaSuccess) return host::cuda_fail(e, "match bf16 memset");
    if (!free_s0) column_mean_kernel<<<d->n_feat, 256, 0, s>>>(d->lib, d->n_lib, d->n_feat, mu);
    const int64_t n_ent = (int64_t)n_tiles * TILE_N;
    pack_library_kernel<<<(unsigned)((n_ent + 255) / 256), 256, 0, s>>>(d->lib, d->n_lib, d->n_feat, n_tiles, mode, mu,
                                                                         tiles, aux);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t n_vtiles = (d->n_vox + TILE_M - 1) / TILE_M;
    const size_t smem = sizeof(Smem);
    // one CTA per SM: it allocates all 512 TMEM columns
    const int grid = (int)std::min<int64_t>(n_vtiles, (int64_t)sms);
#define MADI_LAUNCH_BF16(KK, MD)                                                                          \
    do {                                                                                                  \
        auto k = match_bf16_kernel<KK, MD>;                                                               \
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);             \
        if (e != cudaSuccess) return host::cuda_fail(e, "match bf16 attribute");                          \
        k<<<grid, THREADS, smem, s>>>(d->measured, d->lib, d->n_vox, d->n_lib, d->n_feat, tiles, aux, mu, \
                                      n_tiles, d->best_idx, d->best_resid, d->best_s0, err);              \
    } while (0)
#define MADI_LAUNCH_BF16_K(MD)                                                                            \
    do {                                                                                                  \
        if (d->topk == 8) MADI_LAUNCH_BF16(8, MD);                                                        \
        else if (d->topk == 16) MADI_LAUNCH_BF16(16, MD);                                                 \
        else MADI_LAUNCH_BF16(32, MD);                                                                    \
    } while (0)
    if (mode == MODE_FOLD) MADI_LAUNCH_BF16_K(MODE_FOLD);
    else if (mode == MODE_AUX) MADI_LAUNCH_BF16_K(MODE_AUX);
    else MADI_LAUNCH_BF16_K(MODE_FREE);
#undef MADI_LAUNCH_BF16_K
#undef MADI_LAUNCH_BF16
    e = cudaGetLastError();
    if (e != cudaSuccess) return host::cuda_fail(e, "match bf16 launch");
    return MADI_OK;
}
