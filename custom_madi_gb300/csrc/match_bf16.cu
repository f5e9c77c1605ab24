// BF16 tensor-core library match (tcgen05 / TMEM), replacing the one-thread-per-
// voxel fp64 scan of _map_kernel_fixed / _map_kernel_free_s0
// (madi/fitters_gpu.py:96-154).
//
// One CTA per SM, persistent over voxel tiles of 128 rows.  The voxels of a
// tile are converted to BF16 in shared memory (K = features padded to 32,
// K-major, no-swizzle UMMA layout); the library, pre-packed once into 8 KB
// tiles of 128 entries in the same layout, streams through four shared stages
// by cp.async.bulk, two tiles per step.  Lane 0 of the producer warp issues
// tcgen05.mma (M=128, N=256 = the step's two tiles, K=16, two per step) into
// one of two 256-column FP32 TMEM accumulators.  Epilogue warpgroup h takes
// tile h of every step: every thread owns one voxel row (its TMEM lane) and
// keeps a top-k of that row over its half of the library.
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
// Epilogue per 64-column pass: a warp-uniform test skips passes where no row of
// the warp can hold a candidate; otherwise the keys are staged in shared
// memory, bit masks mark those under the row's current k-th best, and only the
// marked ones are appended to the row's candidate buffer.  When any lane's
// buffer would overflow, the warp folds all buffers into the sorted register
// top-k with bitonic networks.  At the end of a voxel tile each half writes its
// candidates (those under the other half's k-th best); rescore_kernel scores
// them in fp32 from the fp32 data (lowest index on ties).
//
// Scan cut (fixed S0): library and voxels are ordered along the library's
// principal axis, and each voxel tile visits the library tiles nearest its key
// first.  After a tile's first step, the k-th best of each row over those 256
// entries bounds its final k-th best; with the BF16 rounding bound, that and
// |m - L| >= |(m - L).pc| rule out every library tile past a point of the scan
// order, so the tile's scan stops there (first_step_bounds, steplb_kernel).
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
constexpr int PAIR = 2;                         // library tiles per step (one N=256 MMA)
constexpr int MMA_N = PAIR * TILE_N;            // 256
constexpr int STAGES = 4;                       // steps (tile pairs) in flight
constexpr int LOAD_AHEAD = 2;                   // steps loaded ahead of the MMA
constexpr int ACCS = 2;                         // TMEM accumulators of MMA_N columns
constexpr int TMEM_COLS = ACCS * MMA_N;         // 512: the whole TMEM of the SM
constexpr int EPI_WG = 2;                       // epilogue warpgroups (column halves)
constexpr int EPI_THREADS = EPI_WG * TILE_M;    // 256
constexpr int EPI_WARPS = EPI_THREADS / 32;     // 8
constexpr int THREADS = EPI_THREADS + 32;       // + producer warp
constexpr int WG_COLS = 64;                     // columns per epilogue pass (two per step)
constexpr int CAP = 32;                         // per-thread candidate buffer entries
constexpr uint32_t SUSPEND_NS = 20000;          // mbarrier try_wait suspend hint
constexpr uint32_t SPIN_LIMIT = 50000;          // bounded waits: <= SPIN_LIMIT * SUSPEND_NS ~ 1 s
constexpr uint32_t DRAIN_LIMIT = 4 * SPIN_LIMIT; // waits for issued copies / MMAs after an error
constexpr uint32_t STALL_POLLS = 64;            // the test-only stalled wait (MADI_MATCH_FLAG_TEST_STALL)
// Status word in the scratch, read by madi_match_wait: 0 ok, 1 a bounded wait
// ran out (every issued copy and MMA then drained), 2 the drain ran out too.
constexpr int ERR_TIMEOUT = 1;
constexpr float U_BF16 = 0.00390625f;           // BF16 round-to-nearest: |bf16(x) - x| <= 2^-8 |x|
constexpr int SLB_CHUNKS = 4;                   // step bounds prefetched per voxel tile (x 32 steps)
constexpr int ERR_DRAIN = 2;

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

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major, N = 256, M = 128.
MADI_DEV uint32_t make_idesc() {
    uint32_t d = 0;
    d |= 1u << 4;                               // D format F32
    d |= 1u << 7;                               // A format BF16
    d |= 1u << 10;                              // B format BF16
    d |= (uint32_t)(MMA_N >> 3) << 17;          // N >> 3
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

// Bounded parity wait; returns false after `limit` polls.
MADI_DEV bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = SPIN_LIMIT);

// Warp-wide bounded wait polled by lane 0 only (the other lanes would only add
// shared-memory traffic); the result is the same on every lane.
MADI_DEV bool mbar_wait_warp(uint64_t* bar, uint32_t parity, int lane, uint32_t limit = SPIN_LIMIT) {
    bool ok = false;
    if (lane == 0) ok = mbar_wait(bar, parity, limit);
    return __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
}

MADI_DEV bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
    const uint32_t a = smem_u32(bar);
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
                     : "=r"(done) : "r"(a), "r"(parity), "r"(SUSPEND_NS) : "memory");
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

// 64 consecutive FP32 columns of this warp's 32 lanes (one load, one wait).
#define MADI_R8(i) "=r"(r[i]), "=r"(r[i + 1]), "=r"(r[i + 2]), "=r"(r[i + 3]), "=r"(r[i + 4]), "=r"(r[i + 5]), \
                   "=r"(r[i + 6]), "=r"(r[i + 7])
MADI_DEV void tmem_ld64(uint32_t taddr, float* v) {
    uint32_t r[64];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,"
                 "%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,"
                 "%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];"
                 : MADI_R8(0), MADI_R8(8), MADI_R8(16), MADI_R8(24), MADI_R8(32), MADI_R8(40), MADI_R8(48), MADI_R8(56)
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 64; ++i) v[i] = __uint_as_float(r[i]);
}
#undef MADI_R8

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

// Library entry e of the scan order is row lperm[e] of the caller's library.
// Also copies the fp32 row into lrows[e][0..KPAD) (zero padded, 128-byte rows)
// for the rescore.
__global__ void pack_library_kernel(const float* lib, int n_lib, int F, int n_tiles, int mode, const float* mu,
                                    const int32_t* lperm, unsigned char* tiles, float* aux, float* lrows, float* lmax) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)n_tiles * TILE_N) return;
    const int t = (int)(e / TILE_N), n = (int)(e % TILE_N);
    unsigned char* tile = tiles + (size_t)t * B_BYTES;
    const bool live = e < n_lib;
    const int64_t src = live ? lperm[e] : 0;
    double q = 0.0;
    float n2 = 0.f;                                // |L - mu|^2 in fp32 (the bounds' library term)
    for (int k = 0; k < KPAD; ++k) {
        float x = 0.f;
        if (live && k < F) {
            const float v = lib[src * F + k];
            x = mode == MODE_FREE ? v : v - mu[k];
        }
        n2 = fmaf(x, x, n2);
        const __nv_bfloat16 xb = __float2bfloat16_rn(x);
        const double xr = (double)__bfloat162float(xb);
        q += xr * xr;
        *reinterpret_cast<__nv_bfloat16*>(tile + canon_off(n, k)) = xb;
        if (live) lrows[e * KPAD + k] = k < F ? lib[src * F + k] : 0.f;
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
    // non-negative floats order as their bit patterns; rounded up by a relative 2^-20
    if (live && mode != MODE_FREE) atomicMax(reinterpret_cast<int*>(lmax), __float_as_int(sqrtf(n2) * (1.f + 1e-6f)));
    // Padding entries carry NaN in aux: their score fails every "<" test.
    const float qf = (float)q;
    aux[e] = live ? (mode == MODE_FREE ? 1.f / fmaxf(qf, 1e-30f) : qf) : __int_as_float(0x7fc00000);
}

// ---------------------------------------------------------------------------
// Scan order.  Library entries and voxels are put in the order of 256 key
// buckets along the library's principal axis (a stable counting sort: the
// order is deterministic), and each voxel tile visits the library tiles
// nearest its key first, so the rows' k-th best thresholds settle within a
// few tiles and later tiles rarely hold a candidate.  The order changes no
// result beyond the choice among BF16 score ties at the k-th place.  Keys are
// (x - kmu).pc with x the row (free S0: the unit row), kmu the library mean of
// such rows and pc the leading eigenvector of their covariance.
// ---------------------------------------------------------------------------
constexpr int NBUCKET = 256;                    // key buckets
constexpr int VBLK = 1024;                      // rows per ranking block

MADI_DEV float row_scale(const float* x, int F, bool unit) {
    if (!unit) return 1.f;
    float s = 0.f;
    for (int k = 0; k < F; ++k) s = fmaf(x[k], x[k], s);
    return s > 0.f ? rsqrtf(s) : 0.f;
}

// kmu[f] over rows (fp64 sums, fixed order); one block per column.
__global__ void key_mean_kernel(const float* lib, int n_lib, int F, int unit, float* kmu) {
    __shared__ double sh[256];
    const int f = blockIdx.x;
    double acc = 0.0;
    for (int i = threadIdx.x; i < n_lib; i += blockDim.x) {
        const float* x = lib + (size_t)i * F;
        acc += (double)(x[f] * row_scale(x, F, unit != 0));
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) kmu[f] = (float)(sh[0] / n_lib);
}

// cov[a][b] for a <= b (mirrored), one block per pair.
__global__ void key_cov_kernel(const float* lib, int n_lib, int F, int unit, const float* kmu, float* cov) {
    __shared__ double sh[256];
    const int a = blockIdx.x / F, b = blockIdx.x % F;
    if (a > b) return;
    double acc = 0.0;
    for (int i = threadIdx.x; i < n_lib; i += blockDim.x) {
        const float* x = lib + (size_t)i * F;
        const float sc = row_scale(x, F, unit != 0);
        acc += (double)(x[a] * sc - kmu[a]) * (double)(x[b] * sc - kmu[b]);
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) cov[a * F + b] = cov[b * F + a] = (float)(sh[0] / n_lib);
}

// Leading eigenvector by power iteration (one warp, fixed start and count).
__global__ void key_axis_kernel(const float* cov, int F, float* pc) {
    const int lane = threadIdx.x;
    float v = lane < F ? 1.f + 0.01f * lane : 0.f;
    for (int it = 0; it < 200; ++it) {
        float w = 0.f;
        for (int b = 0; b < F; ++b) w = fmaf(lane < F ? cov[lane * F + b] : 0.f, __shfl_sync(0xffffffffu, v, b), w);
        float n2 = w * w;
        for (int o = 16; o > 0; o >>= 1) n2 += __shfl_xor_sync(0xffffffffu, n2, o);
        const float vn = n2 > 0.f ? w * rsqrtf(n2) : v;
        float d2 = (vn - v) * (vn - v);
        for (int o = 16; o > 0; o >>= 1) d2 += __shfl_xor_sync(0xffffffffu, d2, o);
        v = vn;
        if (d2 < 1e-12f) break;                  // warp-uniform: converged to fp32 precision
    }
    if (lane < F) pc[lane] = v;
}

__global__ void key_kernel(const float* x, int64_t n, int F, int unit, const float* kmu, const float* pc, float* key) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* r = x + i * F;
    const float sc = row_scale(r, F, unit != 0);
    float k = 0.f;
    for (int f = 0; f < F; ++f) k = fmaf(r[f] * sc - kmu[f], pc[f], k);
    key[i] = k;
}

// Key range of the library (one CTA).
__global__ void __launch_bounds__(1024) key_range_kernel(const float* key, int n, float* krange) {
    __shared__ float red[2][32];
    float lo = 3.0e38f, hi = -3.0e38f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) { lo = fminf(lo, key[i]); hi = fmaxf(hi, key[i]); }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = lo; red[1][threadIdx.x >> 5] = hi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < (int)(blockDim.x >> 5); ++i) { lo = fminf(red[0][0], red[0][i]); hi = fmaxf(red[1][0], red[1][i]);
                                                            red[0][0] = lo; red[1][0] = hi; }
        krange[0] = red[0][0];
        krange[1] = red[1][0];
    }
}

// Bucket of each key over the library key range (outside values clamp).
MADI_DEV uint8_t key_bucket(float k, const float* krange) {
    const float lo = krange[0], hi = krange[1];
    const float u = hi > lo ? (k - lo) / (hi - lo) : 0.f;
    return (uint8_t)fminf(fmaxf(u * NBUCKET, 0.f), (float)(NBUCKET - 1));
}

__global__ void key_bucket_kernel(const float* key, int64_t n, const float* krange, uint8_t* vb) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) vb[i] = key_bucket(key[i], krange);
}

// Key bounds (min, max) of each library tile in scan order.
__global__ void tile_bounds_kernel(const float* key, const int32_t* lperm, int n_lib, int n_tiles, float* tlo,
                                   float* thi) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tiles) return;
    float lo = 3.0e38f, hi = -3.0e38f;
    for (int e = t * TILE_N; e < min((t + 1) * TILE_N, n_lib); ++e) {
        const float k = key[lperm[e]];
        lo = fminf(lo, k);
        hi = fmaxf(hi, k);
    }
    tlo[t] = lo;
    thi[t] = hi;
}

// Voxel key bucket (over the library key range; outside values clamp).
__global__ void vox_bucket_kernel(const float* meas, int64_t n_vox, int F, int unit, const float* kmu, const float* pc,
                                  const float* krange, float* vkey, uint8_t* vb) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_vox) return;
    const float* r = meas + i * F;
    const float sc = row_scale(r, F, unit != 0);
    float k = 0.f;
    for (int f = 0; f < F; ++f) k = fmaf(r[f] * sc - kmu[f], pc[f], k);
    vkey[i] = k;
    vb[i] = key_bucket(k, krange);
}

// Stable rank of each row (voxel or library entry) among the earlier rows of its block with the
// same bucket (warp match + per-warp histograms), and per-block counts.
__global__ void __launch_bounds__(VBLK) vox_rank_kernel(const uint8_t* vb, int64_t n_vox, uint16_t* vrank,
                                                        uint32_t* cnt) {
    __shared__ uint32_t hw[VBLK / 32][NBUCKET];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < (VBLK / 32) * NBUCKET; i += blockDim.x) (&hw[0][0])[i] = 0u;
    __syncthreads();
    const int64_t v = (int64_t)blockIdx.x * VBLK + threadIdx.x;
    const int b = v < n_vox ? (int)vb[v] : NBUCKET;         // NBUCKET: no voxel
    const uint32_t same = __match_any_sync(0xffffffffu, b);
    const uint32_t rank_w = __popc(same & ((1u << lane) - 1u));
    if (b < NBUCKET && rank_w == 0) hw[warp][b] = __popc(same);
    __syncthreads();
    if (threadIdx.x < NBUCKET) {
        uint32_t run = 0;
        for (int w = 0; w < VBLK / 32; ++w) { const uint32_t c = hw[w][threadIdx.x]; hw[w][threadIdx.x] = run; run += c; }
        cnt[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = run;   // bucket-major
    }
    __syncthreads();
    if (b < NBUCKET) vrank[v] = (uint16_t)(hw[warp][b] + rank_w);
}

// Per bucket (one block each): exclusive prefix of its per-block counts
// (offs[b][blk]) and the bucket total.
__global__ void __launch_bounds__(1024) vox_scan_kernel(const uint32_t* cnt, int nblk, uint32_t* offs, uint32_t* tot) {
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t carry;
    const int b = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nblk; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const uint32_t c = i < nblk ? cnt[(size_t)b * nblk + i] : 0u;
        uint32_t x = c;                                   // inclusive warp scan
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = wsum[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            wsum[lane] = w;                               // inclusive over warps
        }
        __syncthreads();
        const uint32_t before = carry + (warp > 0 ? wsum[warp - 1] : 0u) + x - c;
        if (i < nblk) offs[(size_t)b * nblk + i] = before;
        __syncthreads();
        if (threadIdx.x == 0) carry += wsum[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) tot[b] = carry;
}

// Exclusive scan of the bucket totals (one warp-sized block per 32 buckets, serial).
__global__ void vox_base_kernel(uint32_t* tot) {
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int i = 0; i < NBUCKET; ++i) { const uint32_t c = tot[i]; tot[i] = run; run += c; }
    }
}

__global__ void vox_scatter_kernel(const uint8_t* vb, const uint16_t* vrank, const uint32_t* offs, const uint32_t* base,
                                   int64_t n_vox, int nblk, int32_t* vperm) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_vox) return;
    const int64_t blk = v / VBLK;
    const int b = vb[v];
    vperm[base[b] + offs[(size_t)b * nblk + blk] + vrank[v]] = (int32_t)v;
}

// Scan order of the library tiles for each voxel tile: the tile holding the
// voxel tile's median key first, then outward by key distance.
__global__ void order_kernel(const float* vkey, const int32_t* vperm, int64_t n_vox, int64_t n_vtiles,
                             const float* tlo, const float* thi, int n_tiles, uint16_t* order) {
    const int64_t vt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (vt >= n_vtiles) return;
    uint16_t* o = order + vt * n_tiles;
    const float key = vkey[vperm[min(vt * TILE_M + TILE_M / 2, n_vox - 1)]];
    int t0 = 0;
    while (t0 < n_tiles - 1 && thi[t0] < key) ++t0;
    o[0] = (uint16_t)t0;
    int a = t0 - 1, b = t0 + 1;
    for (int s = 1; s < n_tiles; ++s) {
        const float da = a >= 0 ? key - thi[a] : 3.0e38f;
        const float db = b < n_tiles ? tlo[b] - key : 3.0e38f;
        if (da <= db) o[s] = (uint16_t)(a--);
        else o[s] = (uint16_t)(b++);
    }
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
// MB at a time; every lane of the warp takes part.  Buffer entry e of the
// thread lives at buf[e * EPI_THREADS].  With the batch b sorted ascending and
// padded with +inf to length K, min(ks[i], b[K-1-i]) holds the K smallest of
// both lists as a bitonic sequence; only i >= K - MB can change.  The new
// threshold is the K-th best so far, or thr0 (a bound on the row's final K-th
// best) when that is tighter.
template <int K, int MB>
MADI_DEV void merge_buffer(float (&ks)[K], int (&kj)[K], float& thr, int& cnt, const float2* buf, float thr0) {
    const int cmax = __reduce_max_sync(0xffffffffu, cnt);
#pragma unroll 1
    for (int base = 0; base < cmax; base += MB) {
        float b[MB];
        int bj[MB];
#pragma unroll
        for (int i = 0; i < MB; ++i) {
            float2 e = make_float2(3.0e38f, 0.f);
            if (base + i < cnt) e = buf[(base + i) * EPI_THREADS];
            b[i] = e.x;
            bj[i] = __float_as_int(e.y);
        }
        bitonic_sort<MB>(b, bj);
#pragma unroll
        for (int i = K - MB; i < K; ++i) {
            const float o = b[K - 1 - i];
            if (o < ks[i]) { ks[i] = o; kj[i] = bj[K - 1 - i]; }
        }
        bitonic_clean<K>(ks, kj);
    }
    cnt = 0;
    thr = fminf(ks[K - 1], thr0);
}

// One append pass: up to four marked entries from each of two masks (column
// offsets oa, ob within the staged keys); all eight staged loads issue before
// the stores, so a pass costs about one load latency.
template <int MODE>
MADI_DEV void append_pass(uint32_t& ma, int oa, uint32_t& mb, int ob, float2*& wp, const float* stage_f, int jc) {
    int ix[8];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        ix[u] = ma ? __ffs(ma) - 1 + oa : -1;
        ma &= ma - 1u;
        ix[u + 4] = mb ? __ffs(mb) - 1 + ob : -1;
        mb &= mb - 1u;
    }
    float kv[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) kv[u] = ix[u] >= 0 ? stage_f[(ix[u] >> 2) * (EPI_THREADS * 4) + (ix[u] & 3)] : 0.f;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        if (ix[u] >= 0) {
            *wp = make_float2(MODE == MODE_FOLD ? -2.f * kv[u] : kv[u], __int_as_float(jc + ix[u]));
            wp += EPI_THREADS;
        }
    }
}

// ---------------------------------------------------------------------------
// Packed top-k (fixed S0, scans of at most 2^PK_BITS positions).  A candidate
// is one 32-bit word: the BF16 half-residual d = |m~ - L~|^2 / 2 = |m~|^2 / 2 - t
// (t the folded key), clamped to [0, 3e38], with its low PK_BITS mantissa bits
// replaced by the scan position.  Words order as (d to 2^-8 of itself,
// position), so a compare-exchange of the sorting networks is an unsigned min
// and max, and a buffer entry takes 4 bytes.  The quantisation moves only the
// choice among entries within 2^-8 of each other in d at the k-th place; the
// fp32 rescore decides among the candidates.
// ---------------------------------------------------------------------------
constexpr int PK_BITS = 15;
constexpr uint32_t PK_MASK = (1u << PK_BITS) - 1u;
constexpr uint32_t PK_EMPTY = 0xFFFFFFFFu;
// packed entries per thread: the whole buffer at top-32; at smaller k the
// threshold has to tighten sooner, so the buffer folds as often as the float one
template <int K>
__host__ __device__ constexpr int cap_pk() { return K >= 32 ? 2 * CAP : CAP; }

MADI_DEV uint32_t pk_word(float d, int pos) {
    const float dd = d > 0.f ? fminf(d, 3.0e38f) : (d == d ? 0.f : 3.0e38f);   // NaN sorts last
    return (__float_as_uint(dd) & ~PK_MASK) | (uint32_t)pos;
}
// Folded-key threshold t > tthr equivalent to "d below the top of w's quantum".
MADI_DEV float pk_tthr(uint32_t w, float hm2) {
    return w >= 0x7F800000u ? -3.0e38f : hm2 - __uint_as_float(w | PK_MASK);
}

template <int K>
MADI_DEV void bitonic_sort_u(uint32_t (&a)[K]) {
#pragma unroll
    for (int k = 2; k <= K; k <<= 1)
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
            for (int i = 0; i < K; ++i) {
                const int l = i ^ j;
                if (l > i) {
                    const uint32_t x = a[i], y = a[l];
                    const bool up = (i & k) == 0;
                    a[i] = up ? min(x, y) : max(x, y);
                    a[l] = up ? max(x, y) : min(x, y);
                }
            }
}

template <int K>
MADI_DEV void bitonic_clean_u(uint32_t (&a)[K]) {
#pragma unroll
    for (int j = K >> 1; j > 0; j >>= 1)
#pragma unroll
        for (int i = 0; i < K; ++i) {
            const int l = i ^ j;
            if (l > i) {
                const uint32_t x = a[i], y = a[l];
                a[i] = min(x, y);
                a[l] = max(x, y);
            }
        }
}

// Packed merge_buffer: folds this thread's buffered words into ks, MB at a time.
template <int K, int MB>
MADI_DEV void merge_buffer_u(uint32_t (&ks)[K], uint32_t& thr, int& cnt, const uint32_t* buf, uint32_t thr0) {
    const int cmax = __reduce_max_sync(0xffffffffu, cnt);
#pragma unroll 1
    for (int base = 0; base < cmax; base += MB) {
        uint32_t b[MB];
#pragma unroll
        for (int i = 0; i < MB; ++i) b[i] = base + i < cnt ? buf[(base + i) * EPI_THREADS] : PK_EMPTY;
        bitonic_sort_u<MB>(b);
#pragma unroll
        for (int i = K - MB; i < K; ++i) ks[i] = min(ks[i], b[K - 1 - i]);
        bitonic_clean_u<K>(ks);
    }
    cnt = 0;
    thr = min(ks[K - 1], thr0);
}

// Packed append pass (see append_pass): staged keys are folded keys t.
MADI_DEV void append_pass_u(uint32_t& ma, int oa, uint32_t& mb, int ob, uint32_t*& wp, const float* stage_f, int jc,
                            float hm2) {
    int ix[8];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        ix[u] = ma ? __ffs(ma) - 1 + oa : -1;
        ma &= ma - 1u;
        ix[u + 4] = mb ? __ffs(mb) - 1 + ob : -1;
        mb &= mb - 1u;
    }
    float kv[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) kv[u] = ix[u] >= 0 ? stage_f[(ix[u] >> 2) * (EPI_THREADS * 4) + (ix[u] & 3)] : 0.f;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        if (ix[u] >= 0) {
            *wp = pk_word(hm2 - kv[u], jc + ix[u]);
            wp += EPI_THREADS;
        }
    }
}

// ---------------------------------------------------------------------------
// Main kernel: warps 0-7 are the epilogue (warpgroup h = warp / 4 takes tile
// h of every step, accumulator columns [128h, 128h + 128), in two 64-column
// passes; thread tid % 128 = voxel row = TMEM lane), lane 0 of warp 8 is the
// producer (library loads and MMA issue).
// Hand-offs use mbarriers only (every wait bounded):
//   full[s]             : library stage s loaded (a stage is refilled only once
//                         the acce wait has certified its MMA complete)
//   accf[a]             : accumulator a holds tile scores (and, in the aux and
//                         free modes, the tile's aux row has landed)
//   acce[a]             : the eight epilogue warps are done with accumulator a
//   afull               : a voxel tile (A operand, two buffers) is written
//                         (warpgroup 0, during the previous voxel tile's first step)
//   lfull, lempty       : after a voxel tile's first step (scan cut): warpgroup
//                         1's top-k is in its stage slots / warpgroup 0 has read
//                         it and published the tile's step count and row bounds
//                         (warpgroup 1 waits for that before going on, so lfull
//                         never completes two phases ahead of its waiter)
//   rfull               : warpgroup 0's four partial maxima are written
//   vready              : the voxel tile's step count is written (warpgroup 0,
//                         warp 0; waited by the producer and warpgroup 0)
//   efull, eempty       : packed top-k, end of a voxel tile: warpgroup 1's
//                         final list is in its stage slots / warpgroup 0 has
//                         published each row's union k-th word (warpgroup 1
//                         waits for it, so efull never runs two phases ahead)
// Tile sequence g runs over (voxel tile of this CTA, library tile); stage
// g % STAGES, accumulator g % ACCS.  The k-th completion of a barrier is
// waited with parity k & 1.
// ---------------------------------------------------------------------------
struct Plan {
    const float* meas;
    const float* lib;
    int64_t n_vox;
    int n_lib, F, n_tiles;
    const unsigned char* tiles;         // packed library in scan order
    const float* aux;
    const float* mu;
    const int32_t* vperm;               // voxel tile rows -> caller's voxel rows
    const int32_t* lperm;               // library scan position -> caller's library rows
    const float* lrows;                 // fp32 library rows in scan order, KPAD floats each
    const uint16_t* order;              // [voxel tile][scan position] -> library tile
    const float* steplb;                // [voxel tile][step] lower bound on |m~ - L~| - u |m - mu| - u |L - mu|
    const float2* rownorm;              // [scan row] (|m~|^2 of the BF16 row, |m - mu|)
    const float* lmax;                  // max over the library of |L - mu| (fixed S0), device scalar
    int cut;                            // 1: cut each voxel tile's scan after its first step (fixed S0)
    int32_t* cand;                      // [scan row][half][k] candidate scan positions, -1 terminated
    int32_t* best_idx;
    float* best_resid;
    float* best_s0;
    int* err;
    int test_stall;                     // tests only: one epilogue wait that nothing completes
};

struct Smem {
    unsigned char a[2][A_BYTES];                 // voxel tiles (A operand) of consecutive voxel tiles
    unsigned char b[STAGES][PAIR * B_BYTES];     // a step's two tiles back to back = one 256-row operand
    float aux[ACCS][PAIR][TILE_N];
    float4 stage[WG_COLS / 4][EPI_THREADS];   // the 64 keys of the current tile, 4 per slot
    float2 buf[CAP][EPI_THREADS];       // candidate buffers (score, index)
    uint2 thr_pub[EPI_WG][TILE_M];      // (voxel tile, k-th best score) of each row and half
    uint64_t full[STAGES];
    uint64_t accf[ACCS];
    uint64_t acce[ACCS];
    int lt_stage[STAGES][PAIR];         // library tiles held by each stage (producer only)
    uint64_t afull;
    float thr0[TILE_M];                 // row bounds from the first step (warpgroup 0 -> 1)
    uint32_t ucut[TILE_M];              // packed top-k: the k-th word of the union of both halves, per row
    float red[4][2];                    // warpgroup 0 partial maxima of the residual bound
    int vsteps[2];                      // steps of the current voxel tiles (by parity)
    uint64_t lfull;
    uint64_t lempty;
    uint64_t rfull;
    uint64_t vready;
    uint64_t efull;
    uint64_t eempty;
    uint64_t drain;
    uint64_t never;                     // no thread ever arrives (the test-only stalled wait)
    int64_t n_loaded, n_issued;         // producer: steps whose copies / MMAs were issued
    uint32_t tmem_base;
    int err;
};

MADI_DEV int err_flag_read(const Smem& S) { return *reinterpret_cast<const volatile int*>(&S.err); }

// Voxel tile -> BF16 canonical A rows (warpgroup 0, each thread its own row),
// then hand the tile to the async proxy and signal the producer.
template <int MODE>
MADI_DEV void write_voxel_tile(Smem& S, const Plan& P, int64_t vt, int buf, int r, int lane) {
    const int64_t pos = vt * TILE_M + r;
    const bool live = pos < P.n_vox;
    const int64_t row = live ? P.vperm[pos] : 0;
    for (int kc = 0; kc < KPAD / 8; ++kc) {
        __align__(16) __nv_bfloat16 v8[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int k = kc * 8 + i;
            float x = 0.f;
            if (live && k < P.F) x = P.meas[row * P.F + k] - (MODE == MODE_FREE ? 0.f : __ldg(P.mu + k));
            if (MODE == MODE_FOLD && k >= P.F && k < P.F + BIAS_COLS) x = 1.f;
            v8[i] = __float2bfloat16_rn(x);
        }
        *reinterpret_cast<uint4*>(S.a[buf] + canon_off(r, kc * 8)) = *reinterpret_cast<const uint4*>(v8);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // generic -> async proxy
    __syncwarp();
    if (lane == 0) mbar_arrive(&S.afull);
}

// Steps (library tile pairs) of a whole scan; with the scan cut and more than
// two steps, a voxel tile's count is known only after its first step (at
// least two steps are always scanned).
MADI_DEV int full_steps(const Plan& P) { return (P.n_tiles + PAIR - 1) / PAIR; }
MADI_DEV bool dynamic_steps(const Plan& P) { return P.cut && full_steps(P) > 2; }

// Scan cut bounds (fixed S0), one warp per voxel tile.  Every entry j of
// library tile o has |m~ - L~_j| >= |k(m) - k(L_j)| - u (|m - mu| + |L_j - mu|)
// (k the principal-axis key, u the BF16 unit roundoff), and for every row of
// the voxel tile |k(m) - k(L_j)| >= d(o) - W, with d(o) the distance of the
// tile's key range from the voxel tile's median key and W the rows' largest
// distance from it.  steplb[vt][s] is the smallest of these bounds (less
// fp32 slack) over scan positions 2s and later, so it does not decrease with
// s: a step whose steplb exceeds B, every row's residual bound (from its k-th
// best over the first step) plus u |m - mu| plus u max |L - mu|, and all later
// steps hold no entry that could enter a row's top-k.
__global__ void steplb_kernel(const float* vkey, const int32_t* vperm, int64_t n_vox, int64_t n_vtiles,
                              const float* tlo, const float* thi, const uint16_t* order, int n_tiles, float* steplb) {
    const int64_t vt = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (vt >= n_vtiles) return;
    const float kmed = vkey[vperm[min(vt * TILE_M + TILE_M / 2, n_vox - 1)]];
    float W = 0.f;
    for (int r = lane; r < TILE_M; r += 32) {
        const int64_t pos = vt * TILE_M + r;
        if (pos < n_vox) W = fmaxf(W, fabsf(vkey[vperm[pos]] - kmed));
    }
    for (int o = 16; o > 0; o >>= 1) W = fmaxf(W, __shfl_xor_sync(0xffffffffu, W, o));
    const float slack = 1e-4f * (1.f + fabsf(kmed) + W);      // fp32 keys and |pc| = 1 to ~1e-6
    const int n_steps = (n_tiles + PAIR - 1) / PAIR;
    float carry = 3.0e38f;                          // minimum over the positions after this chunk
    for (int base = ((n_tiles - 1) / 32) * 32; base >= 0; base -= 32) {
        const int i = base + lane;
        float lb = 3.0e38f;
        if (i < n_tiles) {
            const int o = order[vt * n_tiles + i];
            const float d = fmaxf(0.f, fmaxf(tlo[o] - kmed, kmed - thi[o]));
            lb = (d - W) * (1.f - 1e-5f) - slack;
        }
        // suffix minimum within the chunk (lanes above), then the chunks after it
        for (int o = 1; o < 32; o <<= 1) {
            const float y = __shfl_down_sync(0xffffffffu, lb, o);
            if (lane + o < 32) lb = fminf(lb, y);
        }
        lb = fminf(lb, carry);
        carry = __shfl_sync(0xffffffffu, lb, 0);
        if (i < n_tiles && (i & 1) == 0) steplb[vt * n_steps + i / 2] = lb;
    }
}

// (|m~|^2 of the BF16 row the MMA sees, |m - mu|) of each scan row (fixed S0).
__global__ void row_norm_kernel(const float* meas, const int32_t* vperm, int64_t n_vox, int F, const float* mu,
                                float2* rownorm) {
    const int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= n_vox) return;
    const int64_t row = vperm[pos];
    float mh2 = 0.f, mn2 = 0.f;
    for (int k = 0; k < F; ++k) {
        const float x = meas[row * F + k] - mu[k];
        const float xb = __bfloat162float(__float2bfloat16_rn(x));
        mh2 = fmaf(xb, xb, mh2);
        mn2 = fmaf(x, x, mn2);
    }
    rownorm[pos] = make_float2(mh2, sqrtf(mn2));
}

// Library tile at scan position i of voxel tile vt (the all-padding tile past the end).
MADI_DEV int scan_tile(const Plan& P, int64_t vt, int i) {
    return i < P.n_tiles ? (int)P.order[vt * P.n_tiles + i] : P.n_tiles;
}

// Lane 0 of the producer warp waits on barriers and issues the copies and
// MMAs.  The step sequence runs over this CTA's voxel tiles; step s of a tile
// covers scan positions 2s and 2s + 1 of its order (an odd tile count is
// padded with the all-padding tile n_tiles).  Under the scan cut a tile's
// step count comes from warpgroup 0 after its first step (vready): each
// iteration issues its MMA before its loads, so the load that needs the count
// (the tile's third step, or the next tile's first) waits for it only after
// the first step's MMA went out.  Scan order entries are read one load ahead.
template <int MODE>
MADI_DEV void producer(Smem& S, const Plan& P, int64_t my_vt, uint32_t tmem, int lane) {
    const uint32_t idesc = make_idesc();
    int64_t gl = 0;                                  // steps loaded
    int64_t g = 0;                                   // steps whose MMAs were issued
    bool ok = true;
    // The stage refilled with step g + LOAD_AHEAD last held step
    // g + LOAD_AHEAD - STAGES <= g - ACCS; the acce wait that precedes the
    // refill certifies the epilogue of step g - ACCS, hence that MMA's (and all
    // earlier MMAs') completion, so the stage is free without a barrier of its own.
    static_assert(STAGES - LOAD_AHEAD >= ACCS, "a refilled stage must be certified free by the acce wait");
    if (lane == 0) {
        const bool dyn = MODE != MODE_FREE && dynamic_steps(P);
        const int n_first = dyn ? 2 : full_steps(P);    // steps known before a tile's count
        int st_first[STAGES], st_par[STAGES];        // per stage: first step of its voxel tile, tile parity
        // load cursor: voxel tile slot, step, steps known so far, whether that is the count
        int64_t l_lv = 0;
        int l_s = 0, l_n = n_first;
        bool l_final = !dyn;
        // the load cursor on the next step that exists; false past the last one
        auto settle = [&]() -> bool {
            while (l_lv < my_vt) {
                if (l_s < l_n) return true;
                if (!l_final) {
                    if (!mbar_wait(&S.vready, (uint32_t)(l_lv & 1), SPIN_LIMIT)) { ok = false; return false; }
                    l_n = S.vsteps[l_lv & 1];
                    l_final = true;
                    continue;
                }
                ++l_lv;
                l_s = 0;
                l_n = n_first;
                l_final = !dyn;
            }
            return false;
        };
        auto load = [&](int64_t q) {
            const int st = (int)(q % STAGES);
            const int64_t vt = blockIdx.x + l_lv * (int64_t)gridDim.x;
            const int lt0 = scan_tile(P, vt, PAIR * l_s), lt1 = scan_tile(P, vt, PAIR * l_s + 1);
            st_first[st] = l_s == 0;
            st_par[st] = (int)(l_lv & 1);
            ++l_s;
            S.lt_stage[st][0] = lt0;
            S.lt_stage[st][1] = lt1;
            mbar_expect_tx(&S.full[st], PAIR * B_BYTES);
            bulk_g2s(S.b[st], P.tiles + (size_t)lt0 * B_BYTES, B_BYTES, &S.full[st]);
            bulk_g2s(S.b[st] + B_BYTES, P.tiles + (size_t)lt1 * B_BYTES, B_BYTES, &S.full[st]);
        };
        for (; gl < LOAD_AHEAD && settle(); ++gl) load(gl);
        while (ok && g < gl) {                       // loads and MMAs go in the same order, one each per step
            const int st = (int)(g % STAGES), acc = (int)(g % ACCS);
            if (g >= ACCS && !mbar_wait(&S.acce[acc], (uint32_t)((g / ACCS - 1) & 1), SPIN_LIMIT)) { ok = false; break; }
            if (st_first[st] && !mbar_wait(&S.afull, (uint32_t)st_par[st], SPIN_LIMIT)) { ok = false; break; }
            if (!mbar_wait(&S.full[st], (uint32_t)((g / STAGES) & 1), SPIN_LIMIT)) { ok = false; break; }
            fence_after();
            if (MODE != MODE_FOLD) {
                // the step's aux rows ride on accf[acc] (arrive + tx); the MMA commit is its second arrival
                mbar_expect_tx(&S.accf[acc], PAIR * AUX_BYTES);
                bulk_g2s(S.aux[acc][0], P.aux + (size_t)S.lt_stage[st][0] * TILE_N, AUX_BYTES, &S.accf[acc]);
                bulk_g2s(S.aux[acc][1], P.aux + (size_t)S.lt_stage[st][1] * TILE_N, AUX_BYTES, &S.accf[acc]);
            }
            const uint32_t a_base = smem_u32(S.a[st_par[st]]);
            const uint32_t b_base = smem_u32(S.b[st]);
            const uint32_t d = tmem + (uint32_t)(acc * MMA_N);
            mma_bf16(d, make_sdesc(a_base), make_sdesc(b_base), idesc, 0u);
            mma_bf16(d, make_sdesc(a_base + 2 * LBO), make_sdesc(b_base + 2 * LBO), idesc, 1u);
            mma_commit(&S.accf[acc]);
            ++g;
            // loads up to step (g - 1) + LOAD_AHEAD: the acce wait above certified
            // the MMA of the step that last used each refilled stage
            for (; gl < g + LOAD_AHEAD; ++gl) {
                // a load that needs a tile's step count waits for it only once
                // every loaded step's MMA has gone out
                if (l_lv < my_vt && l_s >= l_n && !l_final && g < gl) break;
                if (!settle()) break;
                load(gl);
            }
        }
        S.n_loaded = gl;
        S.n_issued = g;
        if (!ok) S.err = ERR_TIMEOUT;
    }
    __syncwarp();
}

// After an error (the epilogue may have left before consuming every step):
// wait, bounded, for every copy and MMA the producer issued, so that nothing
// lands in shared memory or TMEM once they are released.  The last load into
// each stage completes its `full` phase; the last step on each accumulator
// completes its `accf` phase (the step's aux copies and its MMA commit); a
// final commit on `drain` covers every earlier MMA.  Each of these is the
// latest phase of its barrier, so its parity is unambiguous.  Returns false if
// a wait ran out.
MADI_DEV bool drain_issued(Smem& S) {
    const int64_t gl = S.n_loaded, gi = S.n_issued;
    bool ok = true;
    for (int st = 0; st < STAGES; ++st) {
        const int64_t last = gl - 1 - ((gl - 1 - st) % STAGES + STAGES) % STAGES;   // last load into st
        if (last >= 0) ok = mbar_wait(&S.full[st], (uint32_t)((last / STAGES) & 1), DRAIN_LIMIT) && ok;
    }
    for (int a = 0; a < ACCS; ++a) {
        const int64_t last = gi - 1 - ((gi - 1 - a) % ACCS + ACCS) % ACCS;          // last step on a
        if (last >= 0) ok = mbar_wait(&S.accf[a], (uint32_t)((last / ACCS) & 1), DRAIN_LIMIT) && ok;
    }
    mma_commit(&S.drain);      // arrives once every earlier MMA is done
    return mbar_wait(&S.drain, 0, DRAIN_LIMIT) && ok;
}

// fp32 rescore of the candidates of one voxel against the fp32 data; lowest
// caller index on ties.  Two adjacent threads take the voxel, one per half's
// list (scan positions, a prefix of its K slots with -1 after it), and combine
// their bests by shuffle.  Library rows come from the padded scan-order copy
// (RQ aligned 16-byte loads each, RQ >= F/4), two candidates per round with
// all their loads in flight; many warps per SM cover the latency.
template <int K, bool FREE, int RQ>
__global__ void __launch_bounds__(256, 2) rescore_kernel(const Plan P) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t pos = t >> 1;
    const int h = (int)(t & 1);
    const bool live = pos < P.n_vox;
    const int64_t row = live ? P.vperm[pos] : 0;
    const int F = P.F, nq = (F + 3) / 4;
    float m[4 * RQ];
#pragma unroll
    for (int k = 0; k < 4 * RQ; ++k) m[k] = live && k < F ? P.meas[row * F + k] : 0.f;
    float best = 3.0e38f, bs0 = 0.f;
    int bj = 0x7FFFFFFF;
    const int4* cand = reinterpret_cast<const int4*>(P.cand + (live ? pos : 0) * (EPI_WG * K) + h * K);
#pragma unroll 1
    for (int q4 = 0; live && q4 < K / 4; ++q4) {
        const int4 c4 = cand[q4];
        const int cc[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
        for (int p2 = 0; p2 < 4; p2 += 2) {
            int e[2], j[2];
            float4 lv[2][RQ];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int c = cc[p2 + u];
                e[u] = c >= 0 && c < P.n_lib ? c : -1;
                j[u] = e[u] >= 0 ? __ldg(P.lperm + e[u]) : -1;
                const float4* L = reinterpret_cast<const float4*>(P.lrows + (size_t)(e[u] < 0 ? 0 : e[u]) * KPAD);
#pragma unroll
                for (int q = 0; q < RQ; ++q)
                    lv[u][q] = (e[u] >= 0 && q < nq) ? __ldg(L + q) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (e[u] < 0) continue;
                const float* lf = reinterpret_cast<const float*>(lv[u]);
                float dot = 0.f, rr = 0.f;
#pragma unroll
                for (int k = 0; k < 4 * RQ; ++k) { dot = fmaf(m[k], lf[k], dot); rr = fmaf(lf[k], lf[k], rr); }
                const float s0 = FREE ? dot / fmaxf(rr, 1e-30f) : 1.f;
                float res = 0.f;
#pragma unroll
                for (int k = 0; k < 4 * RQ; ++k) { const float r = m[k] - s0 * lf[k]; res = fmaf(r, r, res); }
                if (FREE && !(dot > 0.f)) res = 3.0e38f;
                if (res < best || (res == best && j[u] < bj)) { best = res; bj = j[u]; bs0 = s0; }
            }
        }
        if (c4.w < 0) break;
    }
    // combine the two halves (lanes 2i, 2i + 1)
    const float ob = __shfl_xor_sync(0xffffffffu, best, 1);
    const int oj = __shfl_xor_sync(0xffffffffu, bj, 1);
    const float os0 = __shfl_xor_sync(0xffffffffu, bs0, 1);
    if (ob < best || (ob == best && oj < bj)) { best = ob; bj = oj; bs0 = os0; }
    if (!live || h != 0 || bj == 0x7FFFFFFF) return;   // no candidates: the voxel's CTA gave up
    P.best_idx[row] = bj;
    P.best_resid[row] = best;
    if (FREE && P.best_s0) P.best_s0[row] = bs0;
}

// Warpgroup 0, after its rows' residual bounds rb: reduce them over the tile
// (rfull), let warp 0 count the steps whose key lower bound (steplb,
// prefetched in slb) does not exceed B = max rb + u max|L - mu| and publish
// the count (vready), then release warpgroup 1 (lempty).  False if a bounded
// wait ran out.
MADI_DEV bool publish_steps(Smem& S, const Plan& P, uint32_t par, int warp, int lane, float rb, float lm,
                            const float (&slb)[SLB_CHUNKS], int64_t vt, int& n_steps) {
    for (int o = 16; o > 0; o >>= 1) rb = fmaxf(rb, __shfl_xor_sync(0xffffffffu, rb, o));
    if (lane == 0) {
        S.red[warp][0] = rb;
        mbar_arrive(&S.rfull);
    }
    if (warp == 0) {
        if (!mbar_wait_warp(&S.rfull, par, lane)) return false;
        const float B = fmaxf(fmaxf(S.red[0][0], S.red[1][0]), fmaxf(S.red[2][0], S.red[3][0])) + U_BF16 * lm;
        const int full = full_steps(P);
        int count = 0;                               // steplb does not decrease: the steps within B are a prefix
#pragma unroll
        for (int c = 0; c < SLB_CHUNKS; ++c)
            count += __popc(__ballot_sync(0xffffffffu, c * 32 + lane < full && slb[c] <= B));
        for (int c = SLB_CHUNKS; c * 32 < full; ++c) {  // libraries beyond SLB_CHUNKS * 32 steps
            const int s2 = c * 32 + lane;
            count += __popc(__ballot_sync(0xffffffffu, s2 < full && P.steplb[vt * full + s2] <= B));
        }
        const int steps = max(2, min(full, count));
        if (lane == 0) {
            S.vsteps[par] = steps;
            mbar_arrive(&S.vready);
        }
        n_steps = steps;
    } else {
        if (!mbar_wait_warp(&S.vready, par, lane)) return false;
        n_steps = S.vsteps[par];
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&S.lempty);
    return true;
}

// Scan cut, after a voxel tile's first step.  Both halves fold their buffers;
// warpgroup 1 hands its ascending top-k to warpgroup 0 in its stage slots;
// warpgroup 0 takes each row's k-th best over the step's 256 entries (the
// union of the two lists) as the row's bound thr0 on its final k-th best and
// its residual bound sqrt(thr0 + |m~|^2) + u |m - mu|, reduces the residual
// bounds over the tile, and warp 0 counts the steps whose key lower bound
// (steplb, prefetched in slb) does not exceed B.  rn is the row's prefetched
// (|m~|^2, |m - mu|).  Every wait is bounded; false if one ran out.
template <int K, int MB>
MADI_DEV bool first_step_bounds(Smem& S, const Plan& P, int64_t lv, bool live, int wg, int r, int warp, int lane,
                                float (&ks)[K], int (&kj)[K], float& thr, int& cnt, const float2* mybuf,
                                float4* mystage, float2 rn, const float (&slb)[SLB_CHUNKS], int64_t vt, float& thr0,
                                int& n_steps) {
    merge_buffer<K, MB>(ks, kj, thr, cnt, mybuf, 3.0e38f);
    const uint32_t par = (uint32_t)(lv & 1);
    if (wg == 1) {
#pragma unroll
        for (int q = 0; q < K / 4; ++q)
            mystage[q * EPI_THREADS] = make_float4(ks[4 * q], ks[4 * q + 1], ks[4 * q + 2], ks[4 * q + 3]);
        __syncwarp();
        if (lane == 0) mbar_arrive(&S.lfull);
        if (!mbar_wait_warp(&S.lempty, par, lane)) return false;
        n_steps = S.vsteps[par];
        thr0 = S.thr0[r];
        thr = fminf(thr, thr0);
        return true;
    }
    if (!mbar_wait_warp(&S.lfull, par, lane)) return false;
    // k-th smallest of the union of the two ascending lists: min over i of max(ks[i - 1], other[k - 1 - i])
    const float* other = reinterpret_cast<const float*>(&S.stage[0][TILE_M + r]);
    float t = 3.0e38f;
#pragma unroll
    for (int i = 0; i <= K; ++i) {
        const int j = K - 1 - i;
        const float a = i > 0 ? ks[i - 1] : -3.0e38f;
        const float b = i < K ? other[(j >> 2) * (EPI_THREADS * 4) + (j & 3)] : -3.0e38f;
        t = fminf(t, fmaxf(a, b));
    }
    const float lm = __ldg(P.lmax);
    float rb = 0.f;
    thr0 = 3.0e38f;
    if (live) {
        thr0 = t + fmaxf(fabsf(t) * 1e-6f, 1e-12f);
        const float r2 = t + rn.x + 1e-5f * (1.f + rn.x + lm * lm);
        rb = sqrtf(fmaxf(r2, 0.f)) * (1.f + 1e-5f) + U_BF16 * rn.y;
        rb = rb < 3.0e38f ? rb : 3.0e38f;
    }
    S.thr0[r] = thr0;
    thr = fminf(thr, thr0);
    return publish_steps(S, P, par, warp, lane, rb, lm, slb, vt, n_steps);
}

// first_step_bounds for the packed top-k: the union of the two halves' lists
// is taken on words, the row's bound thr0 is the union's k-th word, and the
// residual bound is sqrt(2 d) at the top of that word's quantum.
template <int K, int MB>
MADI_DEV bool first_step_bounds_pk(Smem& S, const Plan& P, int64_t lv, bool live, int wg, int r, int warp, int lane,
                                   uint32_t (&ks)[K], uint32_t& thr, int& cnt, const uint32_t* mybuf,
                                   float4* mystage, float2 rn, const float (&slb)[SLB_CHUNKS], int64_t vt,
                                   uint32_t& thr0, int& n_steps) {
    merge_buffer_u<K, MB>(ks, thr, cnt, mybuf, PK_EMPTY);
    const uint32_t par = (uint32_t)(lv & 1);
    if (wg == 1) {
        uint4* st4 = reinterpret_cast<uint4*>(mystage);
#pragma unroll
        for (int q = 0; q < K / 4; ++q) st4[q * EPI_THREADS] = make_uint4(ks[4 * q], ks[4 * q + 1], ks[4 * q + 2], ks[4 * q + 3]);
        __syncwarp();
        if (lane == 0) mbar_arrive(&S.lfull);
        if (!mbar_wait_warp(&S.lempty, par, lane)) return false;
        n_steps = S.vsteps[par];
        thr0 = __float_as_uint(S.thr0[r]);
        thr = min(thr, thr0);
        return true;
    }
    if (!mbar_wait_warp(&S.lfull, par, lane)) return false;
    // k-th smallest of the union of the two ascending lists: min over i of max(ks[i - 1], other[k - 1 - i])
    const uint32_t* other = reinterpret_cast<const uint32_t*>(&S.stage[0][TILE_M + r]);
    uint32_t t = PK_EMPTY;
#pragma unroll
    for (int i = 0; i <= K; ++i) {
        const int j = K - 1 - i;
        const uint32_t a = i > 0 ? ks[i - 1] : 0u;
        const uint32_t b = i < K ? other[(j >> 2) * (EPI_THREADS * 4) + (j & 3)] : 0u;
        t = min(t, max(a, b));
    }
    const float lm = __ldg(P.lmax);
    float rb = 0.f;
    thr0 = PK_EMPTY;
    if (live) {
        thr0 = t;
        const float dhi = t >= 0x7F800000u ? 3.0e38f : __uint_as_float(t | PK_MASK);
        const float r2 = fminf(2.f * dhi, 3.0e38f) + 1e-5f * (1.f + rn.x + lm * lm);
        rb = sqrtf(r2) * (1.f + 1e-5f) + U_BF16 * rn.y;
        rb = rb < 3.0e38f ? rb : 3.0e38f;
    }
    S.thr0[r] = __uint_as_float(thr0);
    thr = min(thr, thr0);
    return publish_steps(S, P, par, warp, lane, rb, lm, slb, vt, n_steps);
}

// Epilogue warps with the packed top-k (fixed S0, scans of at most 2^PK_BITS
// positions): the same steps, hand-offs and scan cut as the kernel's float
// epilogue, on packed words.
template <int K, int MODE>
MADI_DEV void epilogue_pk(Smem& S, const Plan& P, int tid, int warp, int lane, int64_t my_vt, uint32_t tmem) {
    constexpr int MB = K < 16 ? K : 16;
    static_assert(MODE != MODE_FREE, "the packed top-k is for fixed S0");
    const int n_tiles = P.n_tiles;
    const int wg = warp >> 2;                        // column half
    const int r = tid & (TILE_M - 1);                // voxel row = TMEM lane
    uint32_t* mybuf = reinterpret_cast<uint32_t*>(&S.buf[0][0]) + tid;
    float4* mystage = &S.stage[0][tid];
    const float* mystage_f = reinterpret_cast<const float*>(mystage);
    int64_t g = 0;
    bool ok = true;
    if (wg == 0 && my_vt > 0) write_voxel_tile<MODE>(S, P, blockIdx.x, 0, r, lane);
    if (P.test_stall && my_vt > 0 && !mbar_wait_warp(&S.never, 0, lane, STALL_POLLS)) {
        S.err = ERR_TIMEOUT;    // tests only: the wait runs out like any other would
        ok = false;
    }
    for (int64_t lv = 0; lv < my_vt && ok; ++lv) {
        const int64_t vt = blockIdx.x + lv * gridDim.x;
        const bool dyn = dynamic_steps(P);
        int n_steps = dyn ? 2 : full_steps(P);
        const int64_t pos = vt * TILE_M + r;
        uint32_t ks[K];
#pragma unroll
        for (int i = 0; i < K; ++i) ks[i] = PK_EMPTY;
        uint32_t thr0 = PK_EMPTY, thr = PK_EMPTY;
        float2 rn = make_float2(0.f, 0.f);
        if (pos < P.n_vox) rn = P.rownorm[pos];     // |m~|^2, |m - mu|: loaded now, used from the first pass
        float slb[SLB_CHUNKS];
#pragma unroll
        for (int c = 0; c < SLB_CHUNKS; ++c) slb[c] = 3.0e38f;
        if (dyn && warp == 0) {
            const int full = full_steps(P);
#pragma unroll
            for (int c = 0; c < SLB_CHUNKS; ++c)
                if (c * 32 + lane < full) slb[c] = P.steplb[vt * full + c * 32 + lane];
        }
        float hm2 = 0.f;                             // |m~|^2 / 2, set once rn has landed
        float tthr = -3.0e38f;
        int cnt = 0;
        auto my_tile = [&](int t) -> int {
            const int i = PAIR * t + wg;
            return i < n_tiles ? (int)P.order[vt * n_tiles + i] : n_tiles;
        };
        int lt_next = my_tile(0);
        for (int t = 0; t < n_steps; ++t, ++g) {
            const int acc = (int)(g % ACCS);
            const bool got = mbar_wait_warp(&S.accf[acc], (uint32_t)((g / ACCS) & 1), lane) &&
                             !__any_sync(0xffffffffu, err_flag_read(S) != 0);   // warp-uniform
            if (!got) { S.err = ERR_TIMEOUT; ok = false; break; }
            fence_after();
            if (t == 0) hm2 = 0.5f * rn.x;
            const int lt = lt_next;
            if (t + 1 < n_steps) lt_next = my_tile(t + 1);
            const uint32_t tbase = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(acc * MMA_N + wg * TILE_N);
#pragma unroll 1
            for (int c = 0; c < TILE_N; c += WG_COLS) {
                const uint32_t taddr = tbase + (uint32_t)c;
                const float* ax = S.aux[acc][wg] + c;
                const int jb = lt * TILE_N + c;
                float key[WG_COLS];
                tmem_ld64(taddr, key);
                if (MODE == MODE_AUX) {              // folded key t = m~.L~ - |L~|^2 / 2
#pragma unroll
                    for (int i = 0; i < WG_COLS; i += 4) {
                        const float4 q = *reinterpret_cast<const float4*>(ax + i);
                        const float qq[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                        for (int u = 0; u < 4; ++u) key[i + u] = fmaf(-0.5f, qq[u], key[i + u]);
                    }
                }
                uint32_t seeded = 0u;
                if (t == 0 && c == 0) {
                    uint32_t sk[K];
#pragma unroll
                    for (int i = 0; i < K; ++i) sk[i] = pk_word(hm2 - key[i], jb + i);
                    bitonic_sort_u<K>(sk);
#pragma unroll
                    for (int i = 0; i < K; ++i) ks[i] = sk[i];
                    thr = min(ks[K - 1], thr0);
                    tthr = pk_tthr(thr, hm2);
                    S.thr_pub[wg][r] = make_uint2((uint32_t)vt, thr);
                    seeded = K >= 32 ? 0xFFFFFFFFu : ((1u << K) - 1u);
                }
                const uint2 pp = S.thr_pub[wg ^ 1][r];
                const float tthr_e = fmaxf(tthr, pp.x == (uint32_t)vt ? pk_tthr(pp.y, hm2) : -3.0e38f);
                {
                    float ext[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) ext[i] = key[i];
#pragma unroll
                    for (int i = 8; i < WG_COLS; ++i) ext[i & 7] = fmaxf(ext[i & 7], key[i]);
#pragma unroll
                    for (int w = 4; w > 0; w >>= 1)
#pragma unroll
                        for (int i = 0; i < w; ++i) ext[i] = fmaxf(ext[i], ext[i + w]);
                    if (!__any_sync(0xffffffffu, ext[0] > tthr_e || seeded)) continue;
                }
                uint32_t mk[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
#pragma unroll
                for (int i = 0; i < WG_COLS; ++i)
                    if (key[i] > tthr_e) mk[i >> 3] |= 1u << (i & 7);
                uint32_t m0 = (mk[0] | (mk[1] << 8) | (mk[2] << 16) | (mk[3] << 24)) & ~seeded;
                uint32_t m1 = mk[4] | (mk[5] << 8) | (mk[6] << 16) | (mk[7] << 24);
                const int nh0 = __popc(m0), nh1 = __popc(m1);
                if (m0 | m1) {
#pragma unroll
                    for (int i = 0; i < WG_COLS; i += 4)
                        mystage[(i >> 2) * EPI_THREADS] = make_float4(key[i], key[i + 1], key[i + 2], key[i + 3]);
                }
                uint32_t* wp = mybuf + cnt * EPI_THREADS;
                if (!__any_sync(0xffffffffu, cnt + nh0 + nh1 > cap_pk<K>())) {
                    while (__any_sync(0xffffffffu, (m0 | m1) != 0u)) append_pass_u(m0, 0, m1, 32, wp, mystage_f, jb, hm2);
                    cnt += nh0 + nh1;
                } else {
                    uint32_t none = 0u;
                    if (__any_sync(0xffffffffu, cnt + nh0 > cap_pk<K>())) {
                        merge_buffer_u<K, MB>(ks, thr, cnt, mybuf, thr0);
                        tthr = pk_tthr(thr, hm2);
                        S.thr_pub[wg][r] = make_uint2((uint32_t)vt, thr);
                        wp = mybuf;
                    }
                    while (__any_sync(0xffffffffu, m0 != 0u)) append_pass_u(m0, 0, none, 0, wp, mystage_f, jb, hm2);
                    cnt += nh0;
                    if (__any_sync(0xffffffffu, cnt + nh1 > cap_pk<K>())) {
                        merge_buffer_u<K, MB>(ks, thr, cnt, mybuf, thr0);
                        tthr = pk_tthr(thr, hm2);
                        S.thr_pub[wg][r] = make_uint2((uint32_t)vt, thr);
                        wp = mybuf;
                    }
                    while (__any_sync(0xffffffffu, m1 != 0u)) append_pass_u(m1, 32, none, 0, wp, mystage_f, jb, hm2);
                    cnt += nh1;
                }
            }
            if (t == 0 && wg == 0 && lv + 1 < my_vt)
                write_voxel_tile<MODE>(S, P, vt + gridDim.x, (int)((lv + 1) & 1), r, lane);
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.acce[acc]);
            if (dyn && t == 0) {
                if (!first_step_bounds_pk<K, MB>(S, P, lv, pos < P.n_vox, wg, r, warp, lane, ks, thr, cnt, mybuf,
                                                 mystage, rn, slb, vt, thr0, n_steps)) {
                    S.err = ERR_TIMEOUT;
                    ok = false;
                    break;
                }
                tthr = pk_tthr(thr, hm2);
                S.thr_pub[wg][r] = make_uint2((uint32_t)vt, thr);
            }
        }
        if (!ok) break;
        merge_buffer_u<K, MB>(ks, thr, cnt, mybuf, thr0);
        S.thr_pub[wg][r] = make_uint2((uint32_t)vt, thr);
        const int64_t row = pos < P.n_vox ? P.vperm[pos] : -1;
        // The row's top-k is the k smallest words of the two halves' lists: both
        // halves keep only words up to the union's k-th word.
        const uint32_t epar = (uint32_t)(lv & 1);
        uint32_t cut = PK_EMPTY;
        if (wg == 1) {
            uint4* st4 = reinterpret_cast<uint4*>(mystage);
#pragma unroll
            for (int q = 0; q < K / 4; ++q) st4[q * EPI_THREADS] = make_uint4(ks[4 * q], ks[4 * q + 1], ks[4 * q + 2], ks[4 * q + 3]);
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.efull);
            if (!mbar_wait_warp(&S.eempty, epar, lane)) { S.err = ERR_TIMEOUT; ok = false; break; }
            cut = S.ucut[r];
        } else {
            if (!mbar_wait_warp(&S.efull, epar, lane)) { S.err = ERR_TIMEOUT; ok = false; break; }
            const uint32_t* other = reinterpret_cast<const uint32_t*>(&S.stage[0][TILE_M + r]);
#pragma unroll
            for (int i = 0; i <= K; ++i) {
                const int j = K - 1 - i;
                const uint32_t a = i > 0 ? ks[i - 1] : 0u;
                const uint32_t b = i < K ? other[(j >> 2) * (EPI_THREADS * 4) + (j & 3)] : 0u;
                cut = min(cut, max(a, b));
            }
            S.ucut[r] = cut;
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.eempty);
        }
        int nv = 0;
#pragma unroll
        for (int i = 0; i < K; ++i) nv += (ks[i] < 0x7F800000u && ks[i] <= cut) ? 1 : 0;
        if (row >= 0) {
            int4* cp = reinterpret_cast<int4*>(P.cand + (pos * EPI_WG + wg) * K);
#pragma unroll
            for (int i = 0; i < K; i += 4)
                cp[i / 4] = make_int4(i < nv ? (int)(ks[i] & PK_MASK) : -1, i + 1 < nv ? (int)(ks[i + 1] & PK_MASK) : -1,
                                      i + 2 < nv ? (int)(ks[i + 2] & PK_MASK) : -1,
                                      i + 3 < nv ? (int)(ks[i + 3] & PK_MASK) : -1);
        }
    }
}

// Epilogue warps with (score, index) candidates: free S0, and fixed S0 scans
// beyond 2^PK_BITS positions.  Same steps, hand-offs and scan cut as
// epilogue_pk; each half's candidates are those under the other half's k-th
// best.
template <int K, int MODE>
MADI_DEV void epilogue_f(Smem& S, const Plan& P, int tid, int warp, int lane, int64_t my_vt, uint32_t tmem) {
    constexpr int MB = K < 16 ? K : 16;             // merge batch
    static_assert(CAP % MB == 0 && CAP >= 32 && CAP >= K, "buffer holds whole merge batches, a chunk and the top-k");
    constexpr bool FREE = MODE == MODE_FREE;
    const int n_tiles = P.n_tiles;
    const int wg = warp >> 2;                    // column half
    const int r = tid & (TILE_M - 1);            // voxel row = TMEM lane
    const float2* mybuf = &S.buf[0][tid];
    float2* mybuf_w = &S.buf[0][tid];
    float4* mystage = &S.stage[0][tid];
    const float* mystage_f = reinterpret_cast<const float*>(mystage);
    int64_t g = 0;
    bool ok = true;
    if (wg == 0 && my_vt > 0) write_voxel_tile<MODE>(S, P, blockIdx.x, 0, r, lane);
    if (P.test_stall && my_vt > 0 && !mbar_wait_warp(&S.never, 0, lane, STALL_POLLS)) {
        S.err = ERR_TIMEOUT;    // tests only: the wait runs out like any other would
        ok = false;
    }
    for (int64_t lv = 0; lv < my_vt && ok; ++lv) {
        const int64_t vt = blockIdx.x + lv * gridDim.x;
        const bool dyn = MODE != MODE_FREE && dynamic_steps(P);   // the scan cut is for fixed S0
        int n_steps = dyn ? 2 : full_steps(P);   // under the scan cut: set after the first step
        const int64_t pos = vt * TILE_M + r;
        float ks[K];
        int kj[K];
#pragma unroll
        for (int i = 0; i < K; ++i) { ks[i] = 3.0e38f; kj[i] = 0; }
        float thr0 = 3.0e38f;                    // bound on the row's final k-th best (after the first step)
        float thr = thr0;
        // scan cut inputs, loaded now so that their latency hides behind the first step
        float2 rn = make_float2(0.f, 0.f);
        float slb[SLB_CHUNKS];
#pragma unroll
        for (int c = 0; c < SLB_CHUNKS; ++c) slb[c] = 3.0e38f;
        if (dyn) {
            if (pos < P.n_vox) rn = P.rownorm[pos];
            if (warp == 0) {
                const int full = full_steps(P);
#pragma unroll
                for (int c = 0; c < SLB_CHUNKS; ++c)
                    if (c * 32 + lane < full) slb[c] = P.steplb[vt * full + c * 32 + lane];
            }
        }
        float tthr = -0.5f * thr;                // fold mode: key t hits when t > -thr / 2
        int cnt = 0;
        // library tile of this warpgroup at step t (the padding tile past the end)
        auto my_tile = [&](int t) -> int {
            const int i = PAIR * t + wg;
            return i < n_tiles ? (int)P.order[vt * n_tiles + i] : n_tiles;
        };
        int lt_next = my_tile(0);
        for (int t = 0; t < n_steps; ++t, ++g) {
            const int acc = (int)(g % ACCS);
            const bool got = mbar_wait_warp(&S.accf[acc], (uint32_t)((g / ACCS) & 1), lane) &&
                             !__any_sync(0xffffffffu, err_flag_read(S) != 0);   // warp-uniform
            if (!got) { S.err = ERR_TIMEOUT; ok = false; break; }
            fence_after();
            const int lt = lt_next;
            if (t + 1 < n_steps) lt_next = my_tile(t + 1);   // prefetch the next step
            const uint32_t tbase = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(acc * MMA_N + wg * TILE_N);
#pragma unroll 1
            for (int c = 0; c < TILE_N; c += WG_COLS) {
                const uint32_t taddr = tbase + (uint32_t)c;
                const float* ax = S.aux[acc][wg] + c;
                const int jb = lt * TILE_N + c;
                float key[WG_COLS];
                tmem_ld64(taddr, key);
                if (MODE != MODE_FOLD) {
#pragma unroll
                    for (int i = 0; i < WG_COLS; i += 4) {
                        const float4 q = *reinterpret_cast<const float4*>(ax + i);
                        const float qq[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const float v = key[i + u];
                            key[i + u] = FREE ? (-v * fabsf(v)) * qq[u] : fmaf(-2.f, v, qq[u]);
                        }
                    }
                }
                uint32_t seeded = 0u;   // bits of this pass already in ks
            if (t == 0 && c == 0) {
                // seed the top-k with the pass's first K keys (the nearest tile):
                // a finite threshold from the start keeps the early tiles cheap
                float sk[K];
                int sj[K];
#pragma unroll
                for (int i = 0; i < K; ++i) {
                    const float sc = MODE == MODE_FOLD ? -2.f * key[i] : key[i];
                    sk[i] = sc < 3.0e38f ? sc : 3.0e38f;   // padding (inf / NaN) sorts last
                    sj[i] = jb + i;
                }
                bitonic_sort<K>(sk, sj);
#pragma unroll
                for (int i = 0; i < K; ++i) { ks[i] = sk[i]; kj[i] = sj[i]; }
                thr = fminf(ks[K - 1], thr0);
                tthr = -0.5f * thr;
                S.thr_pub[wg][r] = make_uint2((uint32_t)vt, __float_as_uint(thr));
                seeded = K >= 32 ? 0xFFFFFFFFu : ((1u << K) - 1u);
            }
            // An entry at or above the other half's k-th best of this row
                // cannot be in the row's overall top-k: filter with the tighter of
                // the two (a stale read is only looser).
                const uint2 pp = S.thr_pub[wg ^ 1][r];
                const float thr_e = fminf(thr, pp.x == (uint32_t)vt ? __uint_as_float(pp.y) : 3.0e38f);
                const float tthr_e = MODE == MODE_FOLD ? fmaxf(tthr, -0.5f * thr_e) : tthr;
                // fast path: no lane of the warp holds a candidate in this tile
                {
                    float ext[8];   // eight independent running extremes, then a tree
#pragma unroll
                    for (int i = 0; i < 8; ++i) ext[i] = key[i];
#pragma unroll
                    for (int i = 8; i < WG_COLS; ++i)
                        ext[i & 7] = MODE == MODE_FOLD ? fmaxf(ext[i & 7], key[i]) : fminf(ext[i & 7], key[i]);
#pragma unroll
                    for (int w = 4; w > 0; w >>= 1)
#pragma unroll
                        for (int i = 0; i < w; ++i)
                            ext[i] = MODE == MODE_FOLD ? fmaxf(ext[i], ext[i + w]) : fminf(ext[i], ext[i + w]);
                    const bool maybe = MODE == MODE_FOLD ? ext[0] > tthr_e : ext[0] < thr_e;
                    if (!__any_sync(0xffffffffu, maybe || seeded)) continue;   // nothing for this warp here
                }
                // eight independent 8-bit masks, then two 32-bit masks
                uint32_t mk[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
#pragma unroll
                for (int i = 0; i < WG_COLS; ++i) {
                    const bool hit = MODE == MODE_FOLD ? key[i] > tthr_e : key[i] < thr_e;
                    if (hit) mk[i >> 3] |= 1u << (i & 7);
                }
                uint32_t m0 = (mk[0] | (mk[1] << 8) | (mk[2] << 16) | (mk[3] << 24)) & ~seeded;
                uint32_t m1 = mk[4] | (mk[5] << 8) | (mk[6] << 16) | (mk[7] << 24);
                const int nh0 = __popc(m0), nh1 = __popc(m1);
                if (m0 | m1) {   // stage the keys for the append passes (lanes with hits only)
#pragma unroll
                    for (int i = 0; i < WG_COLS; i += 4)
                        mystage[(i >> 2) * EPI_THREADS] = make_float4(key[i], key[i + 1], key[i + 2], key[i + 3]);
                }
                float2* wp = mybuf_w + cnt * EPI_THREADS;
                if (!__any_sync(0xffffffffu, cnt + nh0 + nh1 > CAP)) {
                    while (__any_sync(0xffffffffu, (m0 | m1) != 0u)) append_pass<MODE>(m0, 0, m1, 32, wp, mystage_f, jb);
                    cnt += nh0 + nh1;
                } else {
                    // fold before each half as needed, then append it
                    uint32_t none = 0u;
                    if (__any_sync(0xffffffffu, cnt + nh0 > CAP)) {
                        merge_buffer<K, MB>(ks, kj, thr, cnt, mybuf, thr0);
                        tthr = -0.5f * thr;
                        S.thr_pub[wg][r] = make_uint2((uint32_t)vt, __float_as_uint(thr));
                        wp = mybuf_w;
                    }
                    while (__any_sync(0xffffffffu, m0 != 0u)) append_pass<MODE>(m0, 0, none, 0, wp, mystage_f, jb);
                    cnt += nh0;
                    if (__any_sync(0xffffffffu, cnt + nh1 > CAP)) {
                        merge_buffer<K, MB>(ks, kj, thr, cnt, mybuf, thr0);
                        tthr = -0.5f * thr;
                        S.thr_pub[wg][r] = make_uint2((uint32_t)vt, __float_as_uint(thr));
                        wp = mybuf_w;
                    }
                    while (__any_sync(0xffffffffu, m1 != 0u)) append_pass<MODE>(m1, 32, none, 0, wp, mystage_f, jb);
                    cnt += nh1;
                }
            }
            // After the first step, the next voxel tile's A goes into the other
            // buffer: its last reader, the previous voxel tile's MMAs, completed
            // before this tile's first step did, and the producer has already
            // waited on this tile's afull phase, so afull never runs two phases
            // ahead of its waiter.
            if (t == 0 && wg == 0 && lv + 1 < my_vt)
                write_voxel_tile<MODE>(S, P, vt + gridDim.x, (int)((lv + 1) & 1), r, lane);
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.acce[acc]);
            if (dyn && t == 0 && !first_step_bounds<K, MB>(S, P, lv, pos < P.n_vox, wg, r, warp, lane, ks, kj, thr,
                                                           cnt, mybuf, mystage, rn, slb, vt, thr0, n_steps)) {
                S.err = ERR_TIMEOUT;
                ok = false;
                break;
            }
            if (dyn && t == 0) {
                tthr = -0.5f * thr;
                S.thr_pub[wg][r] = make_uint2((uint32_t)vt, __float_as_uint(thr));
            }
        }
        if (!ok) break;
        merge_buffer<K, MB>(ks, kj, thr, cnt, mybuf, thr0);
        S.thr_pub[wg][r] = make_uint2((uint32_t)vt, __float_as_uint(thr));
        const int64_t row = pos < P.n_vox ? P.vperm[pos] : -1;
        // Candidates above the other half's k-th best cannot be in the row's
        // overall top-k; ks is ascending, so the rest is a prefix of length nv
        // (a stale partner value only keeps more).
        const uint2 pp = S.thr_pub[wg ^ 1][r];
        const float cut = fminf(3.0e38f, pp.x == (uint32_t)vt ? __uint_as_float(pp.y) : 3.0e38f);
        int nv = 0;
#pragma unroll
        for (int i = 0; i < K; ++i) nv += (ks[i] < 3.0e38f && ks[i] <= cut) ? 1 : 0;
        // candidates (scan positions, ascending BF16 score) for the rescore kernel
        if (row >= 0) {
            int4* c = reinterpret_cast<int4*>(P.cand + (pos * EPI_WG + wg) * K);
#pragma unroll
            for (int i = 0; i < K; i += 4)
                c[i / 4] = make_int4(i < nv ? kj[i] : -1, i + 1 < nv ? kj[i + 1] : -1, i + 2 < nv ? kj[i + 2] : -1,
                                     i + 3 < nv ? kj[i + 3] : -1);
        }
    }
}

template <int K, int MODE, bool PK>
__global__ void __launch_bounds__(THREADS, 1) match_bf16_kernel(const Plan P) {
    static_assert(!PK || MODE != MODE_FREE, "packed candidates are for fixed S0");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    Smem& S = *reinterpret_cast<Smem*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int i = 0; i < STAGES; ++i) mbar_init(&S.full[i], 1);
        for (int i = 0; i < ACCS; ++i) {
            mbar_init(&S.accf[i], MODE == MODE_FOLD ? 1 : 2);
            mbar_init(&S.acce[i], EPI_WARPS);
        }
        mbar_init(&S.afull, 4);
        mbar_init(&S.lfull, 4);
        mbar_init(&S.lempty, 4);
        mbar_init(&S.rfull, 4);
        mbar_init(&S.vready, 1);
        mbar_init(&S.efull, 4);
        mbar_init(&S.eempty, 4);
        mbar_init(&S.drain, 1);
        mbar_init(&S.never, 1);
        S.n_loaded = 0;
        S.n_issued = 0;
        S.err = 0;
    }
    if (tid < EPI_THREADS) {
        S.thr_pub[tid / TILE_M][tid % TILE_M] = make_uint2(0xFFFFFFFFu, 0u);
    }
    if (tid == 0) {
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
    const int64_t n_vtiles = (P.n_vox + TILE_M - 1) / TILE_M;
    const int64_t my_vt = (int64_t)blockIdx.x < n_vtiles ? (n_vtiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;

    if (warp == EPI_WARPS) {
        producer<MODE>(S, P, my_vt, tmem, lane);
    } else if constexpr (PK) {
        epilogue_pk<K, MODE>(S, P, tid, warp, lane, my_vt, tmem);
    } else {
        epilogue_f<K, MODE>(S, P, tid, warp, lane, my_vt, tmem);
    }
    // ---- teardown: after an error, drain what the producer issued first ----
    fence_before();
    __syncthreads();
    fence_after();
    if (S.err) {
        if (warp == EPI_WARPS && lane == 0 && !drain_issued(S)) S.err = ERR_DRAIN;
        fence_before();
        __syncthreads();
        fence_after();
    }
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(TMEM_COLS) : "memory");
    }
    if (tid == 0 && S.err) atomicMax(P.err, S.err);
}

}  // namespace bf16m
}  // namespace madi

using namespace madi;
using namespace madi::bf16m;

static int64_t round256(int64_t x) { return (x + 255) & ~int64_t(255); }

namespace {
// Scratch layout of the BF16 path (every part 256-byte aligned).
struct Layout {
    int64_t tiles, aux, mu, err, kmu, pc, cov, lkey, lperm, krange, tlo, thi;
    int64_t lrows, vkey, vb, vrank, cnt, offs, vtot, vperm, order, lmax, cand;
    int64_t lvb, lvrank, lcnt, loffs, ltot, steplb, rownorm, total;
};

Layout layout(int64_t n_vox, int64_t n_lib, int topk) {
    const int64_t n_tiles = (n_lib + TILE_N - 1) / TILE_N;
    const int64_t n_pad = PAIR * ((n_tiles + PAIR - 1) / PAIR);   // + the all-padding tile when odd
    const int64_t n_vtiles = (n_vox + TILE_M - 1) / TILE_M;
    const int64_t nblk = (n_vox + VBLK - 1) / VBLK;
    Layout L{};
    int64_t off = 0;
    auto take = [&](int64_t bytes) { const int64_t o = off; off += round256(bytes); return o; };
    L.tiles = take(n_pad * B_BYTES);
    L.aux = take(n_pad * TILE_N * 4);
    L.mu = take(KPAD * 4);
    L.err = take(4);
    L.kmu = take(KPAD * 4);
    L.pc = take(KPAD * 4);
    L.cov = take(KPAD * KPAD * 4);
    L.lkey = take(n_lib * 4);
    L.lperm = take(n_lib * 4);
    L.krange = take(8);
    L.tlo = take(n_tiles * 4);
    L.thi = take(n_tiles * 4);
    L.lrows = take(n_lib * KPAD * 4);
    L.vkey = take(n_vox * 4);
    L.vb = take(n_vox);
    L.vrank = take(n_vox * 2);
    L.cnt = take(nblk * NBUCKET * 4);
    L.offs = take(nblk * NBUCKET * 4);
    L.vtot = take(NBUCKET * 4);
    L.vperm = take(n_vox * 4);
    L.order = take(n_vtiles * n_tiles * 2);
    L.lmax = take(4);
    L.cand = take(n_vox * EPI_WG * topk * 4);
    const int64_t lnblk = (n_lib + VBLK - 1) / VBLK;
    L.lvb = take(n_lib);
    L.lvrank = take(n_lib * 2);
    L.lcnt = take(lnblk * NBUCKET * 4);
    L.loffs = take(lnblk * NBUCKET * 4);
    L.ltot = take(NBUCKET * 4);
    L.steplb = take(n_vtiles * (n_pad / PAIR) * 4);
    L.rownorm = take(n_vox * 8);
    L.total = off;
    return L;
}

unsigned blocks_for(int64_t n, int per) { return (unsigned)((n + per - 1) / per); }
}  // namespace

int64_t madi_match_bf16_scratch(int64_t n_vox, int32_t n_lib, int32_t n_feat, int32_t topk) {
    (void)n_feat;
    return layout(n_vox, n_lib, topk).total;
}

// Device address of the status word madi_match_bf16 left in the scratch.
const int* madi_match_bf16_status_word(const madi_match_desc* d) {
    return reinterpret_cast<const int*>(static_cast<const unsigned char*>(d->scratch) +
                                        layout(d->n_vox, d->n_lib, d->topk).err);
}

// Library column means (fp64 sums), shared with the fp32 fixed-S0 scan.
void madi_match_column_mean(const float* lib, int32_t n_lib, int32_t n_feat, float* mu, cudaStream_t s) {
    column_mean_kernel<<<n_feat, 256, 0, s>>>(lib, n_lib, n_feat, mu);
}

madi_status madi_match_bf16(const madi_match_desc* d, cudaStream_t s) {
    if (d->topk != 8 && d->topk != 16 && d->topk != 32)
        return host::fail(MADI_ERR_UNSUPPORTED, "match bf16: topk must be 8, 16 or 32");
    const int64_t n_tiles64 = ((int64_t)d->n_lib + TILE_N - 1) / TILE_N;
    if (d->n_vox >= (int64_t(1) << 31) || n_tiles64 > 65535)
        return host::fail(MADI_ERR_UNSUPPORTED, "match bf16: at most 2^31-1 voxels and 65535 library tiles");
    const Layout Ly = layout(d->n_vox, d->n_lib, d->topk);
    if (!d->scratch || d->scratch_bytes < Ly.total)
        return host::fail(MADI_ERR_CAPACITY, "match bf16: scratch %lld < %lld bytes", (long long)d->scratch_bytes,
                          (long long)Ly.total);
    if ((reinterpret_cast<uintptr_t>(d->scratch) & 255) != 0)
        return host::fail(MADI_ERR_INVALID, "match bf16: scratch must be 256-byte aligned");
    unsigned char* base = static_cast<unsigned char*>(d->scratch);
    auto at = [&](int64_t off) { return base + off; };
    const int n_tiles = (int)n_tiles64;
    const int64_t n_vox = d->n_vox, n_vtiles = (n_vox + TILE_M - 1) / TILE_M, nblk = (n_vox + VBLK - 1) / VBLK;
    const int n_lib = d->n_lib, F = d->n_feat;
    const bool free_s0 = d->mode == MADI_MATCH_FREE_S0;
    const int mode = free_s0 ? MODE_FREE : (F + BIAS_COLS <= KPAD ? MODE_FOLD : MODE_AUX);
    const int unit = free_s0 ? 1 : 0;
    float* mu = reinterpret_cast<float*>(at(Ly.mu));
    float* kmu = reinterpret_cast<float*>(at(Ly.kmu));
    float* pc = reinterpret_cast<float*>(at(Ly.pc));
    float* cov = reinterpret_cast<float*>(at(Ly.cov));
    float* lkey = reinterpret_cast<float*>(at(Ly.lkey));
    int32_t* lperm = reinterpret_cast<int32_t*>(at(Ly.lperm));
    float* krange = reinterpret_cast<float*>(at(Ly.krange));
    float* tlo = reinterpret_cast<float*>(at(Ly.tlo));
    float* thi = reinterpret_cast<float*>(at(Ly.thi));
    float* vkey = reinterpret_cast<float*>(at(Ly.vkey));
    uint8_t* vb = reinterpret_cast<uint8_t*>(at(Ly.vb));
    uint16_t* vrank = reinterpret_cast<uint16_t*>(at(Ly.vrank));
    uint32_t* cnt = reinterpret_cast<uint32_t*>(at(Ly.cnt));
    uint32_t* offs = reinterpret_cast<uint32_t*>(at(Ly.offs));
    int32_t* vperm = reinterpret_cast<int32_t*>(at(Ly.vperm));
    uint16_t* order = reinterpret_cast<uint16_t*>(at(Ly.order));
    int* err = reinterpret_cast<int*>(at(Ly.err));

    float* lmax = reinterpret_cast<float*>(at(Ly.lmax));
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(lmax, 0, sizeof(float), s);
    if (e != cudaSuccess) return host::cuda_fail(e, "match bf16 memset");
    if (!free_s0) column_mean_kernel<<<F, 256, 0, s>>>(d->lib, n_lib, F, mu);
    // ---- scan order: library and voxels bucketed along the library's principal axis ----
    // (fixed S0 keys rows as they are, so their mean is the column mean)
    const float* kmean = unit ? kmu : mu;
    if (unit) key_mean_kernel<<<F, 256, 0, s>>>(d->lib, n_lib, F, unit, kmu);
    key_cov_kernel<<<F * F, 256, 0, s>>>(d->lib, n_lib, F, unit, kmean, cov);
    key_axis_kernel<<<1, 32, 0, s>>>(cov, F, pc);
    key_kernel<<<blocks_for(n_lib, 256), 256, 0, s>>>(d->lib, n_lib, F, unit, kmean, pc, lkey);
    key_range_kernel<<<1, 1024, 0, s>>>(lkey, n_lib, krange);
    {
        const int64_t lnblk = (n_lib + VBLK - 1) / VBLK;
        uint8_t* lvb = reinterpret_cast<uint8_t*>(at(Ly.lvb));
        uint16_t* lvrank = reinterpret_cast<uint16_t*>(at(Ly.lvrank));
        uint32_t* lcnt = reinterpret_cast<uint32_t*>(at(Ly.lcnt));
        uint32_t* loffs = reinterpret_cast<uint32_t*>(at(Ly.loffs));
        uint32_t* ltot = reinterpret_cast<uint32_t*>(at(Ly.ltot));
        key_bucket_kernel<<<blocks_for(n_lib, 256), 256, 0, s>>>(lkey, n_lib, krange, lvb);
        vox_rank_kernel<<<(unsigned)lnblk, VBLK, 0, s>>>(lvb, n_lib, lvrank, lcnt);
        vox_scan_kernel<<<NBUCKET, 1024, 0, s>>>(lcnt, (int)lnblk, loffs, ltot);
        vox_base_kernel<<<1, 32, 0, s>>>(ltot);
        vox_scatter_kernel<<<blocks_for(n_lib, 256), 256, 0, s>>>(lvb, lvrank, loffs, ltot, n_lib, (int)lnblk, lperm);
    }
    tile_bounds_kernel<<<blocks_for(n_tiles, 128), 128, 0, s>>>(lkey, lperm, n_lib, n_tiles, tlo, thi);
    vox_bucket_kernel<<<blocks_for(n_vox, 256), 256, 0, s>>>(d->measured, n_vox, F, unit, kmean, pc, krange, vkey, vb);
    vox_rank_kernel<<<(unsigned)nblk, VBLK, 0, s>>>(vb, n_vox, vrank, cnt);
    uint32_t* vtot = reinterpret_cast<uint32_t*>(at(Ly.vtot));
    vox_scan_kernel<<<NBUCKET, 1024, 0, s>>>(cnt, (int)nblk, offs, vtot);
    vox_base_kernel<<<1, 32, 0, s>>>(vtot);
    vox_scatter_kernel<<<blocks_for(n_vox, 256), 256, 0, s>>>(vb, vrank, offs, vtot, n_vox, (int)nblk, vperm);
    order_kernel<<<blocks_for(n_vtiles, 128), 128, 0, s>>>(vkey, vperm, n_vox, n_vtiles, tlo, thi, n_tiles, order);
    const int n_pad = PAIR * ((n_tiles + PAIR - 1) / PAIR);
    pack_library_kernel<<<blocks_for((int64_t)n_pad * TILE_N, 256), 256, 0, s>>>(
        d->lib, n_lib, F, n_pad, mode, mu, lperm, reinterpret_cast<unsigned char*>(at(Ly.tiles)),
        reinterpret_cast<float*>(at(Ly.aux)), reinterpret_cast<float*>(at(Ly.lrows)), lmax);
    e = cudaGetLastError();
    if (e != cudaSuccess) return host::cuda_fail(e, "match bf16 preparation");

    Plan P{};
    P.meas = d->measured;
    P.lib = d->lib;
    P.n_vox = n_vox;
    P.n_lib = n_lib;
    P.F = F;
    P.n_tiles = n_tiles;
    P.tiles = reinterpret_cast<const unsigned char*>(at(Ly.tiles));
    P.aux = reinterpret_cast<const float*>(at(Ly.aux));
    P.mu = mu;
    P.vperm = vperm;
    P.lperm = lperm;
    P.lrows = reinterpret_cast<const float*>(at(Ly.lrows));
    P.order = order;
    P.steplb = reinterpret_cast<const float*>(at(Ly.steplb));
    P.rownorm = reinterpret_cast<const float2*>(at(Ly.rownorm));
    P.lmax = free_s0 ? nullptr : lmax;
    P.cand = reinterpret_cast<int32_t*>(at(Ly.cand));
    P.best_idx = d->best_idx;
    P.best_resid = d->best_resid;
    P.best_s0 = d->best_s0;
    P.err = err;
    P.test_stall = (d->flags & MADI_MATCH_FLAG_TEST_STALL) ? 1 : 0;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t smem = sizeof(Smem);
    // one CTA per SM: it allocates all 512 TMEM columns
    const int grid = (int)std::min<int64_t>(n_vtiles, (int64_t)sms);
    // fixed S0 scans of at most 2^PK_BITS positions keep packed one-word candidates
    const bool packed = mode != MODE_FREE && (int64_t)n_pad * TILE_N <= (int64_t(1) << PK_BITS);
#define MADI_LAUNCH_BF16(KK, MD, PKV)                                                                     \
    do {                                                                                                  \
        auto k = match_bf16_kernel<KK, MD, PKV>;                                                          \
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);             \
        if (e != cudaSuccess) return host::cuda_fail(e, "match bf16 attribute");                          \
        k<<<grid, THREADS, smem, s>>>(P);                                                                 \
    } while (0)
#define MADI_LAUNCH_BF16_K(MD, PKV)                                                                       \
    do {                                                                                                  \
        if (d->topk == 8) MADI_LAUNCH_BF16(8, MD, PKV);                                                   \
        else if (d->topk == 16) MADI_LAUNCH_BF16(16, MD, PKV);                                            \
        else MADI_LAUNCH_BF16(32, MD, PKV);                                                               \
    } while (0)
#define MADI_LAUNCH_BF16_ALL()                                                                            \
    do {                                                                                                  \
        if (mode == MODE_FOLD && packed) MADI_LAUNCH_BF16_K(MODE_FOLD, true);                             \
        else if (mode == MODE_FOLD) MADI_LAUNCH_BF16_K(MODE_FOLD, false);                                 \
        else if (mode == MODE_AUX && packed) MADI_LAUNCH_BF16_K(MODE_AUX, true);                          \
        else if (mode == MODE_AUX) MADI_LAUNCH_BF16_K(MODE_AUX, false);                                   \
        else MADI_LAUNCH_BF16_K(MODE_FREE, false);                                                        \
    } while (0)
    // Fixed S0: each voxel tile's scan stops where the principal-axis bound
    // rules out every later library tile (decided after its first step).
    P.cut = (!free_s0 && !(d->flags & MADI_MATCH_FLAG_FULL_SCAN)) ? 1 : 0;
    const bool dyn = P.cut && (n_tiles + PAIR - 1) / PAIR > 2;
    if (dyn)
        steplb_kernel<<<blocks_for(n_vtiles * 32, 256), 256, 0, s>>>(vkey, vperm, n_vox, n_vtiles, tlo, thi, order, n_tiles,
                                                                     const_cast<float*>(P.steplb));
    if (dyn || packed)
        row_norm_kernel<<<blocks_for(n_vox, 256), 256, 0, s>>>(d->measured, vperm, n_vox, F, mu,
                                                               const_cast<float2*>(P.rownorm));
    // rows of CTAs that give up on a bounded wait keep no candidates (-1)
    e = cudaMemsetAsync(P.cand, 0xFF, (size_t)n_vox * EPI_WG * d->topk * sizeof(int32_t), s);
    if (e != cudaSuccess) return host::cuda_fail(e, "match bf16 memset");
    MADI_LAUNCH_BF16_ALL();
#undef MADI_LAUNCH_BF16_ALL
    // 16-byte chunks of a library row the rescore reads: ceil(F / 4), rounded up to an instantiated size
#define MADI_RESCORE(KK, FR)                                                                              \
    do {                                                                                                  \
        const unsigned rb = blocks_for(2 * n_vox, 256);                                                   \
        if (F <= 8) rescore_kernel<KK, FR, 2><<<rb, 256, 0, s>>>(P);                                      \
        else if (F <= 12) rescore_kernel<KK, FR, 3><<<rb, 256, 0, s>>>(P);                                \
        else if (F <= 20) rescore_kernel<KK, FR, 5><<<rb, 256, 0, s>>>(P);                                \
        else if (F <= 24) rescore_kernel<KK, FR, 6><<<rb, 256, 0, s>>>(P);                                \
        else rescore_kernel<KK, FR, KPAD / 4><<<rb, 256, 0, s>>>(P);                                      \
    } while (0)
#define MADI_RESCORE_K(FR)                                                                                \
    do {                                                                                                  \
        if (d->topk == 8) MADI_RESCORE(8, FR);                                                            \
        else if (d->topk == 16) MADI_RESCORE(16, FR);                                                     \
        else MADI_RESCORE(32, FR);                                                                        \
    } while (0)
    if (free_s0) MADI_RESCORE_K(true);
    else MADI_RESCORE_K(false);
#undef MADI_RESCORE_K
#undef MADI_RESCORE
#undef MADI_LAUNCH_BF16_K
#undef MADI_LAUNCH_BF16
    e = cudaGetLastError();
    if (e != cudaSuccess) return host::cuda_fail(e, "match bf16 launch");
    return MADI_OK;
}
