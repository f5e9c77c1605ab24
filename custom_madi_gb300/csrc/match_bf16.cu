// BF16 tensor-core library match (tcgen05 / TMEM), replacing the one-thread-per-
// voxel fp64 scan of _map_kernel_fixed / _map_kernel_free_s0
// (madi/fitters_gpu.py:96-154).
//
// Per CTA (128 threads, one per voxel row = one TMEM lane; two CTAs per SM)
// and voxel tile of 128: the voxels are converted to BF16 in shared memory
// (K = features padded to 32, K-major, no-swizzle UMMA layout); the library,
// pre-packed once into 8 KB tiles of 128 entries in the same layout, streams
// through three shared stages by cp.async.bulk; one thread issues tcgen05.mma
// (M=128, N=128, K=16, two per tile) into one of two 128-column FP32 TMEM
// accumulators, so the MMA of tile t overlaps the epilogue of tile t-1.  The
// epilogue reads the scores with tcgen05.ld; scores under the thread's current
// k-th best are appended to a shared buffer, which the warp folds into a sorted
// register top-k with bitonic networks when any lane's buffer fills.  The k
// candidates are rescored in fp32 from the fp32 data and the best (lowest
// index on ties) is written.
//
//   fixed S0: score_j = |L~_j|^2 - 2 m~.L~_j  (= |m~ - L~_j|^2 - |m~|^2)
//   free  S0: score_j = -(m.r~_j)^2 / |r~_j|^2 when m.r~_j > 0
// with m~ = bf16(m - mu), L~_j = bf16(L_j - mu) (mu the library column mean:
// centring keeps the BF16 products small) and r~_j = bf16(r_j).
#include <cstdint>
#include <cuda_bf16.h>
#include "madi_device.cuh"
#include "madi_host.h"

namespace madi {
namespace bf16m {

constexpr int TILE_M = 128;                     // voxels per tile (MMA M, TMEM lanes)
constexpr int TILE_N = 128;                     // library entries per tile (MMA N)
constexpr int KPAD = 32;                        // features padded to 32 (two K=16 MMAs)
constexpr int CORE = 128;                       // bytes of one 8x8 BF16 core matrix
constexpr int SBO = (KPAD / 8) * CORE;          // 512 B between 8-row groups
constexpr int LBO = CORE;                       // 128 B between K-adjacent core matrices
constexpr int A_BYTES = TILE_M * KPAD * 2;      // 8 KB
constexpr int B_BYTES = TILE_N * KPAD * 2;      // 8 KB
constexpr int AUX_BYTES = TILE_N * 4;           // per-entry |L~|^2 (fixed) or 1/|r~|^2 (free)
constexpr int STAGES = 3;                       // library tiles in flight
constexpr int ACCS = 2;                         // TMEM accumulators (MMA t || epilogue t-1)
constexpr int TMEM_COLS = ACCS * TILE_N;        // 256: two CTAs share an SM's 512 columns
constexpr int CAP = 64;                         // per-thread candidate buffer entries
constexpr uint32_t SPIN_LIMIT = 1u << 22;       // bounded waits (~0.1-1 s)

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

__global__ void pack_library_kernel(const float* lib, int n_lib, int F, int n_tiles, int free_s0, const float* mu,
                                    unsigned char* tiles, float* aux) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)n_tiles * TILE_N) return;
    const int t = (int)(e / TILE_N), n = (int)(e % TILE_N);
    unsigned char* tile = tiles + (size_t)t * B_BYTES;
    float q = 0.f;
    for (int k = 0; k < KPAD; ++k) {
        float x = 0.f;
        if (e < n_lib && k < F) {
            const float v = lib[e * F + k];
            x = free_s0 ? v : v - mu[k];
        }
        const __nv_bfloat16 xb = __float2bfloat16_rn(x);
        const float xr = __bfloat162float(xb);
        q = fmaf(xr, xr, q);
        *reinterpret_cast<__nv_bfloat16*>(tile + canon_off(n, k)) = xb;
    }
    // The norm is taken of the ROUNDED entry, so the fixed-S0 score is exactly
    // |m~ - L~|^2 - |m~|^2 of the rounded vectors: its error then scales with the
    // residual |m - L| rather than with |m - mu| |L - mu|, and near-ties keep
    // their order (free S0 likewise scores the rounded pair, through 1/|r~|^2).
    // Padding entries carry NaN: their score fails every "<" test.
    aux[e] = e < n_lib ? (free_s0 ? 1.f / fmaxf(q, 1e-30f) : q) : __int_as_float(0x7fc00000);
}

// ---------------------------------------------------------------------------
// Per-thread top-K: sorted registers + a shared-memory append buffer that is
// merged warp-synchronously by bitonic networks (no serial insertion chains,
// no divergence inside the merge).
// ---------------------------------------------------------------------------
template <int K>
MADI_DEV void cswap(float (&a)[K], int (&ai)[K], int i, int l) {   // ascending at (i, l), i < l
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
// K at a time; every lane of the warp takes part.  Buffer entry e of thread
// tid lives at buf[e * TILE_M].
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
            if (base + i < cnt) e = buf[(base + i) * TILE_M];
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
// Main kernel.
// ---------------------------------------------------------------------------
struct Smem {
    unsigned char a[A_BYTES];
    unsigned char b[STAGES][B_BYTES];
    float aux[STAGES][TILE_N];
    float2 buf[CAP][TILE_M];
    uint64_t bar_load[STAGES];
    uint64_t bar_mma[ACCS];
    uint32_t tmem_base;
    int err;
};

template <int K, bool FREE>
__global__ void __launch_bounds__(128, 2) match_bf16_kernel(const float* __restrict__ meas, const float* __restrict__ lib,
                                                            int64_t n_vox, int n_lib, int F,
                                                            const unsigned char* __restrict__ tiles,
                                                            const float* __restrict__ aux, const float* __restrict__ mu,
                                                            int n_tiles, int32_t* best_idx, float* best_resid,
                                                            float* best_s0, int* err_flag) {
    static_assert(CAP % K == 0 && CAP >= 64, "buffer holds whole merge batches and a 32-column chunk");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    Smem& S = *reinterpret_cast<Smem*>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0) {
        for (int i = 0; i < STAGES; ++i) mbar_init(&S.bar_load[i], 1);
        for (int i = 0; i < ACCS; ++i) mbar_init(&S.bar_mma[i], 1);
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
    const uint32_t idesc = make_idesc();
    // mbarrier phase bits and thread 0's in-flight async work (drained on
    // error), one bit per stage / accumulator so they stay in registers
    uint32_t ph_load = 0, ph_mma = 0, load_busy = 0, mma_busy = 0;
    const int64_t n_vtiles = (n_vox + TILE_M - 1) / TILE_M;
    const float2* mybuf = &S.buf[0][tid];
    float2* mybuf_w = &S.buf[0][tid];
    const uint32_t a_base = smem_u32(S.a);
    bool ok = true;

    for (int64_t vt = blockIdx.x; vt < n_vtiles && ok; vt += gridDim.x) {
        // ---- prologue loads: the stages are free (previous tile fully drained) ----
        if (tid == 0) {
            for (int s = 0; s < STAGES && s < n_tiles; ++s) {
                mbar_expect_tx(&S.bar_load[s], B_BYTES + AUX_BYTES);
                bulk_g2s(S.b[s], tiles + (size_t)s * B_BYTES, B_BYTES, &S.bar_load[s]);
                bulk_g2s(S.aux[s], aux + (size_t)s * TILE_N, AUX_BYTES, &S.bar_load[s]);
                load_busy |= 1u << s;
            }
        }
        const int64_t row = vt * TILE_M + tid;
        const bool live = row < n_vox;
        // ---- voxel tile -> BF16 canonical A (each thread its own row) ----
        for (int kc = 0; kc < KPAD / 8; ++kc) {
            __align__(16) __nv_bfloat16 v8[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int k = kc * 8 + i;
                float x = 0.f;
                if (live && k < F) x = meas[row * F + k] - (FREE ? 0.f : __ldg(mu + k));
                v8[i] = __float2bfloat16_rn(x);
            }
            *reinterpret_cast<uint4*>(S.a + canon_off(tid, kc * 8)) = *reinterpret_cast<const uint4*>(v8);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // generic -> async proxy (A tile)
        __syncthreads();
        float ks[K];
        int kj[K];
#pragma unroll
        for (int i = 0; i < K; ++i) { ks[i] = 3.0e38f; kj[i] = 0; }
        float thr = 3.0e38f;
        int cnt = 0;
        for (int t = 0; t <= n_tiles && ok; ++t) {
            // ---- issue the MMA of tile t into accumulator t & 1 ----
            if (t < n_tiles && tid == 0) {
                const int st = t % STAGES;
                if (mbar_wait(&S.bar_load[st], (ph_load >> st) & 1u)) {
                    load_busy &= ~(1u << st);
                    ph_load ^= 1u << st;
                } else {
                    S.err = 1;
                }
                if (!S.err) {
                    fence_after();
                    const uint32_t b_base = smem_u32(S.b[st]);
                    const uint32_t d = tmem + (uint32_t)((t & 1) * TILE_N);
                    mma_bf16(d, make_sdesc(a_base), make_sdesc(b_base), idesc, 0u);
                    mma_bf16(d, make_sdesc(a_base + 2 * LBO), make_sdesc(b_base + 2 * LBO), idesc, 1u);
                    mma_commit(&S.bar_mma[t & 1]);
                    mma_busy |= 1u << (t & 1);
                }
            }
            if (t == 0) continue;
            // ---- epilogue of tile t-1 while MMA t runs ----
            const int tt = t - 1, acc = tt & 1, st = tt % STAGES;
            if (mbar_wait(&S.bar_mma[acc], (ph_mma >> acc) & 1u)) mma_busy &= ~(1u << acc);
            else S.err = 1;
            ph_mma ^= 1u << acc;
            fence_after();
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(acc * TILE_N);
            const float* ax = S.aux[st];
            const int jb = tt * TILE_N;
#pragma unroll 1
            for (int c = 0; c < TILE_N; c += 32) {
                if (__any_sync(0xffffffffu, cnt > CAP - 32)) merge_buffer<K>(ks, kj, thr, cnt, mybuf);
                float v[32];
                tmem_ld32(taddr + (uint32_t)c, v);
                float q[32];
#pragma unroll
                for (int i = 0; i < 32; i += 4) {
                    const float4 a4 = *reinterpret_cast<const float4*>(ax + c + i);
                    q[i] = a4.x; q[i + 1] = a4.y; q[i + 2] = a4.z; q[i + 3] = a4.w;
                }
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const float sc = FREE ? (-v[i] * fabsf(v[i])) * q[i] : fmaf(-2.f, v[i], q[i]);
                    if (sc < thr) {
                        mybuf_w[cnt * TILE_M] = make_float2(sc, __int_as_float(jb + c + i));
                        ++cnt;
                    }
                }
            }
            fence_before();
            __syncthreads();   // accumulator acc and stage st are free again
            if (tid == 0 && tt + STAGES < n_tiles && !S.err) {
                mbar_expect_tx(&S.bar_load[st], B_BYTES + AUX_BYTES);
                bulk_g2s(S.b[st], tiles + (size_t)(tt + STAGES) * B_BYTES, B_BYTES, &S.bar_load[st]);
                bulk_g2s(S.aux[st], aux + (size_t)(tt + STAGES) * TILE_N, AUX_BYTES, &S.bar_load[st]);
                load_busy |= 1u << st;
            }
            if (S.err) ok = false;
        }
        if (!ok) break;
        merge_buffer<K>(ks, kj, thr, cnt, mybuf);
        // the (now empty) buffer carries the candidates to the rescore loop, so
        // ks/kj are only ever indexed by constants and stay in registers
#pragma unroll
        for (int i = 0; i < K; ++i) mybuf_w[i * TILE_M] = make_float2(ks[i], __int_as_float(kj[i]));
        // ---- fp32 rescore of the k candidates from the fp32 data ----
        if (live) {
            float m[KPAD];
#pragma unroll
            for (int k = 0; k < KPAD; ++k) m[k] = k < F ? meas[row * F + k] : 0.f;
            float best = 3.0e38f, bs0 = 0.f;
            int bj = 0x7FFFFFFF;
#pragma unroll 1
            for (int i = 0; i < K; ++i) {
                const float2 cand = mybuf[i * TILE_M];
                const int j = __float_as_int(cand.y);
                if (!(cand.x < 3.0e38f) || j < 0 || j >= n_lib) continue;
                const float* L = lib + (size_t)j * F;
                float dot = 0.f, rr = 0.f;
#pragma unroll
                for (int k = 0; k < KPAD; ++k)
                    if (k < F) { dot = fmaf(m[k], L[k], dot); rr = fmaf(L[k], L[k], rr); }
                const float s0 = FREE ? dot / fmaxf(rr, 1e-30f) : 1.f;
                float res = 0.f;
#pragma unroll
                for (int k = 0; k < KPAD; ++k)
                    if (k < F) { const float r = m[k] - s0 * L[k]; res = fmaf(r, r, res); }
                if (FREE && !(dot > 0.f)) res = 3.0e38f;
                if (res < best || (res == best && j < bj)) { best = res; bj = j; bs0 = s0; }
            }
            best_idx[row] = bj == 0x7FFFFFFF ? 0 : bj;
            best_resid[row] = best;
            if (FREE && best_s0) best_s0[row] = bs0;
        }
        __syncthreads();
    }
    // ---- teardown: no copy or MMA may still be in flight when TMEM is freed ----
    if (tid == 0 && S.err) {
        for (int b = 0; b < STAGES; ++b)
            if ((load_busy >> b) & 1u) mbar_wait(&S.bar_load[b], (ph_load >> b) & 1u);
        for (int b = 0; b < ACCS; ++b)
            if ((mma_busy >> b) & 1u) mbar_wait(&S.bar_mma[b], (ph_mma >> b) & 1u);
    }
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
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(int), s);
    if (e != cudaSuccess) return host::cuda_fail(e, "match bf16 memset");
    if (!free_s0) column_mean_kernel<<<d->n_feat, 256, 0, s>>>(d->lib, d->n_lib, d->n_feat, mu);
    const int64_t n_ent = (int64_t)n_tiles * TILE_N;
    pack_library_kernel<<<(unsigned)((n_ent + 255) / 256), 256, 0, s>>>(d->lib, d->n_lib, d->n_feat, n_tiles,
                                                                         free_s0 ? 1 : 0, mu, tiles, aux);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t n_vtiles = (d->n_vox + TILE_M - 1) / TILE_M;
    const size_t smem = sizeof(Smem);
#define MADI_LAUNCH_BF16(KK, FR)                                                                          \
    do {                                                                                                  \
        auto k = match_bf16_kernel<KK, FR>;                                                               \
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);             \
        if (e != cudaSuccess) return host::cuda_fail(e, "match bf16 attribute");                          \
        int per_sm = 0;                                                                                   \
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 128, smem);                         \
        if (e != cudaSuccess) return host::cuda_fail(e, "match bf16 occupancy");                          \
        /* TMEM: at most 512 / TMEM_COLS CTAs may hold columns on one SM */                               \
        per_sm = std::max(1, std::min(per_sm, 512 / TMEM_COLS));                                          \
        const int grid = (int)std::min<int64_t>(n_vtiles, (int64_t)sms * per_sm);                        \
        k<<<grid, 128, smem, s>>>(d->measured, d->lib, d->n_vox, d->n_lib, d->n_feat, tiles, aux, mu,    \
                                  n_tiles, d->best_idx, d->best_resid, d->best_s0, err);                 \
    } while (0)
    if (free_s0) {
        if (d->topk == 8) MADI_LAUNCH_BF16(8, true);
        else if (d->topk == 16) MADI_LAUNCH_BF16(16, true);
        else MADI_LAUNCH_BF16(32, true);
    } else {
        if (d->topk == 8) MADI_LAUNCH_BF16(8, false);
        else if (d->topk == 16) MADI_LAUNCH_BF16(16, false);
        else MADI_LAUNCH_BF16(32, false);
    }
#undef MADI_LAUNCH_BF16
    e = cudaGetLastError();
    if (e != cudaSuccess) return host::cuda_fail(e, "match bf16 launch");
    return MADI_OK;
}
