// Library match (MAP nearest library entry per voxel), replacing
// _map_kernel_fixed / _map_kernel_free_s0 (madi/fitters_gpu.py:96-154).
//
// FP32 path: exhaustive fp32 scan on the CUDA cores, library streamed through
// shared memory in chunks, one voxel per thread.  Fixed S0 scores the centred
// pair (m - mu, L_j - mu), mu the library column mean: the uncentred expanded
// form |L_j|^2 - 2 m.L_j rounds at ~|L|^2 2^-24, coarser than the gap between
// near-tied entries of a dense library, while the centred form rounds at
// ~|L - mu|^2 2^-24.
#include <cstdint>
#include "madi_device.cuh"
#include "madi_host.h"

namespace madi {

constexpr int MATCH_THREADS = 256;
constexpr int MATCH_CHUNK = 128;

// fixed S0: score_j = |L_j - mu|^2 - 2 (m - mu).(L_j - mu) = |m - L_j|^2 - |m - mu|^2 ;
// free S0: score_j = -(m.r)^2/|r|^2 when m.r > 0 (mu unused).
template <int FMAX, int MODE>
__global__ void __launch_bounds__(MATCH_THREADS) match_fp32_kernel(const float* __restrict__ meas,
                                                                   const float* __restrict__ lib,
                                                                   const float* __restrict__ mu, int64_t n_vox,
                                                                   int n_lib, int n_feat, int32_t* best_idx,
                                                                   float* best_resid, float* best_s0) {
    __shared__ float sl[MATCH_CHUNK][FMAX];
    __shared__ float sn[MATCH_CHUNK];
    __shared__ float smu[FMAX];
    const int64_t v = (int64_t)blockIdx.x * MATCH_THREADS + threadIdx.x;
    if (threadIdx.x < FMAX)
        smu[threadIdx.x] = (MODE == MADI_MATCH_FIXED_S0 && (int)threadIdx.x < n_feat) ? mu[threadIdx.x] : 0.f;
    __syncthreads();
    float m[FMAX];
#pragma unroll
    for (int f = 0; f < FMAX; ++f) m[f] = (v < n_vox && f < n_feat) ? meas[v * n_feat + f] - smu[f] : 0.f;
    float best = 3.0e38f;
    int bj = 0;
    for (int base = 0; base < n_lib; base += MATCH_CHUNK) {
        const int cnt = min(MATCH_CHUNK, n_lib - base);
        __syncthreads();
        for (int t = threadIdx.x; t < MATCH_CHUNK * FMAX; t += MATCH_THREADS) {
            const int e = t / FMAX, f = t - e * FMAX;
            sl[e][f] = (e < cnt && f < n_feat) ? lib[(int64_t)(base + e) * n_feat + f] - smu[f] : 0.f;
        }
        __syncthreads();
        if (threadIdx.x < MATCH_CHUNK) {
            float s = 0.f;
#pragma unroll
            for (int f = 0; f < FMAX; ++f) s = fmaf(sl[threadIdx.x][f], sl[threadIdx.x][f], s);
            sn[threadIdx.x] = MODE == MADI_MATCH_FREE_S0 ? fmaxf(s, 1e-30f) : s;
        }
        __syncthreads();
        for (int e = 0; e < cnt; ++e) {
            float dot = 0.f;
#pragma unroll
            for (int f = 0; f < FMAX; ++f) dot = fmaf(m[f], sl[e][f], dot);
            float score;
            if (MODE == MADI_MATCH_FIXED_S0) {
                score = fmaf(-2.f, dot, sn[e]);
            } else {
                score = dot > 0.f ? -(dot * dot) / sn[e] : 3.0e38f;
            }
            if (score < best) { best = score; bj = base + e; }
        }
    }
    if (v >= n_vox) return;
    // Residual of the chosen entry from the direct difference of the raw data.
#pragma unroll
    for (int f = 0; f < FMAX; ++f) m[f] = f < n_feat ? meas[v * n_feat + f] : 0.f;
    const float* L = lib + (int64_t)bj * n_feat;
    float dot = 0.f, rr = 0.f;
#pragma unroll
    for (int f = 0; f < FMAX; ++f) {
        if (f < n_feat) { dot = fmaf(m[f], L[f], dot); rr = fmaf(L[f], L[f], rr); }
    }
    float s0 = 1.f;
    if (MODE == MADI_MATCH_FREE_S0) s0 = dot / fmaxf(rr, 1e-30f);
    float res = 0.f;
#pragma unroll
    for (int f = 0; f < FMAX; ++f) {
        if (f < n_feat) {
            const float r = m[f] - s0 * L[f];
            res = fmaf(r, r, res);
        }
    }
    if (MODE == MADI_MATCH_FREE_S0 && !(dot > 0.f)) res = 3.0e38f;
    best_idx[v] = bj;
    best_resid[v] = res;
    if (MODE == MADI_MATCH_FREE_S0 && best_s0) best_s0[v] = s0;
}

template <int FMAX>
static madi_status launch_fp32(const madi_match_desc* d, float* mu, cudaStream_t s) {
    const int64_t blocks = (d->n_vox + MATCH_THREADS - 1) / MATCH_THREADS;
    if (d->mode == MADI_MATCH_FIXED_S0)
        match_fp32_kernel<FMAX, MADI_MATCH_FIXED_S0><<<(unsigned)blocks, MATCH_THREADS, 0, s>>>(
            d->measured, d->lib, mu, d->n_vox, d->n_lib, d->n_feat, d->best_idx, d->best_resid, d->best_s0);
    else
        match_fp32_kernel<FMAX, MADI_MATCH_FREE_S0><<<(unsigned)blocks, MATCH_THREADS, 0, s>>>(
            d->measured, d->lib, nullptr, d->n_vox, d->n_lib, d->n_feat, d->best_idx, d->best_resid, d->best_s0);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return host::cuda_fail(e, "match fp32 launch");
    return MADI_OK;
}

}  // namespace madi

using namespace madi;

madi_status madi_match_bf16(const madi_match_desc* d, cudaStream_t s);
const int* madi_match_bf16_status_word(const madi_match_desc* d);
int64_t madi_match_bf16_scratch(int64_t n_vox, int32_t n_lib, int32_t n_feat, int32_t topk);
void madi_match_column_mean(const float* lib, int32_t n_lib, int32_t n_feat, float* mu, cudaStream_t s);

// fp32 needs room for the column means (either mode, so one size fits both).
static constexpr int64_t FP32_SCRATCH = 256;

extern "C" int64_t madi_match_scratch_bytes(int64_t n_vox, int32_t n_lib, int32_t n_feat, int32_t precision,
                                            int32_t topk) {
    if (precision == MADI_MATCH_BF16) return madi_match_bf16_scratch(n_vox, n_lib, n_feat, topk);
    return FP32_SCRATCH;
}

extern "C" madi_status madi_match(const madi_match_desc* d, void* stream) {
    host::clear_error();
    if (!d || !d->measured || !d->lib || !d->best_idx || !d->best_resid || d->n_vox < 0 || d->n_lib < 1 ||
        d->n_feat < 1)
        return host::fail(MADI_ERR_INVALID, "match: bad arguments");
    if (d->n_feat > 32) return host::fail(MADI_ERR_UNSUPPORTED, "match: at most 32 features");
    if (d->mode != MADI_MATCH_FIXED_S0 && d->mode != MADI_MATCH_FREE_S0)
        return host::fail(MADI_ERR_INVALID, "match: unknown mode");
    if (d->n_vox == 0) return MADI_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (d->precision == MADI_MATCH_BF16) return madi_match_bf16(d, s);
    if (d->precision != MADI_MATCH_FP32) return host::fail(MADI_ERR_INVALID, "match: unknown precision");
    float* mu = nullptr;
    if (d->mode == MADI_MATCH_FIXED_S0) {
        if (!d->scratch || d->scratch_bytes < FP32_SCRATCH)
            return host::fail(MADI_ERR_CAPACITY, "match fp32: scratch %lld < %lld bytes", (long long)d->scratch_bytes,
                              (long long)FP32_SCRATCH);
        if ((reinterpret_cast<uintptr_t>(d->scratch) & 255) != 0)
            return host::fail(MADI_ERR_INVALID, "match fp32: scratch must be 256-byte aligned");
        mu = static_cast<float*>(d->scratch);
        madi_match_column_mean(d->lib, d->n_lib, d->n_feat, mu, s);
    }
    if (d->n_feat <= 8) return launch_fp32<8>(d, mu, s);
    if (d->n_feat <= 16) return launch_fp32<16>(d, mu, s);
    if (d->n_feat <= 24) return launch_fp32<24>(d, mu, s);
    return launch_fp32<32>(d, mu, s);
}

extern "C" madi_status madi_match_wait(const madi_match_desc* d, void* stream) {
    host::clear_error();
    if (!d) return host::fail(MADI_ERR_INVALID, "match_wait: null descriptor");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return host::cuda_fail(e, "match_wait: stream");
    if (d->precision != MADI_MATCH_BF16 || d->n_vox == 0) return MADI_OK;
    if (!d->scratch || d->scratch_bytes < madi_match_bf16_scratch(d->n_vox, d->n_lib, d->n_feat, d->topk))
        return host::fail(MADI_ERR_INVALID, "match_wait: descriptor has no BF16 scratch");
    int word = 0;
    e = cudaMemcpyAsync(&word, madi_match_bf16_status_word(d), sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return host::cuda_fail(e, "match_wait: status word");
    if (word == 1)
        return host::fail(MADI_ERR_TIMEOUT, "match bf16: a bounded wait ran out; the rows of the CTAs that gave up "
                                            "have no result (issued copies and MMAs were drained)");
    if (word != 0)
        return host::fail(MADI_ERR_TIMEOUT, "match bf16: a bounded wait ran out and so did the drain of the issued "
                                            "copies and MMAs");
    return MADI_OK;
}
