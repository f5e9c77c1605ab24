// Bayesian posterior-mean fit over the library, replacing _bayes_kernel_fixed /
// _bayes_kernel_free_s0 (madi/fitters_gpu.py:156-294) and the CPU bayes_fit
// (madi/fitters.py:110-243).
//
// Per voxel, library entry j gets log-weight e_j = log q_j - rw_j / (2 sigma^2)
// with q_j the quadrature weight and rw_j the residual on the normalised scale
// (fixed S0: |m - L_j|^2; free S0: |m/s0_j - L_j|^2, s0_j = m.L_j / |L_j|^2 > 0,
// other entries weight 0).  Outputs are the posterior means and standard
// deviations of (kio, rho, V), the weighted residual, n_eff = W^2 / sum w^2 and
// (free S0) the weighted S0.
//
// One voxel per thread, the library streamed through shared memory twice:
//   pass 1: the fp32 scores of every entry (the match kernel's centred fixed-S0
//           score, or the free-S0 projection), argmax of e_j -> j*; e_j* is then
//           recomputed from the direct difference and is the shift S (the
//           reference shifts by the minimum residual or the maximum log-weight;
//           any shift gives the same normalised weights).
//   pass 2: entries whose screened e_j (with its fp32 error bound) is above
//           S - CUT get the direct-difference residual (error ~F ulp of the
//           residual itself, which is small where weights matter) and add
//           w = exp(e_j - S) to Kahan-compensated fp32 sums of w, w d, w d^2
//           (d = parameter minus that of j*, so narrow posteriors keep their
//           variance), w r, w^2 and w s0.  Entries below the cut weigh less
//           than e^-CUT of entry j*.
#include <cstdint>
#include "madi_device.cuh"
#include "madi_host.h"

namespace madi {
namespace bayes {

constexpr int THREADS = 256;
constexpr int CHUNK = 128;
constexpr float CUT = 60.f;          // exp(-60) ~ 9e-27 of the shift entry's weight

struct Kahan {
    float s = 0.f, c = 0.f;
    MADI_DEV void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    MADI_DEV void scale(float f) { s *= f; c *= f; }
    MADI_DEV double value() const { return (double)s - (double)c; }
};

struct Plan {
    const float* meas;
    const float* lib;
    const float* mu;                 // column means (fixed S0), zeros (free S0)
    const double* logq;
    const double* kio;
    const double* rho;
    const double* V;
    int64_t n_vox;
    int n_lib, F;
    float inv2s2;
    double* out;
};

// Screened log-weight of one entry from the fp32 score, and its error bound.
template <int FMAX, bool FREE>
MADI_DEV void screen(const float* m, const float* l, float sn, float lq, float m2, float inv2s2, float& e,
                     float& err) {
    float dot = 0.f;
#pragma unroll
    for (int f = 0; f < FMAX; ++f) dot = fmaf(m[f], l[f], dot);
    if (!FREE) {
        // centred: r = |m~|^2 + |L~|^2 - 2 m~.L~ ; fp32 error <= (F + 4) 2^-23 (|m~|^2 + |L~|^2)
        const float r = fmaxf(fmaf(-2.f, dot, sn) + m2, 0.f);
        e = lq - r * inv2s2;
        err = ((float)(FMAX + 4) * 1.2e-7f * (m2 + sn)) * inv2s2 + 1e-3f;
    } else {
        // rw = |L|^2 (|m|^2 |L|^2 / (m.L)^2 - 1) when m.L > 0
        if (!(dot > 0.f)) { e = -3.0e38f; err = 0.f; return; }
        const float ratio = m2 * sn / (dot * dot);
        const float rw = fmaxf(sn * (ratio - 1.f), 0.f);
        e = lq - rw * inv2s2;
        err = (sn * ratio * (float)(FMAX + 8) * 2.4e-7f) * inv2s2 + 1e-3f;
    }
}

// Residuals of one entry from the direct difference (raw data): resid (the
// reported residual) and rw (normalised), s0 (free S0; 1 for fixed).
template <int FMAX, bool FREE>
MADI_DEV bool exact(const float* mr, const float* L, int F, float& resid, float& rw, float& s0) {
    s0 = 1.f;
    if (FREE) {
        float dot = 0.f, rr = 0.f;
#pragma unroll
        for (int f = 0; f < FMAX; ++f) {
            if (f < F) { dot = fmaf(mr[f], L[f], dot); rr = fmaf(L[f], L[f], rr); }
        }
        if (!(dot > 0.f)) return false;
        s0 = dot / fmaxf(rr, 1e-30f);
    }
    float r = 0.f;
#pragma unroll
    for (int f = 0; f < FMAX; ++f) {
        if (f < F) {
            const float d = mr[f] - s0 * L[f];
            r = fmaf(d, d, r);
        }
    }
    resid = r;
    rw = FREE ? r / (s0 * s0) : r;
    return true;
}

template <int FMAX, bool FREE>
__global__ void __launch_bounds__(THREADS) bayes_kernel(const Plan P) {
    __shared__ float sl[CHUNK][FMAX];        // centred (fixed) or raw (free) library rows
    __shared__ float sraw[CHUNK][FMAX];      // raw rows for the exact residual
    __shared__ float sn[CHUNK];              // |L~|^2
    __shared__ float slq[CHUNK];
    __shared__ double spar[3][CHUNK];
    __shared__ float smu[FMAX];
    const int F = P.F;
    const int64_t v = (int64_t)blockIdx.x * THREADS + threadIdx.x;
    const bool live = v < P.n_vox;
    if (threadIdx.x < FMAX) smu[threadIdx.x] = (!FREE && (int)threadIdx.x < F) ? P.mu[threadIdx.x] : 0.f;
    __syncthreads();
    float m[FMAX], mr[FMAX];
    float m2 = 0.f;
#pragma unroll
    for (int f = 0; f < FMAX; ++f) {
        mr[f] = (live && f < F) ? P.meas[v * F + f] : 0.f;
        m[f] = f < F ? mr[f] - smu[f] : 0.f;
        m2 = fmaf(m[f], m[f], m2);
    }
    auto stage = [&](int base, int cnt) {
        __syncthreads();
        for (int t = threadIdx.x; t < CHUNK * FMAX; t += THREADS) {
            const int e = t / FMAX, f = t - e * FMAX;
            const float x = (e < cnt && f < F) ? P.lib[(int64_t)(base + e) * F + f] : 0.f;
            sraw[e][f] = x;
            sl[e][f] = f < F ? x - smu[f] : 0.f;
        }
        for (int e = threadIdx.x; e < CHUNK; e += THREADS) {
            const bool ok = e < cnt;
            slq[e] = ok ? (float)P.logq[base + e] : -3.0e38f;
            spar[0][e] = ok ? P.kio[base + e] : 0.0;
            spar[1][e] = ok ? P.rho[base + e] : 0.0;
            spar[2][e] = ok ? P.V[base + e] : 0.0;
        }
        __syncthreads();
        if (threadIdx.x < CHUNK) {
            float s = 0.f;
#pragma unroll
            for (int f = 0; f < FMAX; ++f) s = fmaf(sl[threadIdx.x][f], sl[threadIdx.x][f], s);
            sn[threadIdx.x] = FREE ? fmaxf(s, 1e-30f) : s;
        }
        __syncthreads();
    };
    // ---- pass 1: argmax of the screened log-weight ----
    float best = -3.0e38f;
    int bj = -1;
    for (int base = 0; base < P.n_lib; base += CHUNK) {
        const int cnt = min(CHUNK, P.n_lib - base);
        stage(base, cnt);
        for (int e = 0; e < cnt; ++e) {
            float ee, err;
            screen<FMAX, FREE>(m, sl[e], sn[e], slq[e], m2, P.inv2s2, ee, err);
            if (ee > best) { best = ee; bj = base + e; }
        }
    }
    // shift and centre from the exact residual of j*
    float S = 0.f;
    double x0[3] = {0.0, 0.0, 0.0};
    bool any = bj >= 0;
    if (any) {
        float Lj[FMAX];
#pragma unroll
        for (int f = 0; f < FMAX; ++f) Lj[f] = f < F ? P.lib[(int64_t)bj * F + f] : 0.f;
        float resid, rw, s0;
        any = exact<FMAX, FREE>(mr, Lj, F, resid, rw, s0);
        S = (float)P.logq[bj] - rw * P.inv2s2;
        x0[0] = P.kio[bj];
        x0[1] = P.rho[bj];
        x0[2] = P.V[bj];
    }
    // ---- pass 2: exp-weighted sums over the entries above the cut ----
    Kahan W, W2, R, S0, d1[3], d2[3];
    for (int base = 0; base < P.n_lib; base += CHUNK) {
        const int cnt = min(CHUNK, P.n_lib - base);
        stage(base, cnt);
        if (!any) continue;
        for (int e = 0; e < cnt; ++e) {
            float ee, err;
            screen<FMAX, FREE>(m, sl[e], sn[e], slq[e], m2, P.inv2s2, ee, err);
            if (!(ee + err - S > -CUT)) continue;
            float resid, rw, s0;
            if (!exact<FMAX, FREE>(mr, sraw[e], F, resid, rw, s0)) continue;
            float x = slq[e] - rw * P.inv2s2 - S;
            if (!(x > -CUT)) continue;
            if (x > 0.f) {
                // an entry above the screened maximum (within the screen's error):
                // move the shift to it so that every weight stays <= 1
                const float f = expf(-x);
                W.scale(f);
                W2.scale(f * f);
                R.scale(f);
                S0.scale(f);
#pragma unroll
                for (int k = 0; k < 3; ++k) { d1[k].scale(f); d2[k].scale(f); }
                S += x;
                x = 0.f;
            }
            const float w = expf(x);
            W.add(w);
            W2.add(w * w);
            R.add(w * resid);
            if (FREE) S0.add(w * s0);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float d = (float)(spar[k][e] - x0[k]);
                d1[k].add(w * d);
                d2[k].add(w * d * d);
            }
        }
    }
    if (!live) return;
    const int64_t n = P.n_vox;
    double* o = P.out;
    const double Wv = any ? W.value() : 0.0;
    const double Wd = fmax(Wv, 1e-300);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double a = d1[k].value() / Wd, b = d2[k].value() / Wd;
        o[(int64_t)k * n + v] = Wv > 0.0 ? x0[k] + a : 0.0;                      // kio, rho, V means
        o[(int64_t)(3 + k) * n + v] = Wv > 0.0 ? sqrt(fmax(b - a * a, 0.0)) : 0.0; // their std
    }
    o[6 * n + v] = Wv > 0.0 ? R.value() / Wd : 0.0;
    o[7 * n + v] = Wv > 0.0 ? Wv * Wv / fmax(W2.value(), 1e-300) : 0.0;
    o[8 * n + v] = (FREE && Wv > 0.0) ? S0.value() / Wd : 0.0;
}

template <int FMAX>
static madi_status launch(const madi_bayes_desc* d, const Plan& P, cudaStream_t s) {
    const unsigned blocks = (unsigned)((d->n_vox + THREADS - 1) / THREADS);
    if (d->mode == MADI_MATCH_FREE_S0) bayes_kernel<FMAX, true><<<blocks, THREADS, 0, s>>>(P);
    else bayes_kernel<FMAX, false><<<blocks, THREADS, 0, s>>>(P);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return host::cuda_fail(e, "bayes launch");
    return MADI_OK;
}

}  // namespace bayes
}  // namespace madi

using namespace madi;

void madi_match_column_mean(const float* lib, int32_t n_lib, int32_t n_feat, float* mu, cudaStream_t s);

extern "C" int64_t madi_bayes_scratch_bytes(int32_t n_lib, int32_t n_feat) {
    (void)n_lib;
    (void)n_feat;
    return 256;                     // the column means
}

extern "C" madi_status madi_bayes(const madi_bayes_desc* d, void* stream) {
    host::clear_error();
    if (!d || !d->measured || !d->lib || !d->log_weight || !d->kio || !d->rho || !d->V || !d->out ||
        d->n_vox < 0 || d->n_lib < 1 || d->n_feat < 1)
        return host::fail(MADI_ERR_INVALID, "bayes: bad arguments");
    if (d->n_feat > 32) return host::fail(MADI_ERR_UNSUPPORTED, "bayes: at most 32 features");
    if (d->mode != MADI_MATCH_FIXED_S0 && d->mode != MADI_MATCH_FREE_S0)
        return host::fail(MADI_ERR_INVALID, "bayes: unknown mode");
    if (!(d->sigma_m > 0.0)) return host::fail(MADI_ERR_INVALID, "bayes: sigma_m must be > 0, got %g", d->sigma_m);
    const double inv = 1.0 / (2.0 * d->sigma_m * d->sigma_m);
    if (!(inv < 3.0e38)) return host::fail(MADI_ERR_UNSUPPORTED, "bayes: sigma_m %g too small for fp32 exponents", d->sigma_m);
    if (!d->scratch || d->scratch_bytes < 256) return host::fail(MADI_ERR_CAPACITY, "bayes: scratch < 256 bytes");
    if ((reinterpret_cast<uintptr_t>(d->scratch) & 255) != 0)
        return host::fail(MADI_ERR_INVALID, "bayes: scratch must be 256-byte aligned");
    if (d->n_vox == 0) return MADI_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    float* mu = static_cast<float*>(d->scratch);
    if (d->mode == MADI_MATCH_FIXED_S0) {
        madi_match_column_mean(d->lib, d->n_lib, d->n_feat, mu, s);
    } else {
        const cudaError_t e = cudaMemsetAsync(mu, 0, 32 * sizeof(float), s);
        if (e != cudaSuccess) return host::cuda_fail(e, "bayes memset");
    }
    bayes::Plan P{};
    P.meas = d->measured;
    P.lib = d->lib;
    P.mu = mu;
    P.logq = d->log_weight;
    P.kio = d->kio;
    P.rho = d->rho;
    P.V = d->V;
    P.n_vox = d->n_vox;
    P.n_lib = d->n_lib;
    P.F = d->n_feat;
    P.inv2s2 = (float)inv;
    P.out = d->out;
    if (d->n_feat <= 8) return bayes::launch<8>(d, P, s);
    if (d->n_feat <= 16) return bayes::launch<16>(d, P, s);
    if (d->n_feat <= 24) return bayes::launch<24>(d, P, s);
    return bayes::launch<32>(d, P, s);
}
