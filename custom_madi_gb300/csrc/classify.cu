// Point classifier entry point: labels a batch of points with the SI Eq. S2
// contracted-Voronoi rule (madi/ensemble.py:213-256), either by the reference's
// fp64 stackless KD traversal or by the walker's fp32 voxel-grid rule.
#include "madi_device.cuh"
#include "madi_host.h"

namespace madi {

template <bool F32IN>
__global__ void __launch_bounds__(128) classify_kernel(const madi_geometry gd, const void* pts, int64_t n,
                                                       int method, int32_t* cell_out, uint8_t* inside_out,
                                                       uint8_t* path_out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Geo g = make_geo(gd, reinterpret_cast<const unsigned char*>(gd.stage));
    double px, py, pz;
    if (F32IN) {
        const float* p = reinterpret_cast<const float*>(pts) + 3 * i;
        px = p[0]; py = p[1]; pz = p[2];
    } else {
        const double* p = reinterpret_cast<const double*>(pts) + 3 * i;
        px = p[0]; py = p[1]; pz = p[2];
    }
    int seed = 0, inside = 0, path = 2, st;
    if (!gd.has_cells) {
        st = CLS_OK; path = 0;
    } else if (method == 0) {
        st = classify_kd_f64(g, px, py, pz, seed, inside);
    } else {
        path = 0;
        float rs;
        if (F32IN) {
            st = classify_f32(g, (float)px, (float)py, (float)pz, -1, seed, inside, rs);
        } else {
            // fp64 input: the fp32 rule only sees rounded coordinates, so decide in fp64.
            st = CLS_FALLBACK;
        }
        if (st == CLS_FALLBACK) {
            st = classify_list_f64(g, px, py, pz, seed, inside);
            path = 1;
        }
    }
    if (st != CLS_OK) { seed = -1; inside = 0; path = 255; }
    cell_out[i] = (seed >= 0 && gd.has_cells) ? cell_of(g, seed) : (seed < 0 ? -1 : 0);
    inside_out[i] = (uint8_t)inside;
    if (path_out) path_out[i] = (uint8_t)path;
}

}  // namespace madi

using namespace madi;

extern "C" madi_status madi_classify(const madi_geometry* geom, const void* points, int points_f32, int64_t n,
                                     int method, int32_t* cell_out, uint8_t* inside_out, uint8_t* path_out,
                                     void* stream) {
    host::clear_error();
    if (!geom || n < 0 || (n > 0 && (!points || !cell_out || !inside_out)))
        return host::fail(MADI_ERR_INVALID, "classify: bad arguments");
    if (method != 0 && method != 1) return host::fail(MADI_ERR_INVALID, "classify: method must be 0 (KD) or 1 (grid)");
    if (n == 0) return MADI_OK;
    const int threads = 128;
    const int64_t blocks = (n + threads - 1) / threads;
    if (blocks > 0x7FFFFFFF) return host::fail(MADI_ERR_INVALID, "classify: too many points");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (points_f32)
        classify_kernel<true><<<(unsigned)blocks, threads, 0, s>>>(*geom, points, n, method, cell_out, inside_out, path_out);
    else
        classify_kernel<false><<<(unsigned)blocks, threads, 0, s>>>(*geom, points, n, method, cell_out, inside_out, path_out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return host::cuda_fail(e, "classify launch");
    return MADI_OK;
}
