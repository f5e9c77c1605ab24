// Host-side native code: error plumbing and the geometry builders that run on
// the CPU before any walk (KD tree of madi/ensemble.py:525-563 and the voxel
// candidate grid used by the fp32 walker).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>
#include <filesystem>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <new>
#include "madi_host.h"

namespace madi {
namespace host {
static thread_local char g_err[512] = {0};

void clear_error() { g_err[0] = 0; }

madi_status fail(madi_status code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

madi_status cuda_fail(cudaError_t e, const char* what) {
    return fail(MADI_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}
}  // namespace host

// Runs job(t) for t in [0, T): t >= 1 on new threads where the system gives
// them, every other t (always t = 0) on the calling thread; returns when all
// have ended.  A thread that cannot be created costs time, not correctness:
// every range is still processed, and the results are joined in order.
template <class F>
static void run_parallel(int T, F job) {
    std::vector<std::thread> workers;
    std::vector<int> here;
    try {
        here.reserve(T);
        workers.reserve(T);
    } catch (...) {
    }
    here.push_back(0);
    for (int t = 1; t < T; ++t) {
        try {
            workers.emplace_back(job, t);
        } catch (...) {
            here.push_back(t);
        }
    }
    for (int t : here) job(t);
    for (std::thread& w : workers) w.join();
}
}  // namespace madi

using namespace madi;

extern "C" const char* madi_last_error_string(void) { return host::g_err; }
extern "C" int32_t madi_abi_version(void) { return MADI_ABI_VERSION; }

// ---------------------------------------------------------------------------
// KD tree: each node takes the median (rank n/2) of its subset along the axis of
// widest coordinate spread (first axis on ties); the lower-rank half becomes the
// left subtree, the rest the right one; nodes are numbered in preorder.
// ---------------------------------------------------------------------------
namespace {
struct KdBuilder {
    const double* s;
    int32_t *seed, *left, *right, *parent;
    int8_t* axis;
    int32_t next = 0;

    int32_t build(int32_t* idx, int32_t n, int32_t up) {
        if (n <= 0) return -1;
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int32_t i = 0; i < n; ++i)
            for (int a = 0; a < 3; ++a) {
                const double v = s[3 * (size_t)idx[i] + a];
                lo[a] = std::min(lo[a], v);
                hi[a] = std::max(hi[a], v);
            }
        int ax = 0;
        for (int a = 1; a < 3; ++a)
            if (hi[a] - lo[a] > hi[ax] - lo[ax]) ax = a;
        const int32_t mid = n / 2;
        std::nth_element(idx, idx + mid, idx + n, [&](int32_t a, int32_t b) {
            const double va = s[3 * (size_t)a + ax], vb = s[3 * (size_t)b + ax];
            return va < vb || (va == vb && a < b);
        });
        const int32_t node = next++;
        seed[node] = idx[mid];
        axis[node] = (int8_t)ax;
        parent[node] = up;
        left[node] = build(idx, mid, node);
        right[node] = build(idx + mid + 1, n - mid - 1, node);
        return node;
    }
};
}  // namespace

static madi_status kdtree_build_impl(const double* seeds_xyz, int32_t n, int32_t* node_seed,
                                         int8_t* node_axis, int32_t* node_left, int32_t* node_right,
                                         int32_t* node_parent) {
    host::clear_error();
    if (n < 1 || !seeds_xyz || !node_seed || !node_axis || !node_left || !node_right || !node_parent)
        return host::fail(MADI_ERR_INVALID, "kdtree_build: bad arguments");
    std::vector<int32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    KdBuilder b{seeds_xyz, node_seed, node_left, node_right, node_parent, node_axis};
    const int32_t root = b.build(idx.data(), n, -1);
    if (root != 0 || b.next != n) return host::fail(MADI_ERR_INVALID, "kdtree_build: inconsistent tree");
    return MADI_OK;
}

// ---------------------------------------------------------------------------
// Voxel candidate grid.  For voxel V (grown by eps) let
//   D(V) = min over seeds s of the distance from s to the farthest point of V,
// an upper bound of the nearest-seed distance d1(p) for every p in V.  A seed j
// can (a) be nearest, (b) bind a facet (d_j < d1 + 2 alpha_1), or (c) have a
// shifted facet within `cap` of p's label boundary only if
//   dist(s_j, V) <= D(V) + 2 alpha_max + 2 cap,
// because m_j >= (d_j - d1) / 2 for every seed.  Every such seed is listed.
// ---------------------------------------------------------------------------
namespace {
struct Bins {
    double lo[3], b;
    int nb[3];
    std::vector<int32_t> start, items;
    int clampi(int v, int a) const { return std::min(std::max(v, 0), nb[a] - 1); }
};

Bins make_bins(const double* s, int32_t n, double b) {
    Bins B;
    double hi[3];
    for (int a = 0; a < 3; ++a) { B.lo[a] = 1e300; hi[a] = -1e300; }
    for (int32_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            B.lo[a] = std::min(B.lo[a], s[4 * (size_t)i + a]);
            hi[a] = std::max(hi[a], s[4 * (size_t)i + a]);
        }
    B.b = b;
    for (int a = 0; a < 3; ++a) B.nb[a] = std::max(1, (int)std::ceil((hi[a] - B.lo[a]) / b) + 1);
    const size_t nbin = (size_t)B.nb[0] * B.nb[1] * B.nb[2];
    std::vector<int32_t> cnt(nbin + 1, 0), which(n);
    for (int32_t i = 0; i < n; ++i) {
        int c[3];
        for (int a = 0; a < 3; ++a) c[a] = B.clampi((int)std::floor((s[4 * (size_t)i + a] - B.lo[a]) / b), a);
        which[i] = (int32_t)(((size_t)c[2] * B.nb[1] + c[1]) * B.nb[0] + c[0]);
        cnt[which[i] + 1]++;
    }
    for (size_t k = 0; k < nbin; ++k) cnt[k + 1] += cnt[k];
    B.start = cnt;
    B.items.assign(n, 0);
    std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
    for (int32_t i = 0; i < n; ++i) B.items[fill[which[i]]++] = i;
    return B;
}

template <class F>
void for_bins_in_box(const Bins& B, const double lo[3], const double hi[3], F f) {
    int a0[3], a1[3];
    for (int a = 0; a < 3; ++a) {
        a0[a] = B.clampi((int)std::floor((lo[a] - B.lo[a]) / B.b), a);
        a1[a] = B.clampi((int)std::floor((hi[a] - B.lo[a]) / B.b), a);
    }
    for (int z = a0[2]; z <= a1[2]; ++z)
        for (int y = a0[1]; y <= a1[1]; ++y)
            for (int x = a0[0]; x <= a1[0]; ++x) {
                const size_t k = ((size_t)z * B.nb[1] + y) * B.nb[0] + x;
                for (int32_t t = B.start[k]; t < B.start[k + 1]; ++t) f(B.items[t]);
            }
}
}  // namespace

namespace {
// Candidate lists of voxels [v0, v1) (linear index, x fastest), in order.
struct GridChunk {
    std::vector<int32_t> ids;
    std::vector<uint32_t> count;
    bool oom = false;               // a host allocation failed in this range
};

void grid_range(const double* seeds, const Bins& B, int G, double h, double eps, double amax, double safe_cap,
                int64_t v0, int64_t v1, GridChunk& out) {
    const double span = G * h;
    std::vector<int32_t> list;
    for (int64_t v = v0; v < v1; ++v) {
        const int ix = (int)(v % G), iy = (int)((v / G) % G), iz = (int)(v / ((int64_t)G * G));
        const double vlo[3] = {ix * h - eps, iy * h - eps, iz * h - eps};
        const double vhi[3] = {(ix + 1) * h + eps, (iy + 1) * h + eps, (iz + 1) * h + eps};
        const double c[3] = {0.5 * (vlo[0] + vhi[0]), 0.5 * (vlo[1] + vhi[1]), 0.5 * (vlo[2] + vhi[2])};
        const double half_diag = 0.5 * std::sqrt(3.0) * (h + 2 * eps);
        // nearest seed to the centre by growing search boxes
        double best_c = 1e300;
        for (double r = B.b;; r *= 2.0) {
            const double lo[3] = {c[0] - r, c[1] - r, c[2] - r}, hi[3] = {c[0] + r, c[1] + r, c[2] + r};
            for_bins_in_box(B, lo, hi, [&](int32_t j) {
                const double* q = seeds + 4 * (size_t)j;
                const double dx = q[0] - c[0], dy = q[1] - c[1], dz = q[2] - c[2];
                best_c = std::min(best_c, std::sqrt(dx * dx + dy * dy + dz * dz));
            });
            if (best_c <= r - B.b || r > 4.0 * (span + B.b * (B.nb[0] + B.nb[1] + B.nb[2]))) break;
        }
        // D(V): min over seeds of the farthest-corner distance; only seeds within
        // best_c + half_diag of the centre can improve on the nearest one.
        const double r1 = best_c + half_diag;
        double D = 1e300;
        {
            const double lo[3] = {c[0] - r1, c[1] - r1, c[2] - r1}, hi[3] = {c[0] + r1, c[1] + r1, c[2] + r1};
            for_bins_in_box(B, lo, hi, [&](int32_t j) {
                const double* q = seeds + 4 * (size_t)j;
                double acc = 0.0;
                for (int a = 0; a < 3; ++a) {
                    const double e = std::max(std::fabs(q[a] - vlo[a]), std::fabs(q[a] - vhi[a]));
                    acc += e * e;
                }
                D = std::min(D, std::sqrt(acc));
            });
        }
        const double R = (D + 2.0 * amax + 2.0 * safe_cap) * (1.0 + 1e-9) + 1e-9;
        list.clear();
        {
            const double lo[3] = {vlo[0] - R, vlo[1] - R, vlo[2] - R}, hi[3] = {vhi[0] + R, vhi[1] + R, vhi[2] + R};
            for_bins_in_box(B, lo, hi, [&](int32_t j) {
                const double* q = seeds + 4 * (size_t)j;
                double acc = 0.0;
                for (int a = 0; a < 3; ++a) {
                    const double e = std::max(std::max(vlo[a] - q[a], q[a] - vhi[a]), 0.0);
                    acc += e * e;
                }
                if (acc <= R * R) list.push_back(j);
            });
        }
        std::sort(list.begin(), list.end());
        out.ids.insert(out.ids.end(), list.begin(), list.end());
        out.count.push_back((uint32_t)list.size());
    }
}
}  // namespace

static madi_status grid_build_impl(const double* seeds, int32_t n, int32_t G, double h, double eps,
                                       double safe_cap, uint32_t* offsets, void* ids, int32_t ids_u32,
                                       int64_t capacity, int64_t* total) {
    host::clear_error();
    if (!seeds || n < 1 || G < 1 || !(h > 0.0) || eps < 0.0 || safe_cap < 0.0 || !total)
        return host::fail(MADI_ERR_INVALID, "grid_build: bad arguments");
    if (!ids_u32 && n > 65535) return host::fail(MADI_ERR_INVALID, "grid_build: uint16 ids need n <= 65535");
    double amax = 0.0;
    for (int32_t i = 0; i < n; ++i) amax = std::max(amax, seeds[4 * (size_t)i + 3]);
    const double span = G * h;
    const double spacing = std::cbrt(std::max(span * span * span, 1e-30) / std::max(n, 1));
    const Bins B = make_bins(seeds, n, std::max(h, 0.5 * spacing));
    // voxels are independent: contiguous ranges on host threads, joined in order
    const int64_t nv = (int64_t)G * G * G;
    const int hw = std::max(1, (int)std::thread::hardware_concurrency());
    const int T = (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)hw, 32, (nv + 511) / 512}));
    std::vector<GridChunk> chunks(T);
    run_parallel(T, [&](int t) {
        try { grid_range(seeds, B, G, h, eps, amax, safe_cap, nv * t / T, nv * (t + 1) / T, chunks[t]); }
        catch (const std::bad_alloc&) { chunks[t].oom = true; }
    });
    for (const GridChunk& ch : chunks)
        if (ch.oom) return host::fail(MADI_ERR_HOST_MEMORY, "grid_build: out of host memory");
    int64_t count = 0;
    if (offsets) offsets[0] = 0;
    int64_t v = 0;
    for (const GridChunk& ch : chunks)
        for (uint32_t k : ch.count) {
            count += k;
            if (offsets && count <= 0xFFFFFFFFll) offsets[++v] = (uint32_t)count;
        }
    *total = count;
    if (count > 0xFFFFFFFFll) return host::fail(MADI_ERR_CAPACITY, "grid_build: more than 2^32 candidate ids");
    if (ids && count > capacity) return host::fail(MADI_ERR_CAPACITY, "grid_build: capacity %lld < %lld ids",
                                                   (long long)capacity, (long long)count);
    if (ids) {
        int64_t o = 0;
        for (const GridChunk& ch : chunks) {
            if (ids_u32) std::copy(ch.ids.begin(), ch.ids.end(), static_cast<uint32_t*>(ids) + o);
            else std::copy(ch.ids.begin(), ch.ids.end(), static_cast<uint16_t*>(ids) + o);
            o += (int64_t)ch.ids.size();
        }
    }
    return MADI_OK;
}

// ---------------------------------------------------------------------------
// Cell facet tables.  A cell's Voronoi polytope is cut out of a cube of
// half-side r around its seed by the bisector half-spaces {x : n.x <= h}
// (x = q - c, u = c_j - c, n = u/|u|, h = |u|/2), taken in order of |u|.  The
// polytope is kept in fp64 as faces with ordered vertex polygons.  A plane is
// skipped only when every vertex lies below it by more than eps, so it is
// redundant for the exact polytope too; the pass ends once |u|/2 exceeds the
// largest vertex distance by eps, after which no plane can reach the cell.  The
// candidate radius r doubles until it covers twice that distance.
// ---------------------------------------------------------------------------
namespace {
struct P3 {
    double x, y, z;
};
inline P3 operator+(P3 a, P3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline P3 operator-(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline P3 operator*(double t, P3 a) { return {t * a.x, t * a.y, t * a.z}; }
inline double dot(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline P3 cross(P3 a, P3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double norm(P3 a) { return std::sqrt(dot(a, a)); }

struct Face {
    P3 n;
    double h;
    int32_t nbr;             // base cell across the plane; -2 for the bounding cube
    std::vector<P3> poly;    // ordered vertices; empty when the plane only touches
};

struct Polytope {
    std::vector<Face> faces;
    double eps = 0.0;

    void cube(double B) {
        faces.clear();
        const P3 ax[3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        for (int a = 0; a < 3; ++a)
            for (int sgn = -1; sgn <= 1; sgn += 2) {
                Face f;
                f.n = (double)sgn * ax[a];
                f.h = B;
                f.nbr = -2;
                const P3 u = ax[(a + 1) % 3], v = ax[(a + 2) % 3];
                const P3 c = (sgn * B) * ax[a];
                f.poly = {c + B * u + B * v, c - B * u + B * v, c - B * u - B * v, c + B * u - B * v};
                faces.push_back(f);
            }
    }
    double excess(P3 n, double h) const {
        double m = -1e300;
        for (const Face& f : faces)
            for (const P3& v : f.poly) m = std::max(m, dot(n, v) - h);
        return m;
    }
    double radius() const {
        double r = 0.0;
        for (const Face& f : faces)
            for (const P3& v : f.poly) r = std::max(r, dot(v, v));
        return std::sqrt(r);
    }
    // Vertices on the new plane, deduplicated and ordered by angle about n.
    std::vector<P3> ring(std::vector<P3>& pts, P3 n) const {
        std::vector<P3> u;
        for (const P3& p : pts) {
            bool dup = false;
            for (const P3& q : u) dup |= norm(p - q) <= 1e-3 * eps;
            if (!dup) u.push_back(p);
        }
        if (u.size() < 3) return {};
        P3 c{0, 0, 0};
        for (const P3& p : u) c = c + p;
        c = (1.0 / (double)u.size()) * c;
        const P3 t = std::fabs(n.x) < 0.6 ? P3{1, 0, 0} : P3{0, 1, 0};
        P3 e1 = cross(n, t);
        e1 = (1.0 / norm(e1)) * e1;
        const P3 e2 = cross(n, e1);
        std::vector<std::pair<double, size_t>> ang(u.size());
        for (size_t i = 0; i < u.size(); ++i) ang[i] = {std::atan2(dot(u[i] - c, e2), dot(u[i] - c, e1)), i};
        std::sort(ang.begin(), ang.end());
        std::vector<P3> out(u.size());
        for (size_t i = 0; i < u.size(); ++i) out[i] = u[ang[i].second];
        return out;
    }
    void clip(P3 n, double h, int32_t nbr) {
        std::vector<P3> fresh;
        std::vector<Face> kept;
        kept.reserve(faces.size() + 1);
        const double on = 1e-6 * eps;
        for (Face& f : faces) {
            if (f.poly.empty()) { kept.push_back(std::move(f)); continue; }
            const size_t m = f.poly.size();
            std::vector<P3> out;
            double smin = 1e300;
            for (size_t i = 0; i < m; ++i) {
                const P3 a = f.poly[i], b = f.poly[(i + 1) % m];
                const double sa = dot(n, a) - h, sb = dot(n, b) - h;
                smin = std::min(smin, sa);
                if (sa <= 0.0) {
                    out.push_back(a);
                    if (sa >= -on) fresh.push_back(a);
                }
                if ((sa <= 0.0) != (sb <= 0.0)) {
                    const P3 p = a + (sa / (sa - sb)) * (b - a);
                    out.push_back(p);
                    fresh.push_back(p);
                }
            }
            if (out.size() >= 3) {
                f.poly.swap(out);
                kept.push_back(std::move(f));
            } else if (smin <= eps) {       // reduced to an edge or a point: keep the plane
                f.poly.clear();
                kept.push_back(std::move(f));
            }                               // else wholly beyond the new plane
        }
        Face nf;
        nf.n = n;
        nf.h = h;
        nf.nbr = nbr;
        nf.poly = ring(fresh, n);
        kept.push_back(std::move(nf));
        faces.swap(kept);
    }
};
}  // namespace

namespace {
// Facet records of a range of cells, in order: per cell its padded record count.
struct FacetChunk {
    std::vector<float> planes;      // 4 floats per record
    std::vector<int32_t> nbr;
    std::vector<uint32_t> count;
    double h_max = 0.0, reach = 0.0;
    int32_t err_cell = -1, err_other = -1;
    bool oom = false;               // a host allocation failed in this range
};

struct FacetInput {
    const double* seeds;
    const std::vector<double>* pts;     // candidates: x, y, z, base id
    const Bins* B;
    double spacing, r_max;
};

void facets_range(const FacetInput& X, int32_t c0, int32_t c1, FacetChunk& out) {
    const std::vector<double>& pts = *X.pts;
    std::vector<std::pair<double, int32_t>> cand;
    std::vector<const Face*> fl;
    for (int32_t c = c0; c < c1; ++c) {
        const double* sc = X.seeds + 4 * (size_t)c;
        const P3 x0{sc[0], sc[1], sc[2]};
        Polytope P;
        bool closed = false;
        for (double r = std::min(3.0 * X.spacing, X.r_max);; r = std::min(2.0 * r, X.r_max)) {
            cand.clear();
            const double blo[3] = {x0.x - r, x0.y - r, x0.z - r}, bhi[3] = {x0.x + r, x0.y + r, x0.z + r};
            for_bins_in_box(*X.B, blo, bhi, [&](int32_t j) {
                const P3 u = P3{pts[4 * (size_t)j], pts[4 * (size_t)j + 1], pts[4 * (size_t)j + 2]} - x0;
                const double d = norm(u);
                if (d <= r && !(d == 0.0 && (int32_t)pts[4 * (size_t)j + 3] == c)) cand.push_back({d, j});
            });
            std::sort(cand.begin(), cand.end());
            P.eps = 1e-9 * r;
            P.cube(r);
            bool ended = false;
            for (const auto& cj : cand) {
                if (cj.first == 0.0) {
                    out.err_cell = c;
                    out.err_other = (int32_t)pts[4 * (size_t)cj.second + 3];
                    return;
                }
                if (0.5 * cj.first > P.radius() + P.eps) { ended = true; break; }
                const size_t j = (size_t)cj.second;
                const P3 u = P3{pts[4 * j], pts[4 * j + 1], pts[4 * j + 2]} - x0;
                const P3 nv = (1.0 / cj.first) * u;
                const double h = 0.5 * cj.first;
                if (P.excess(nv, h) < -P.eps) continue;
                P.clip(nv, h, (int32_t)pts[4 * j + 3]);
            }
            if (ended || 2.0 * (P.radius() + P.eps) <= r) { closed = true; break; }
            if (r >= X.r_max) break;
        }
        fl.clear();
        if (closed) {
            for (const Face& f : P.faces)
                if (f.nbr >= 0) fl.push_back(&f);
            std::sort(fl.begin(), fl.end(), [](const Face* a, const Face* b) { return a->h < b->h; });
            out.reach = std::max(out.reach, P.radius());
            for (const Face* f : fl) out.h_max = std::max(out.h_max, f->h);
        }
        const int64_t nf = closed ? (int64_t)fl.size() : 0;
        const int64_t padded = std::max<int64_t>(4, (nf + 3) & ~3ll);
        for (int64_t k = 0; k < padded; ++k) {
            if (k < nf) {
                const Face* f = fl[k];
                out.planes.insert(out.planes.end(), {(float)f->n.x, (float)f->n.y, (float)f->n.z, (float)f->h});
                out.nbr.push_back(f->nbr);
            } else {
                out.planes.insert(out.planes.end(), {0.0f, 0.0f, 0.0f, closed ? 3.0e38f : -3.0e38f});
                out.nbr.push_back(-1);
            }
        }
        out.count.push_back((uint32_t)padded);
    }
}
}  // namespace

static madi_status facets_build_impl(const double* seeds, int32_t n, int32_t periodic, double L,
                                         uint32_t* begin, float* planes, int32_t* nbr, int64_t capacity,
                                         int64_t* total, double* stats) {
    host::clear_error();
    if (!seeds || n < 2 || !begin || !total || (periodic && !(L > 0.0)))
        return host::fail(MADI_ERR_INVALID, "facets_build: bad arguments");
    // candidate points: the seeds, plus their 26 neighbouring images when periodic
    std::vector<double> pts;
    const int K = periodic ? 1 : 0;
    for (int kz = -K; kz <= K; ++kz)
        for (int ky = -K; ky <= K; ++ky)
            for (int kx = -K; kx <= K; ++kx)
                for (int32_t i = 0; i < n; ++i) {
                    const double* s = seeds + 4 * (size_t)i;
                    pts.insert(pts.end(), {s[0] + kx * L, s[1] + ky * L, s[2] + kz * L, (double)i});
                }
    const int32_t np = (int32_t)(pts.size() / 4);
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int32_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], seeds[4 * (size_t)i + a]);
            hi[a] = std::max(hi[a], seeds[4 * (size_t)i + a]);
        }
    const double ext = periodic ? L : std::max({hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2], 1e-30});
    const double spacing = std::cbrt(ext * ext * ext / n);
    const Bins B = make_bins(pts.data(), np, spacing);
    // periodic: images within +-1 box cover every candidate up to r = L.  A
    // finite population's cells close within a few spacings except on its outer
    // surface; past 12 spacings a cell is left open (the walker's voxel-grid
    // classifier decides there) instead of scanning the whole population.
    const FacetInput X{seeds, &pts, &B, spacing, periodic ? L : std::min(4.0 * ext, 12.0 * spacing)};
    // cells are independent: contiguous ranges on host threads, joined in order
    const int hw = std::max(1, (int)std::thread::hardware_concurrency());
    const int T = std::max(1, std::min({hw, 32, (n + 255) / 256}));
    std::vector<FacetChunk> chunks(T);
    run_parallel(T, [&](int t) {
        try { facets_range(X, (int32_t)((int64_t)n * t / T), (int32_t)((int64_t)n * (t + 1) / T), chunks[t]); }
        catch (const std::bad_alloc&) { chunks[t].oom = true; }
    });
    for (const FacetChunk& ch : chunks) {
        if (ch.oom) return host::fail(MADI_ERR_HOST_MEMORY, "facets_build: out of host memory");
        if (ch.err_cell >= 0)
            return host::fail(MADI_ERR_GEOMETRY, "facets_build: seeds %d and %d coincide", ch.err_cell, ch.err_other);
    }
    int64_t count = 0;
    double h_max = 0.0, reach = 0.0;
    int32_t c = 0;
    for (const FacetChunk& ch : chunks) {
        for (uint32_t k : ch.count) {
            begin[c++] = (uint32_t)count;
            count += k;
        }
        h_max = std::max(h_max, ch.h_max);
        reach = std::max(reach, ch.reach);
    }
    if (count > 0xFFFFFFFFll) return host::fail(MADI_ERR_CAPACITY, "facets_build: more than 2^32 facets");
    begin[n] = (uint32_t)count;
    *total = count;
    if (stats) { stats[0] = h_max; stats[1] = reach; }
    if (planes && count > capacity)
        return host::fail(MADI_ERR_CAPACITY, "facets_build: capacity %lld < %lld facets", (long long)capacity,
                          (long long)count);
    if (planes) {
        int64_t o = 0;
        for (const FacetChunk& ch : chunks) {
            std::copy(ch.planes.begin(), ch.planes.end(), planes + 4 * o);
            if (nbr) std::copy(ch.nbr.begin(), ch.nbr.end(), nbr + o);
            o += (int64_t)ch.nbr.size();
        }
    }
    return MADI_OK;
}

// ---------------------------------------------------------------------------
// Autotuner cache: one "key\ttile\tbps\tminb\tstage\trate" line per key.
// ---------------------------------------------------------------------------
namespace {
std::mutex g_tune_mu;

bool valid_key(const char* key) {
    if (!key || !*key) return false;
    for (const char* c = key; *c; ++c)
        if (*c == '\t' || *c == '\n' || *c == '\r') return false;
    return true;
}

bool parse_line(const std::string& line, std::string& key, madi_launch_shape& sh) {
    std::istringstream in(line);
    if (!std::getline(in, key, '\t') || key.empty()) return false;
    return static_cast<bool>(in >> sh.tile_walkers >> sh.blocks_per_sm >> sh.min_blocks >> sh.stage_budget >>
                             sh.walker_steps_per_s);
}
}  // namespace


// C entry point: no C++ exception crosses the ABI (host allocation failures
// return MADI_ERR_HOST_MEMORY).
extern "C" madi_status madi_kdtree_build(const double* seeds_xyz, int32_t n, int32_t* node_seed,
                                         int8_t* node_axis, int32_t* node_left, int32_t* node_right,
                                         int32_t* node_parent) {
    try {
        return kdtree_build_impl(seeds_xyz, n, node_seed, node_axis, node_left, node_right, node_parent);
    } catch (const std::bad_alloc&) {
        return host::fail(MADI_ERR_HOST_MEMORY, "kdtree_build: out of host memory");
    } catch (...) {
        return host::fail(MADI_ERR_INVALID, "kdtree_build: unexpected host error");
    }
}

// C entry point: no C++ exception crosses the ABI (host allocation failures
// return MADI_ERR_HOST_MEMORY).
extern "C" madi_status madi_grid_build(const double* seeds, int32_t n, int32_t G, double h, double eps,
                                       double safe_cap, uint32_t* offsets, void* ids, int32_t ids_u32,
                                       int64_t capacity, int64_t* total) {
    try {
        return grid_build_impl(seeds, n, G, h, eps, safe_cap, offsets, ids, ids_u32, capacity, total);
    } catch (const std::bad_alloc&) {
        return host::fail(MADI_ERR_HOST_MEMORY, "grid_build: out of host memory");
    } catch (...) {
        return host::fail(MADI_ERR_INVALID, "grid_build: unexpected host error");
    }
}

// C entry point: no C++ exception crosses the ABI (host allocation failures
// return MADI_ERR_HOST_MEMORY).
extern "C" madi_status madi_facets_build(const double* seeds, int32_t n, int32_t periodic, double L,
                                         uint32_t* begin, float* planes, int32_t* nbr, int64_t capacity,
                                         int64_t* total, double* stats) {
    try {
        return facets_build_impl(seeds, n, periodic, L, begin, planes, nbr, capacity, total, stats);
    } catch (const std::bad_alloc&) {
        return host::fail(MADI_ERR_HOST_MEMORY, "facets_build: out of host memory");
    } catch (...) {
        return host::fail(MADI_ERR_INVALID, "facets_build: unexpected host error");
    }
}

extern "C" madi_status madi_autotune_load(const char* path, const char* key, madi_launch_shape* out) {
    host::clear_error();
    if (!path || !out || !valid_key(key)) return host::fail(MADI_ERR_INVALID, "autotune_load: bad arguments");
    std::lock_guard<std::mutex> g(g_tune_mu);
    *out = madi_launch_shape{};
    std::ifstream f(path);
    if (!f) return MADI_OK;
    std::string line, k;
    while (std::getline(f, line)) {
        madi_launch_shape sh{};
        if (parse_line(line, k, sh) && k == key) *out = sh;   // last entry wins
    }
    return MADI_OK;
}

extern "C" madi_status madi_autotune_store(const char* path, const char* key, const madi_launch_shape* shape) {
    host::clear_error();
    if (!path || !shape || !valid_key(key) || shape->tile_walkers <= 0)
        return host::fail(MADI_ERR_INVALID, "autotune_store: bad arguments");
    std::lock_guard<std::mutex> g(g_tune_mu);
    std::vector<std::string> keep;
    {
        std::ifstream f(path);
        std::string line, k;
        while (f && std::getline(f, line)) {
            madi_launch_shape sh{};
            if (parse_line(line, k, sh) && k != key) keep.push_back(line);
        }
    }
    std::ostringstream row;
    row.precision(17);
    row << key << '\t' << shape->tile_walkers << '\t' << shape->blocks_per_sm << '\t' << shape->min_blocks << '\t'
        << shape->stage_budget << '\t' << shape->walker_steps_per_s;
    keep.push_back(row.str());
    std::error_code ec;
    const std::filesystem::path p(path);
    if (p.has_parent_path()) std::filesystem::create_directories(p.parent_path(), ec);
    const std::string tmp = std::string(path) + ".tmp";
    {
        std::ofstream o(tmp, std::ios::trunc);
        if (!o) return host::fail(MADI_ERR_INVALID, "autotune_store: cannot write %s", tmp.c_str());
        for (const auto& l : keep) o << l << '\n';
        if (!o) return host::fail(MADI_ERR_INVALID, "autotune_store: write failed for %s", tmp.c_str());
    }
    std::filesystem::rename(tmp, p, ec);
    if (ec) return host::fail(MADI_ERR_INVALID, "autotune_store: rename to %s failed", path);
    return MADI_OK;
}
