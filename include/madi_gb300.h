/*
 * madi_gb300.h -- C ABI of the GB300 (sm_103a) MADI Monte Carlo diffusion path.
 *
 * The reference (jadenfigger/Custom_MADI) is Python with Numba-CUDA kernels; it
 * has no foreign-function boundary of its own.  Each entry point below replaces
 * one of its device launches (cited per function) and is bound from Python by
 * custom_madi_gb300/_native.py through ctypes.
 *
 * Conventions
 *   - Plain C types only: device pointers, sizes, a cudaStream_t passed as void*.
 *   - Every function returns a madi_status; no exception crosses the ABI.  On
 *     failure madi_last_error_string() holds a one-line reason (thread-local).
 *   - The library never allocates device memory: every buffer, including the
 *     zero-initialised scratch words named in the descriptors, belongs to the
 *     caller.  Launches are asynchronous on the given stream.
 *   - Units: um, ms.  Geometry is a cubic walk box [0, L)^3.
 */
#ifndef MADI_GB300_H
#define MADI_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MADI_ABI_VERSION 1

typedef enum madi_status {
    MADI_OK = 0,
    MADI_ERR_INVALID = 1,      /* bad argument or descriptor (ValueError upstream)          */
    MADI_ERR_CUDA = 2,         /* a CUDA runtime call failed                                */
    MADI_ERR_CAPACITY = 3,     /* an output or scratch capacity is too small                */
    MADI_ERR_TIMEOUT = 4,      /* a bounded device or host wait ran out                     */
    MADI_ERR_UNSUPPORTED = 5,  /* configuration this build does not handle                 */
    MADI_ERR_GEOMETRY = 6,     /* geometry the classifier cannot prove (RuntimeError)       */
    MADI_ERR_HOST_MEMORY = 7   /* a host allocation failed; size outputs are not written    */
} madi_status;

/* ------------------------------------------------------------------------ */
/* Geometry                                                                 */
/* ------------------------------------------------------------------------ */

enum { MADI_BOUNDARY_FATAL = 0, MADI_BOUNDARY_PERIODIC = 1 };

/*
 * One ensemble resident in device memory.  Built on the host by
 * custom_madi_gb300.ensemble (seeds as in madi/ensemble.py:585-638 and :679,
 * KD tree as in :525-563) and packed into two device buffers:
 *
 *   stage  -- 16-byte aligned block copied whole into shared memory by the
 *             walker when stage_bytes fits; otherwise read in place.
 *             [ seed : float4 x n_seeds ]  x,y,z rounded to fp32, w = alpha (fp32)
 *             [ cell : int32 x n_seeds, padded to 16 bytes ]  base cell id of each seed
 *             [ grid_offset : uint32 x (G^3 + 1), padded to 16 bytes ]
 *             [ grid_ids : uint16 (or uint32 when ids_u32) x grid_total, padded ]
 *   seed_f64 -- double4 x n_seeds: x, y, z, alpha (the exact geometry).
 *   kd_*     -- balanced KD tree over the seeds, node 0 the root, -1 = none.
 *
 * grid_ids of voxel v (voxel edge grid_h) list every seed that can be the
 * nearest seed of, or bind a shifted facet for, any point of the voxel grown by
 * grid_eps, plus every seed whose facet can come within safe_cap of the
 * contracted cell boundary: a proven superset, so the fp32 and fp64 rules run
 * on these lists return the labels of the all-seed rule.
 */
typedef struct madi_geometry {
    const void*    stage;          /* device, 16-byte aligned                     */
    const double*  seed_f64;       /* device, [n_seeds][4]                        */
    const int32_t* kd_seed;        /* device, [n_seeds]                           */
    const int32_t* kd_left;        /* device, [n_seeds]                           */
    const int32_t* kd_right;       /* device, [n_seeds]                           */
    const int32_t* kd_parent;      /* device, [n_seeds]                           */
    const int8_t*  kd_axis;        /* device, [n_seeds]                           */
    uint32_t off_cell;             /* byte offsets inside stage                   */
    uint32_t off_grid_offset;
    uint32_t off_grid_ids;
    uint32_t stage_bytes;          /* multiple of 16                              */
    int32_t  n_seeds;              /* seeds in the arrays (tiled images included) */
    int32_t  grid_n;               /* voxels per axis (G)                         */
    int32_t  ids_u32;              /* 1 when grid_ids are uint32                  */
    int32_t  boundary;             /* MADI_BOUNDARY_*                             */
    int32_t  has_cells;            /* 0 = free water (no membranes)               */
    int32_t  pad0;
    double   L;                    /* walk box edge                               */
    double   grid_h;               /* voxel edge (G * grid_h >= L)                */
    double   safe_cap;             /* extra list radius (0: nearest + binding only) */
    double   source_lo;            /* walkers start uniform in [lo, hi)^3         */
    double   source_hi;
    double   coord_err;            /* bound on |fp32 seed - fp64 seed| per axis   */
    /* Cell facet table (madi_facets_build), byte offsets inside stage; cell c
     * owns slots c * facet_stride .. + facet_stride - 1, unused slots hold
     * (0, 0, 0, 3e38) and neighbour -1.  With n_cells = 0 the walker labels
     * every step with the voxel-grid classifier. */
    uint32_t off_cell_center;      /* float4 [n_cells]: base seed x, y, z, alpha  */
    uint32_t facet_stride;         /* facet slots per cell, a multiple of 32      */
    uint32_t off_facet_plane;      /* float4 [n_cells][facet_stride]: n, offset h */
    uint32_t off_facet_nbr;        /* int32 [n_cells][facet_stride]: cell across  */
    int32_t  n_cells;              /* cells in the table (0 = no table)           */
    int32_t  pad1;
    double   facet_tol;            /* fp32 error of h - n.w, without the |w| term */
} madi_geometry;

/* Replaces Ensemble.classify_cpu (madi/ensemble.py:213-256) and the device
 * classifier _classify_full_facet (madi/walker_gpu.py:272-335).
 * points: device [n][3], fp64 (points_f32 = 0) or fp32 (points_f32 = 1), in
 * [0, L)^3 (periodic points are wrapped by the caller).
 * method 0 = stackless KD traversal in fp64 (the reference rule);
 * method 1 = voxel-grid classifier in fp32 with an fp64 guard-band fallback.
 * cell_out: nearest seed id (periodic: cell id of the seed); inside_out: 0/1;
 * path_out (optional): 0 fp32 decision, 1 fp64 fallback, 2 KD fp64. */
madi_status madi_classify(const madi_geometry* geom, const void* points, int points_f32,
                          int64_t n, int method, int32_t* cell_out, uint8_t* inside_out,
                          uint8_t* path_out, void* stream);

/* ------------------------------------------------------------------------ */
/* Walker                                                                   */
/* ------------------------------------------------------------------------ */

#define MADI_MAX_PAIRS 8
#define MADI_MAX_B 32
#define MADI_MAX_DIRS 32
#define MADI_MAX_GRID 512

enum { MADI_RNG_PHILOX = 0, MADI_RNG_STREAM = 1 };
enum { MADI_OUT_FUSED = 0, MADI_OUT_Y = 1 };

/* One walk job: one ensemble at one membrane probability (one (e, kio) pair of
 * madi/walker_gpu.py:1218-1232), n_walkers walkers. */
typedef struct madi_walk_job {
    int32_t  geom;            /* index into the geometry array                       */
    int32_t  n_walkers;
    uint32_t walker_base;     /* Philox counter of the first walker (CRN identity)   */
    uint32_t key0, key1;      /* Philox key: walk seed (madi/walker_gpu.py:81-83)   */
    int32_t  slot;            /* accumulator slot receiving this job's sums          */
    int32_t  tile_begin;      /* first work tile of this job (prefix over jobs)      */
    int32_t  y_row;           /* first output row in Y / inside_trace (OUT_Y)       */
    double   pp;              /* membrane transmission probability, [0, 1]           */
    uint64_t thr1;            /* floor(pp   * 2^64), accept iff U64 < thr           */
    uint64_t thr2;            /* floor(pp^2 * 2^64)                                  */
} madi_walk_job;

/* Device counters per slot (uint64 each), zeroed by the caller.  FULL:
 * voxel-grid classifications; TIER1: steps labelled from facet planes (label
 * cache or full facet pass); FALLBACK64: fp64 decisions; FACET_PASS: full
 * facet passes (label cache misses). */
enum {
    MADI_CNT_WALKERS = 0, MADI_CNT_ESCAPED, MADI_CNT_CLASSIFIER_ERROR,
    MADI_CNT_FULL, MADI_CNT_TIER1, MADI_CNT_FALLBACK64, MADI_CNT_CROSS_ACCEPT,
    MADI_CNT_CROSS_REJECT, MADI_CNT_FACET_PASS, MADI_CNT_N
};

/*
 * Replaces _walk_kernel + _reduce_kernel (madi/walker_gpu.py:520-695), their
 * launch in _run_walk_one_ensemble / _walk_and_reduce_one_ensemble
 * (:843-951, :989-1063), and the per-ensemble / per-kio loop of
 * run_simulation_multi_kio_reduced (:1218-1232): every job is one work list of
 * walker tiles consumed by one persistent launch.
 *
 * Fused output (out_mode FUSED): for job j, accum[slot][col][dir][2] holds
 * round(2^32 * sum over walkers of cos / sin (coef[col] * u_dir . dM_pair)), an
 * exact 64-bit fixed-point sum (order independent), with
 * dM = Y(delta) + Y(Delta) - Y(Delta + delta) per axis; occupancy[slot][j_grid]
 * counts inside walkers at each Y grid point; counters[slot][MADI_CNT_*].
 *
 * Y output (out_mode Y): Y[y_row + w][j][3] (fp64, reference origin L/2 as in
 * madi/walker_gpu.py:562-564) and inside_trace[y_row + w][j] (int8).
 *
 * rng MADI_RNG_STREAM replays init[w][3], incr[step][w][3], unif[step][w]
 * (WalkRandomStream, madi/walker_gpu.py:86-127), fp64 arrays.
 *
 * precision 64 is the reference's walker design (madi/walker_gpu.py:520-585):
 * one thread per walker of jobs[0], separately rounded fp64 arithmetic, the
 * exact KD rule at every step, Y output only; n_tiles = ceil(n_walkers / 128).
 * With MADI_RNG_PHILOX it evaluates the fp32 walker's Philox numbers in fp64.
 */
typedef struct madi_walk_desc {
    const madi_geometry* geoms;    /* device array                                    */
    const madi_walk_job* jobs;     /* device array                                    */
    int32_t n_geoms, n_jobs;
    int32_t n_tiles;               /* total tiles over all jobs                       */
    int32_t tile_walkers;          /* walkers per tile (= threads per block)          */
    int32_t grid_blocks;           /* persistent CTAs; 0 = one per tile               */
    int32_t stage_smem;            /* max stage_bytes over geoms; 0 = read in place   */
    int32_t boundary;              /* MADI_BOUNDARY_* shared by every geometry        */
    int32_t precision;             /* 32 = fp32 production walker, 64 = fp64 walker   */
    int32_t rng;                   /* MADI_RNG_*                                      */
    int32_t out_mode;              /* MADI_OUT_*                                      */
    int32_t n_steps, steps_per_h, n_grid;
    double  sigma, ts;
    /* fused epilogue */
    int32_t n_pairs, n_b, n_dirs;
    int32_t min_blocks;            /* register budget: 1 = 255 regs, 2 = 128 regs/thread */
    int32_t pair_jd[MADI_MAX_PAIRS], pair_jD[MADI_MAX_PAIRS], pair_js[MADI_MAX_PAIRS];
    float   coef[MADI_MAX_PAIRS * MADI_MAX_B];   /* phase coefficient per (pair, b)  */
    float   dirs[MADI_MAX_DIRS * 3];
    /* outputs */
    int64_t*  accum;               /* [n_slots][n_pairs*n_b][n_dirs][2]               */
    uint64_t* occupancy;           /* [n_slots][n_grid]                               */
    uint64_t* counters;            /* [n_slots][MADI_CNT_N]                           */
    double*   Y;                   /* OUT_Y: [rows][n_grid][3]                        */
    int8_t*   inside_trace;        /* OUT_Y: [rows][n_grid]                           */
    /* replay stream (MADI_RNG_STREAM) */
    const double* init;            /* [n_walkers][3]                                  */
    const double* incr;            /* [n_steps][n_walkers][3]                         */
    const double* unif;            /* [n_steps][n_walkers]                            */
    /* scratch: one zeroed uint32 work counter */
    uint32_t* work_counter;
} madi_walk_desc;

madi_status madi_walk(const madi_walk_desc* desc, void* stream);

/* madi_walk without any caller-provided scratch; no counterpart in the reference.
 * For callers that cannot allocate device memory around a walk: code recording a
 * CUDA graph by stream capture (a cudaMalloc there breaks the capture), plug-in
 * hosts that hand the library only their own pre-sized input and output buffers,
 * and services working from a fixed memory pool with no room left for another
 * buffer.  Same inputs, outputs and results as madi_walk; desc->work_counter is
 * ignored.  The one zeroed word the persistent walk needs comes from a 256-byte
 * static device array that every GPU loading the library holds until the process
 * exits; each call clears it on its stream, all calls share it, and calls that
 * overlap on the GPU race on it (order them on one stream or with events).  The
 * first call on a device resolves the array's address (cudaGetSymbolAddress) and
 * must come before any stream capture.  Walks whose n_tiles + grid_blocks reach
 * 2^31 - 1 are rejected (MADI_ERR_CAPACITY).  Calls no cudaMalloc or cudaFree. */
madi_status madi_walk_noalloc(const madi_walk_desc* desc, void* stream);

/* Upper bound of the dynamic shared memory of one fp32 walker CTA: a staged
 * geometry of stage_bytes, tile_walkers threads, n_grid storage points, at the
 * largest output layout (MADI_MAX_PAIRS x MADI_MAX_B x MADI_MAX_DIRS). */
int64_t madi_walk_smem_bytes(int32_t stage_bytes, int32_t tile_walkers, int32_t n_grid);

/* Resident CTAs per SM of the fp32 walker for this descriptor's shape
 * (tile_walkers threads, stage_smem + epilogue shared memory); 0 on error. */
int32_t madi_walk_blocks_per_sm(const madi_walk_desc* desc);

/* The batched (persistent, work-queue) walk: madi_walk with a persistent grid.
 * grid_blocks == 0 means SMs x madi_walk_blocks_per_sm(desc).  Replaces the
 * per-ensemble launches of _run_walk_one_ensemble (madi/walker_gpu.py:843-953)
 * driven from the ensemble x kio loop (:1218-1232). */
madi_status madi_walk_batched(const madi_walk_desc* desc, void* stream);

/* Replaces _reduce_kernel (madi/walker_gpu.py:658-695) for grids too large for
 * the fused epilogue: Y [n_walkers][n_grid][3] fp64 -> cos_sum / sin_sum
 * [n_cols] fp64, the sums over walkers and the 3 axes of cos / sin(coef dM),
 * dM = Y[jd] + Y[jD] - Y[js] per column (jd, jD, js, coef).  Y is read once per
 * block of 1,024 columns; per-CTA fp64 partials are added as 2^-32 fixed-point
 * integers, so the result is independent of scheduling (each partial rounded
 * once: |error| <= 2^-33 per walker block and column).  scratch: device,
 * 8-byte aligned, madi_reduce_Y_scratch_bytes(n_cols) bytes, no initialisation
 * needed. */
int64_t madi_reduce_Y_scratch_bytes(int32_t n_cols);
madi_status madi_reduce_Y(const double* Y, int64_t n_walkers, int32_t n_grid, const int32_t* jd,
                          const int32_t* jD, const int32_t* js, const double* coef, int32_t n_cols,
                          double* cos_sum, double* sin_sum, void* scratch, int64_t scratch_bytes, void* stream);

/* ------------------------------------------------------------------------ */
/* Library match                                                            */
/* ------------------------------------------------------------------------ */

enum { MADI_MATCH_FIXED_S0 = 0, MADI_MATCH_FREE_S0 = 1 };
enum { MADI_MATCH_FP32 = 0, MADI_MATCH_BF16 = 1 };

/*
 * Replaces _map_kernel_fixed / _map_kernel_free_s0 and their launches
 * (madi/fitters_gpu.py:96-154, :414-463), i.e. the argmin of
 * match_voxels_batch (madi/library.py:1444-1450) and
 * match_voxels_batch_fits0 (:1495-1522).
 *   fixed S0: best = argmin_j (|L_j|^2 - 2 m.L_j), resid = |m|^2 + that
 *   free  S0: best = argmin_j over m.L_j > 0 of |m|^2 - (m.L_j)^2/|L_j|^2
 * Ties pick the lowest library index.
 * FP32: exhaustive fp32 scan on the CUDA cores; fixed S0 scores the pair
 *       centred on the library column mean (same argmin, ~|L|^2/|L-mu|^2
 *       smaller rounding than the uncentred form).
 * BF16: tcgen05 BF16 x BF16 -> FP32 (TMEM) scores, a per-voxel top-k (k of 8,
 *       16, 32) candidate list, then an fp32 rescore of the k candidates.
 *       Fixed S0 (library <= 32768 entries): a first launch over each voxel
 *       tile's nearest library tile pair bounds every voxel's k-th best BF16
 *       residual; each voxel tile then scans only the library tiles that the
 *       principal-axis bound (|m - L| >= |(m - L).pc|, widened by the BF16
 *       rounding of both vectors) leaves possible.  The cut changes the top-k
 *       set only in the choice among entries tied in BF16 score at the k-th
 *       place.
 * measured: device fp32 [n_vox][n_feat]; lib: device fp32 [n_lib][n_feat].
 * scratch: 256-byte aligned device buffer of madi_match_scratch_bytes(...)
 * bytes (contents need no initialisation; FP32 free S0 ignores it).
 */
typedef struct madi_match_desc {
    const float* measured;
    const float* lib;
    int64_t n_vox;
    int32_t n_lib, n_feat;
    int32_t mode;                  /* MADI_MATCH_FIXED_S0 / FREE_S0 */
    int32_t precision;             /* MADI_MATCH_FP32 / BF16       */
    int32_t topk;                  /* BF16 candidates rescored     */
    int32_t flags;                 /* 0, or MADI_MATCH_FLAG_*      */
    int32_t* best_idx;             /* [n_vox]                      */
    float*   best_resid;           /* [n_vox]                      */
    float*   best_s0;              /* [n_vox] (free S0) or NULL    */
    void*    scratch;
    int64_t  scratch_bytes;
} madi_match_desc;

/* Tests only: every CTA of the BF16 scan makes one bounded wait on a barrier
 * that nothing completes, so the timeout path runs (the CTA drains its issued
 * copies and MMAs, frees TMEM, leaves its rows at the caller's fill value) and
 * madi_match_wait reports MADI_ERR_TIMEOUT.  Nothing faults or hangs. */
#define MADI_MATCH_FLAG_TEST_STALL 1
/* BF16 fixed S0: scan every library tile for every voxel (no principal-axis
 * cut); the result is the same up to BF16 score ties at the k-th place. */
#define MADI_MATCH_FLAG_FULL_SCAN 2

int64_t madi_match_scratch_bytes(int64_t n_vox, int32_t n_lib, int32_t n_feat, int32_t precision,
                                 int32_t topk);
madi_status madi_match(const madi_match_desc* desc, void* stream);

/* Completion status of the last madi_match enqueued with this descriptor on
 * `stream` (same scratch; no GB300 counterpart: the reference's Numba launch is
 * synchronous, madi/fitters_gpu.py:414-438).  Synchronizes the stream, then
 * returns MADI_OK; MADI_ERR_TIMEOUT if a bounded wait of the BF16 scan ran out
 * (the rows of the CTAs that gave up keep the value the caller left in
 * best_idx, e.g. -1; every issued copy and MMA was drained before TMEM was
 * freed, unless the message says the drain ran out too); MADI_ERR_CUDA if the
 * stream reports an error.  The FP32 scan has no bounded waits. */
madi_status madi_match_wait(const madi_match_desc* desc, void* stream);

/* ------------------------------------------------------------------------ */
/* Bayesian posterior-mean fit (madi/fitters.py:110-243, the two-pass kernels  */
/* of madi/fitters_gpu.py:156-294 and bayes_fit_gpu :466-528)               */
/* ------------------------------------------------------------------------ */

/* Per voxel, entry j weighs w_j = q_j exp(-rw_j / (2 sigma_m^2)) with rw_j the
 * normalised residual (fixed S0: |m - L_j|^2; free S0: |m/s0_j - L_j|^2 with
 * s0_j = m.L_j / |L_j|^2, entries with s0_j <= 0 weigh 0); q_j = exp(log_weight[j]).
 * out: device fp64 [MADI_BAYES_N_OUT][n_vox] = kio, rho, V posterior means,
 * their standard deviations, the weighted residual (raw units for free S0),
 * n_eff = (sum w)^2 / sum w^2 and (free S0) the weighted S0.  A free-S0 voxel
 * that no entry fits with s0 > 0 gets zeros.  Entries whose weight is below
 * e^-60 of the voxel's largest weight are dropped.  Arithmetic: fp32 scores
 * screen the entries; the kept ones get a direct-difference fp32 residual
 * (error ~F ulp of the residual) and Kahan-compensated fp32 sums of
 * parameter differences from the best entry, combined in fp64.
 * scratch: 256-byte aligned, madi_bayes_scratch_bytes() bytes. */
#define MADI_BAYES_N_OUT 9
typedef struct madi_bayes_desc {
    const float* measured;         /* [n_vox][n_feat] (fixed: normalised; free: raw) */
    const float* lib;              /* [n_lib][n_feat]               */
    const double* log_weight;      /* [n_lib] log quadrature weight */
    const double* kio;             /* [n_lib]                       */
    const double* rho;             /* [n_lib]                       */
    const double* V;               /* [n_lib]                       */
    int64_t n_vox;
    int32_t n_lib, n_feat;
    int32_t mode;                  /* MADI_MATCH_FIXED_S0 / FREE_S0 */
    int32_t pad0;
    double sigma_m;
    double* out;                   /* [MADI_BAYES_N_OUT][n_vox]     */
    void* scratch;
    int64_t scratch_bytes;
} madi_bayes_desc;

int64_t madi_bayes_scratch_bytes(int32_t n_lib, int32_t n_feat);
madi_status madi_bayes(const madi_bayes_desc* desc, void* stream);

/* ------------------------------------------------------------------------ */
/* Host-side geometry builders (native C++; no device work)                 */
/* ------------------------------------------------------------------------ */

/* Balanced KD tree as in _build_gpu_kdtree (madi/ensemble.py:525-563): median
 * on the widest-spread axis, preorder node numbering, root = node 0. */
madi_status madi_kdtree_build(const double* seeds_xyz, int32_t n, int32_t* node_seed,
                              int8_t* node_axis, int32_t* node_left, int32_t* node_right,
                              int32_t* node_parent);

/* Candidate lists of a G^3 voxel grid over [0, G*h)^3 (madi_geometry above).
 * seeds: [n][4] x, y, z, alpha.  Two passes: call with ids == NULL to get
 * *total, then with capacity >= *total (MADI_ERR_CAPACITY with *total set
 * when it is smaller).  MADI_ERR_HOST_MEMORY: the host ran out of memory and
 * *total is not written. */
madi_status madi_grid_build(const double* seeds, int32_t n, int32_t G, double h,
                            double eps, double safe_cap, uint32_t* offsets,
                            void* ids, int32_t ids_u32, int64_t capacity, int64_t* total);

/* Facet table of every cell's Voronoi polytope.  The reference has no
 * counterpart: its classifier searches a KD tree at every step, while the
 * walker labels most steps from the planes of the cell it is in.
 * seeds: [n][4] x, y, z, alpha of the base cells (periodic: in [0, L)^3, the
 * images are generated here).  For cell c and facet k,
 *   m_k(q) = h_k - n_k.(q - c)
 * is the signed distance of q to the bisector plane between c and the cell
 * nbr_k (periodic: q - c is the nearest image).  Every Voronoi facet of the
 * cell is listed; planes that only touch the polytope may be listed too.  Each
 * cell's range begin[c] .. begin[c + 1] is padded to a multiple of 4 with
 * (0, 0, 0, 3e38) and nbr -1.  A cell whose polytope the other seeds do not
 * close within 12 seed spacings (the outer cells of a finite population) gets
 * one padded group with h = -3e38, which sends every step there to the
 * voxel-grid classifier.
 * begin: [n + 1]; planes: [capacity][4] (fp32, n_k then h_k); nbr: [capacity].
 * If capacity < *total the call fails with MADI_ERR_CAPACITY and *total holds
 * the size needed; MADI_ERR_HOST_MEMORY (host out of memory) leaves *total
 * unwritten.  stats (optional, [2]): the largest h over all facets and the
 * largest distance from a seed to a vertex of its closed cell. */
madi_status madi_facets_build(const double* seeds, int32_t n, int32_t periodic, double L,
                              uint32_t* begin, float* planes, int32_t* nbr,
                              int64_t capacity, int64_t* total, double* stats);

/* ------------------------------------------------------------------------ */
/* Serving loop (no counterpart in the reference)                           */
/* ------------------------------------------------------------------------ */

/* Continuous batching of simulation requests over madi_walk.  Requests are
 * admitted in submission order while their declared device bytes fit the
 * budget and an output slot is free; active requests are cut into
 * tile-aligned walker chunks and every launch takes the next chunk of each
 * active request (round robin, up to launch_walkers), up to `inflight`
 * launches on server-owned streams.  A request's sums land in its slot row of
 * the pools given in `walk` (accum/occupancy/counters) and are bit-identical
 * however it was chunked or mixed.  Not thread-safe across servers sharing
 * pools; calls on one server are serialised internally. */
typedef struct madi_serve_config {
    madi_walk_desc walk;           /* template: fused Philox walk; geoms/jobs/n_* /grid_blocks/work_counter
                                      are the server's, accum/occupancy/counters = [n_slots] pools */
    int32_t n_slots;
    int32_t chunk_walkers;         /* multiple of walk.tile_walkers */
    int32_t launch_walkers;        /* >= chunk_walkers */
    int32_t inflight;              /* 1..4 launches in flight */
    int64_t budget_bytes;          /* device bytes admitted requests may hold together */
    void*   arena;                 /* device, 256-byte aligned, madi_serve_arena_bytes() bytes */
    int64_t arena_bytes;
} madi_serve_config;

typedef struct madi_serve_request {
    madi_geometry geometry;        /* device pointers valid until the request is released */
    double   pp;
    uint32_t seed;                 /* Philox key word 0 */
    uint32_t pad0;
    int64_t  n_walkers;
    int64_t  nbytes;               /* device bytes the request holds while admitted */
} madi_serve_request;

typedef struct madi_serve_done {
    int64_t request_id;
    int32_t slot;                  /* row of the pools holding the result */
    int32_t pad0;
    double  submit_s, admit_s, finish_s;   /* seconds since madi_serve_create */
} madi_serve_done;

int64_t madi_serve_arena_bytes(const madi_serve_config* cfg);
madi_status madi_serve_create(const madi_serve_config* cfg, void** server);
madi_status madi_serve_submit(void* server, const madi_serve_request* req, int64_t* request_id);
/* Non-blocking: admits, launches, reaps finished launches; reports up to
 * max_done finished requests (each once) and the number still queued or active. */
madi_status madi_serve_poll(void* server, int32_t max_done, madi_serve_done* done, int32_t* n_done,
                            int32_t* n_pending);
/* The caller has read request_id's slot: its slot and bytes return to the pool. */
madi_status madi_serve_release(void* server, int64_t request_id);
madi_status madi_serve_destroy(void* server);

/* ------------------------------------------------------------------------ */
/* Autotuner cache (no counterpart in the reference)                        */
/* ------------------------------------------------------------------------ */

/* Launch shape of the batched walk chosen for one workload class. */
typedef struct madi_launch_shape {
    int32_t tile_walkers;          /* 0: no entry for the key        */
    int32_t blocks_per_sm;         /* 0: occupancy-derived           */
    int32_t min_blocks;            /* register budget (1 or 2)       */
    int32_t stage_budget;          /* bytes; 0: geometry read in place */
    double  walker_steps_per_s;    /* rate measured when stored      */
} madi_launch_shape;

/* Text file of "key<TAB>tile<TAB>bps<TAB>minb<TAB>stage<TAB>rate" lines; keys hold
 * no tab or newline.  load: an absent file or key gives tile_walkers = 0.
 * store: replaces or appends the key, written to path.tmp then renamed (the
 * parent directory is created).  Thread-safe within a process. */
madi_status madi_autotune_load(const char* path, const char* key, madi_launch_shape* out);
madi_status madi_autotune_store(const char* path, const char* key, const madi_launch_shape* shape);

/* ------------------------------------------------------------------------ */
/* Misc                                                                     */
/* ------------------------------------------------------------------------ */
int32_t madi_abi_version(void);
const char* madi_last_error_string(void);

#ifdef __cplusplus
}
#endif
#endif /* MADI_GB300_H */
