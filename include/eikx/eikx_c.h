/*
 * eikx_c.h -- the C ABI of the GB300-native eikonal solver.
 *
 * This is the drop-in boundary for the level-set fast-sweeping path of
 * uofuseismo/eikonalxx v0.2.0.  Every call takes plain pointers and sizes; no
 * CUDA or C++ types cross it.  The C++ API in include/eikonalxx/ (Solver3D,
 * Solver2D, Model3D, ... with the reference's names and exceptions) is a thin
 * layer over these entry points, and a Python, Go (cgo), Java (JNI/Panama) or
 * Node (N-API) binding can bind them directly.
 *
 * Conventions
 *   - Grids are node-based: nx*ny*nz travel-time nodes, (nx-1)*(ny-1)*(nz-1)
 *     slowness cells, natural order (x fastest, then y, then z), exactly as
 *     include/private/grid.hpp:15-53 of the reference.
 *   - Every entry point returns an eikx_status (0 = success).  On failure the
 *     thread-local message from eikx_last_error() says why.
 *   - A context owns one CUDA device, its stream, device buffers and the CUDA
 *     graphs of the sweep schedules it has run.  Contexts are independent; one
 *     context must not be used from two threads at once (as the reference's
 *     solvers, which are not thread-safe).
 *   - Solves are synchronous: when eikx_solve* returns, the output is written.
 */
#ifndef EIKX_C_H
#define EIKX_C_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct eikx_ctx eikx_ctx;
typedef int eikx_status;

enum {
    EIKX_OK = 0,
    EIKX_ERR_INVALID = -1,     /* bad argument: maps to std::invalid_argument */
    EIKX_ERR_STATE = -2,       /* call out of order: maps to std::runtime_error */
    EIKX_ERR_CUDA = -3,        /* CUDA runtime error (device missing, launch failed) */
    EIKX_ERR_TIMEOUT = -4,     /* a bounded inter-tile wait ran out; field not valid */
    EIKX_ERR_ALLOC = -5,       /* device or host allocation failed */
    EIKX_ERR_UNSUPPORTED = -6  /* option combination not supported */
};

enum { EIKX_F32 = 0, EIKX_F64 = 1 };                 /* arithmetic / storage type */
enum { EIKX_ORDER_NATURAL = 0, EIKX_ORDER_TRANSPOSED = 1 }; /* Ordering3D::ZYX / XYZ */
enum { EIKX_HOST = 0, EIKX_DEVICE = 1 };             /* where a pointer lives */

/* Solver options.  The first four mirror SolverOptions
 * (include/eikonalxx/solverOptions.hpp:11-111, defaults src/solverOptions.cpp:5-21). */
typedef struct {
    int n_sweeps;          /* refinement iterations, each = all 8 (3D) / 4 (2D) sweeps; default 5 */
    double tolerance;      /* s; a field stops once each of its last 8 (3D) / 4 (2D)
                              refinement sweeps decreased no node by this or more (a window
                              that slides sweep by sweep across iterations; the reference
                              stores the tolerance but never applies it); <= 0 runs all
                              n_sweeps iterations, as the reference does; default 1e-5 */
    int factored_radius;   /* factored-eikonal radius in grid points; default 3 */
    int init_sweeps;       /* 1 = run the source-limited initialisation pass first; default 1 */
    int init_fp64;         /* 1 = source-corner times computed in FP64 then rounded to the
                              field type (default); 0 = in the field type, as the reference */
    int spin_limit_log2;   /* bound on each inter-tile wait: 2^n polls (0 = default 22) */
    int test_drop_blocks;  /* test hook, 0 in production: the host leaves the first n warp
                              blocks of the work queue out, so the blocks downstream of them
                              wait on progress that never comes; their bounded waits run
                              out and the solve returns EIKX_ERR_TIMEOUT (the context stays
                              usable).  Exercises failure detection without a GPU fault. */
    int profile_sweeps;    /* 1 = run the schedule without the CUDA graph and time every sweep
                              kernel with CUDA events (eikx_stats.sweep_ms); 0 = graph replay */
    int pair_fields;       /* 1 = FP32 uniform-grid batches of >= 2 fields run two fields per
                              GPU lane (shared slowness work, packed FP32 math); 0 (default)
                              = one field per lane, measured faster on GB300 at every batch
                              size (the paired kernel needs 168 registers per thread, which
                              leaves 12 resident warps per SM).  Both give identical times. */
    int sweep_kernel;      /* 3D sweep kernel: 0 (default) = the tuned kernel of this grid class
                              if eikx_autotune3d ran, else chunk-step; 1 = node-step (a
                              lane updates one node per wavefront step), 2 = chunk-step (a
                              lane updates one 16-byte chunk, 4 FP32 / 2 FP64 nodes, per
                              step).  2D: 0 and 1 = warp blocks of 32 rows; 2 = one CTA
                              per field, one thread per row (grids of up to 512 rows; slower
                              on GB300, whose FP64 units one SM cannot keep fed).  All give
                              identical travel times. */
    int block_shape;       /* 3D chunk-step warp block (pencils along y' x z'): 0 (default) =
                              the tuned shape of this grid class if eikx_autotune3d ran, else
                              8x4; 1 = 8x4, 2 = 4x8, 3 = 16x2.  Identical travel times. */
    int blocks_per_sm;     /* persistent sweep grid: resident blocks per SM; 0 (default) = as
                              many as fit (or the tuned value) */
    int test_tag_margin;   /* test hook, 0 in production: before the first solve of a context,
                              start the 32-bit sweep-tag base this many tags below 2^32, so
                              that the next few solves cross the wrap-around (the host then
                              clears the mailbox and restarts the base at 1) */
    int near_fp64;         /* 3D FP32 solves: 1 = the factored (near-source) branch forms its
                              analytic factor in FP64: the distance D = |x - xs| and direction
                              (x - xs) / D from FP64 offsets and spacing (tabulated once per
                              solve around each source), T0 = s0 D with s0 the node's cell
                              slowness, its gradient, the differences tau = t - T0 at the 7
                              upwind neighbours and the candidate T0 + correction, each
                              rounded to FP32; the quadratic solves stay in FP32.  0 (default)
                              = all in FP32, as the reference's sweep type.  Runs on the
                              chunk-step kernel (sweep_kernel and pair_fields give way).
                              Ignored by FP64 solves and 2D. */
    int warm_gate;         /* eikx_solve3d_warm's residual gate: 0 (default) = reset nodes
                              whose initial time lies more than gate_tol below the smallest
                              upwind update of their initial neighbourhood (one-sided);
                              1 = also reset nodes more than gate_tol above it (two-sided) */
    int max_in_flight;     /* eikx_solve3d: 0 (default) = all sources in one batch; 0 < n <
                              n_src = a stream: n slots, each solving one source at a time;
                              a slot whose field has converged (or reached n_sweeps) is
                              copied out and takes the next source at the next iteration
                              boundary, its initialisation sweeps running inside the same
                              launches as the other slots' refinement sweeps.  The fields
                              are bit-identical to solving each source alone.  Chunk-step
                              kernel (sweep_kernel and pair_fields give way); no CUDA graph
                              (the schedule follows convergence); the fields do not stay on
                              the device for eikx_gradient3d / eikx_station_times3d. */
    int reserved;
} eikx_options;

/* Fills *opt with the defaults above. */
void eikx_options_default(eikx_options *opt);

/* A source (or, by reciprocity, a station) at an absolute position in metres.
 * Its cell is min(nCell-1, floor((x-x0)/dx)) per axis, as Source3D
 * (src/source3d.cpp:161-297). */
typedef struct { double x, y, z; } eikx_source3d;
typedef struct { double x, z; } eikx_source2d;

/* Per-solve statistics of the last eikx_solve3d/2d call on a context. */
typedef struct {
    int n_fields;            /* fields solved by the call */
    int iterations_max;      /* largest number of refinement iterations any field began */
    int iterations_min;
    int sweeps_launched;     /* sweep kernels launched (init pass included) */
    int kernel_launches;     /* all kernels launched by the call (graph nodes included) */
    double residual_last;    /* largest decrease over each field's last 8 (3D) / 4 (2D)
                                refinement sweeps, over all fields (s) */
    double device_ms;        /* device time of the solve incl. the copy-out (CUDA events) */
    double sweep_ms;         /* summed device time of the sweep kernels (profile_sweeps), else -1 */
    long long reset_nodes;   /* warm start: initial nodes reset as underestimated (else 0) */
    long long refine_node_updates;  /* node updates of the refinement sweeps actually run: nodes
                                       x refinement sweeps, summed over the fields (a field
                                       that has converged is skipped, so fields differ) */
} eikx_stats;

/* ---- context ----------------------------------------------------------- */
/* Replaces: the implicit per-solver state of Solver3D/Solver2D
 * (src/solver3d.cpp:16-111 Solver3DImpl, src/solver2d.cpp:28-225 Solver2DImpl). */
eikx_status eikx_create(eikx_ctx **ctx, int device);
eikx_status eikx_destroy(eikx_ctx *ctx);
const char *eikx_last_error(void);
eikx_status eikx_get_stats(const eikx_ctx *ctx, eikx_stats *stats);

/* ---- 3D ---------------------------------------------------------------- */
/* Replaces Solver3D::initialize (src/solver3d.cpp:148-194): grid points (>= 3 per
 * axis, include/eikonalxx/geometry3d.hpp / src/geometry3d.cpp:73-80), spacing (> 0)
 * and origin. */
eikx_status eikx_set_grid3d(eikx_ctx *ctx, int nx, int ny, int nz, double dx, double dy,
                            double dz, double x0, double y0, double z0);

/* Replaces Solver3D::setVelocityModel (src/solver3d.cpp:197-249) with a model given
 * as cell slowness (s/m, as Model3D::getSlownessPointer, src/model3d.cpp:407-415).
 * dtype: EIKX_F32/F64; ordering: natural or transposed; where: host or device. */
eikx_status eikx_set_slowness3d(eikx_ctx *ctx, const void *slowness, int dtype, int ordering,
                                int where);

/* Replaces Model3D::setNodalVelocities (src/model3d.cpp:286-314) + setVelocityModel:
 * nodal velocities (m/s) -> cell slowness 8/sum(8 corners) computed on the GPU. */
eikx_status eikx_set_nodal_velocity3d(eikx_ctx *ctx, const void *velocity, int dtype,
                                      int ordering, int where);

/* Copies the cell slowness the context holds (natural order) to host memory. */
eikx_status eikx_get_slowness3d(const eikx_ctx *ctx, void *slowness, int dtype);

/* Replaces Solver3D::setSource + Solver3D::solve + getTravelTimeField
 * (src/solver3d.cpp:351-500, :503-525).  Solves n_src independent fields (one per
 * source) on the context's model in one batched launch schedule.
 * precision: EIKX_F32 (FP32 sweeps, FP64 corner init) or EIKX_F64.
 * t_out: n_src * nx*ny*nz values of the precision's type, natural order, host or
 * device (where).  opt may be NULL for the defaults. */
eikx_status eikx_solve3d(eikx_ctx *ctx, const eikx_source3d *src, int n_src,
                         const eikx_options *opt, int precision, void *t_out, int where);

/* ---- 2D ---------------------------------------------------------------- */
/* No counterpart in the reference: a 3D solve warm-started from initial fields, one per
 * source (natural order, the solve precision, host or device by init_where) -- e.g. a
 * learned prediction inflated to bound the solution from above.  A node whose initial
 * time lies more than gate_tol seconds below the smallest upwind update its initial
 * neighbourhood gives, over all 8 sweep orderings, is reset to HUGE (sweeps only lower
 * times, so it could not recover); a corner of a source cell keeps the smaller of its
 * initial value and the analytic initialisation (the cold start's sweeps may lower it
 * below the analytic value, so a converged field is a fixed point of the warm start), or
 * takes the analytic value when the gate rejects it; then refinement iterations run to
 * the tolerance without the initialisation pass.  eikx_stats.reset_nodes counts the
 * resets.  Note: the reference's local solver is not monotone in its neighbours (the
 * causality windows of the 2D and 3D operators, the factored branch): raising a
 * neighbour can lower a node.  Sweeps started from any field other than the cold
 * start's own result -- even that result inflated by 0.1 % -- can settle on a different
 * fixed point, by milliseconds on layered models. */
eikx_status eikx_solve3d_warm(eikx_ctx *ctx, const eikx_source3d *src, int n_src, const eikx_options *opt,
                              int precision, const void *t_init, int init_where, double gate_tol, void *t_out,
                              int where);

/* ---- products of the last solve ---------------------------------------- */

/* Travel-time gradient of field `field` (0-based source index) of the last eikx_solve3d /
 * eikx_solve2d on this context, in that solve's precision, natural node order,
 * interleaved per node: (dT/dx, dT/dy, dT/dz) in 3D, (dT/dx, dT/dz) in 2D.  Replaces
 * Solver2D::computeTravelTimeGradientField (src/solver2d.cpp:865-879) with the
 * reference's central-difference scheme (src/gradient.hpp:20-289): central differences
 * inside, second-order one-sided differences on the first and last node of each axis,
 * the analytic constant-slowness gradient at the corners of the source cell; the 3D
 * gradient, declared but never computed by the reference's Solver3D, applies the same
 * rule per axis.  grad: 3 (2) * nodes values, host or device (where). */
eikx_status eikx_gradient3d(eikx_ctx *ctx, int field, void *grad, int where);
eikx_status eikx_gradient2d(eikx_ctx *ctx, int field, void *grad, int where);

/* Travel times of field `field` of the last solve at stations given by their positions
 * (m): a station in the source cell gets |x - x_s| * s_src, any other the trilinear (3D:
 * x, then y, then z) / bilinear (2D) interpolation of its cell's corner times, in FP64.
 * Replaces Solver2D::interpolateTravelTimes (src/solver2d.cpp:106-167); the reference's
 * Solver3D stores stations but computes no times.  times: n host doubles. */
eikx_status eikx_station_times3d(eikx_ctx *ctx, int field, const eikx_source3d *stations, int n, double *times);
eikx_status eikx_station_times2d(eikx_ctx *ctx, int field, const eikx_source2d *stations, int n, double *times);

/* ---- 2D gradient ray tracing ---------------------------------------------- */
/* Step rule of Ray::GradientTracerOptions (include/eikonalxx/ray/gradientTracerOptions.hpp,
 * src/ray/gradientTracerOptions.cpp): where the ray is within radius[k] cells of the source
 * cell (the smaller of the x and z cell distances) it steps scale[k] * min(dx, dz).  The
 * pairs are sorted by radius; when the largest radius is below INT_MAX a pair (INT_MAX,
 * last scale) is added, as setRadiusScaleFactor does. */
typedef struct {
    int n_radii;           /* pairs used, 1..16 */
    int radius[16];        /* non-negative, distinct */
    double scale[16];      /* in (machine epsilon, 1) */
    int max_steps;         /* bound on one ray's march; 0 = ceil(4 (nx + nz) / smallest scale) + 16
                              (the reference has no bound) */
    int reserved;
} eikx_ray_options;

/* Defaults of GradientTracerOptions: (1, 0.05), (2, 0.10), (3, 0.20), (5, 0.30), (INT_MAX, 0.45). */
void eikx_ray_options_default(eikx_ray_options *opt);

/* One segment of a ray path (Ray::Segment2D, include/eikonalxx/ray/segment2d.hpp). */
typedef struct {
    double x0, z0, x1, z1; /* start and end point, absolute (m) */
    double slowness;       /* s/m of the cell the segment crosses */
    int cell;              /* velocity-model cell index, or -1 where the reference leaves it unset */
    int reserved;
} eikx_ray_segment2d;

/* Replaces Ray::GradientTracer2D::trace (src/ray/gradientTracer2d.cpp:339-600): a ray from
 * each station to the source, marched down the travel-time gradient (bilinear in the
 * current cell) until it ends within one cell of the source cell, then healed into
 * segments that end where the ray leaves a cell, source to station; a station in the
 * source cell gets the straight segment.  One GPU thread per station, FP64.
 *   grid: nx x nz nodes, spacing dx, dz, origin x0, z0 (Geometry2D);
 *   gradient: host array of nz x nx x 2 values (d/dx, d/dz per node, natural order),
 *     dtype EIKX_F32 or EIKX_F64 (ISolver2D::getTravelTimeGradientFieldPointer);
 *   slowness: host array of (nz-1) x (nx-1) cell slownesses, FP64;
 *   source, stations: absolute positions (m), stations as n (x, z) pairs;
 *   segments: n x capacity entries, station i's path in [i * capacity, ...);
 *   counts[i]: segments of station i, or -1 when the march did not reach the source within
 *     max_steps (the reference prints "did not converge"), -2 when the path needs more than
 *     capacity segments, -3 when the march left the grid (where the reference reads outside
 *     its arrays).
 * The call succeeds (EIKX_OK) when some rays fail; counts tell which. */
eikx_status eikx_trace_rays2d(eikx_ctx *ctx, int nx, int nz, double dx, double dz, double x0, double z0,
                              const void *gradient, int dtype, const double *slowness, double source_x,
                              double source_z, const double *stations, int n_stations, const eikx_ray_options *opt,
                              int capacity, eikx_ray_segment2d *segments, int *counts);

/* ---- autotuning ---------------------------------------------------------- */

/* The configuration eikx_autotune3d chose for one grid class. */
typedef struct {
    int sweep_kernel;              /* 1 = node-step, 2 = chunk-step */
    int pair_fields;               /* 1 = two FP32 fields per lane */
    int block_shape;               /* 1 = 8x4, 2 = 4x8, 3 = 16x2 (chunk-step) */
    int blocks_per_sm;             /* resident blocks per SM of the persistent grid */
    double ms_per_sweep;           /* measured mean sweep launch of the choice */
    double default_ms_per_sweep;   /* the untuned default (chunk-step, 8x4, full grid) */
    int candidates;                /* configurations timed */
} eikx_tuning;

/* No counterpart in the reference.  Times the sweep kernels, warp-block shapes and grid
 * sizes on the context's 3D model with these sources -- one refinement iteration per
 * candidate, CUDA events around every sweep launch, each candidate run twice and the
 * second run kept -- and records the fastest for the grid class (precision, uniform
 * spacing, nx, ny, nz rounded up to multiples of 32, source count rounded up to a power
 * of two).  Later eikx_solve3d calls of the same class whose options leave sweep_kernel,
 * block_shape and blocks_per_sm at 0 and pair_fields at 0 use it.  All candidates give
 * identical travel times. */
eikx_status eikx_autotune3d(eikx_ctx *ctx, const eikx_source3d *src, int n_src, int precision,
                            eikx_tuning *out);
/* Writes the context's tuning table to `path` (one JSON object per line) / merges the
 * table at `path` into the context. */
eikx_status eikx_tuning_save(const eikx_ctx *ctx, const char *path);
eikx_status eikx_tuning_load(eikx_ctx *ctx, const char *path);

/* ---- multi-model batch ------------------------------------------------- */

/* One model of a multi-model batch and the sources to solve on it. */
typedef struct {
    int nx, ny, nz;               /* grid points (>= 3 each) */
    double dx, dy, dz;            /* spacing (m, > 0) */
    double x0, y0, z0;            /* origin (m) */
    const void *model;            /* cell slowness ((nx-1)(ny-1)(nz-1) values, s/m) or nodal
                                     velocity (nx*ny*nz values, m/s), as model_kind says */
    int model_kind;               /* EIKX_CELL_SLOWNESS or EIKX_NODAL_VELOCITY */
    int dtype;                    /* EIKX_F32 / EIKX_F64 of `model` */
    int ordering;                 /* EIKX_ORDER_NATURAL / EIKX_ORDER_TRANSPOSED of `model` */
    int where;                    /* EIKX_HOST / EIKX_DEVICE of `model` */
    int n_src;                    /* sources on this model (>= 1) */
    const eikx_source3d *src;     /* host array of n_src source positions (m) */
    void *t_out;                  /* n_src * nx*ny*nz values of the solve precision, natural order */
    int t_where;                  /* EIKX_HOST / EIKX_DEVICE of t_out */
} eikx_model3d;
enum { EIKX_CELL_SLOWNESS = 0, EIKX_NODAL_VELOCITY = 1 };

/* No single counterpart in the reference: a loop of Solver3D::setVelocityModel +
 * setSource + solve (src/solver3d.cpp:197-249, :351-525) over many models, run as one
 * schedule.  Every (model, source) field of the batch is a work unit of the same
 * persistent sweep launches, whatever the grid sizes; models with uniform spacing and
 * models with non-uniform spacing run as two schedules.  Fields are identical to
 * eikx_solve3d on each model alone.  Uses the chunk-step sweep kernel; the context's own
 * model (eikx_set_slowness3d) is not touched.  eikx_get_stats reports the batch. */
eikx_status eikx_solve3d_batch(eikx_ctx *ctx, const eikx_model3d *models, int n_models,
                               const eikx_options *opt, int precision);

/* Replaces Solver2D::initialize (src/solver2d.cpp:291-343). */
eikx_status eikx_set_grid2d(eikx_ctx *ctx, int nx, int nz, double dx, double dz, double x0,
                            double z0);
/* Replaces Solver2D::setVelocityModel (src/solver2d.cpp:406-438). */
eikx_status eikx_set_slowness2d(eikx_ctx *ctx, const void *slowness, int dtype, int ordering,
                                int where);
/* Replaces Model2D::setNodalVelocities (src/model2d.cpp:263-290). */
eikx_status eikx_set_nodal_velocity2d(eikx_ctx *ctx, const void *velocity, int dtype,
                                      int ordering, int where);
/* Replaces Solver2D::setSource + Solver2D::solve + getTravelTimeField
 * (src/solver2d.cpp:462-565, :883-905). */
eikx_status eikx_solve2d(eikx_ctx *ctx, const eikx_source2d *src, int n_src,
                         const eikx_options *opt, int precision, void *t_out, int where);

/* ---- level-set tables (host) ------------------------------------------- */
/* Replaces Graph3D<E>::initialize and its accessors (src/graph3d.cpp:120-317):
 * sweep = 0..7 (Sweep1..Sweep8).  Arrays: level_start[nx+ny+nz-1],
 * node_to_index/to_x/to_y/to_z/index_to_level[nx*ny*nz].  Returns the number of
 * levels (> 0) or an eikx_status (< 0). */
int eikx_graph3d_tables(int sweep, int nx, int ny, int nz, int *level_start,
                        int *node_to_index, int *to_x, int *to_y, int *to_z,
                        int *index_to_level, int *max_level_size);

/* Replaces the 2D level helpers makeLevelOffset / sweepLevelIndexToGrid
 * (solverUtilities2d.hpp:1063-1266): the (ix, iz) visiting order of sweep 0..3.
 * Arrays: level_start[nx+nz], order_ix/order_iz[nx*nz].  Returns the number of
 * levels or an eikx_status. */
int eikx_levels2d(int sweep, int nx, int nz, int *level_start, int *order_ix, int *order_iz);

/* ---- analytic fields on the GPU (FP64) ---------------------------------- */
/* Replaces Analytic::LinearGradient3D::solve / Homogeneous3D::solve
 * (src/analytic/linearGradient3d.cpp:28-116, homogeneous3d.cpp:22-70): travel times
 * for v(z) = vTop + (vBottom-vTop)*z/((nz-1)dz) (vTop == vBottom: homogeneous) on the
 * context's 3D grid.  t_out: nx*ny*nz doubles, host or device. */
eikx_status eikx_analytic3d(eikx_ctx *ctx, const eikx_source3d *src, double v_top,
                            double v_bottom, double *t_out, int where);
eikx_status eikx_analytic2d(eikx_ctx *ctx, const eikx_source2d *src, double v_top,
                            double v_bottom, double *t_out, int where);

/* ---- solve without allocating ------------------------------------------ */
/* No counterpart in the reference: an addition of this library for callers that must
 * not allocate GPU memory while they run -- hosts whose framework owns every device
 * allocation through its own pool, real-time pipelines that forbid allocation after
 * start-up, code running where cudaMalloc would synchronise or is not allowed.
 * One FP32 3D field (FP64 corner initialisation) is solved with the sweep schedule of
 * eikx_solve3d; every intermediate buffer lives in a fixed 64 MiB array compiled into
 * the library, so once the array is resident the call makes no cudaMalloc, cudaFree or
 * other allocating call.
 *   slowness: device pointer, (nx-1)(ny-1)(nz-1) cell slownesses (s/m), natural order;
 *             checked on the device like eikx_set_slowness3d (a non-positive or
 *             non-finite value returns EIKX_ERR_INVALID before any sweep runs).
 *   src, opt: host pointers (opt may be NULL for the defaults).  The options are checked
 *             as eikx_solve3d checks them; sweep_kernel, block_shape and blocks_per_sm
 *             are honoured, and the value 0 means the untuned default (chunk-step
 *             kernel, 8x4 warp blocks, full occupancy): there is no context, so no
 *             autotuned choice applies.
 *   t_out:    device pointer, nx*ny*nz travel times, natural order.
 *   stream:   a cudaStream_t (NULL = the legacy default stream); the call returns when
 *             the field is written.
 * Residency: under CUDA's default lazy module loading the driver reserves the array (and
 * loads the sweep kernels) on a device the first time this function runs there; with
 * CUDA_MODULE_LOADING=EAGER it does so when the library is loaded.  That device then
 * holds the array until the process exits.  A caller that cannot allocate makes one
 * warm-up call per device at start-up, before its own memory pool takes the device's
 * memory and before any stream capture; that first call also looks up the array's
 * device address and clears it.
 * Limit: a grid needs about 15 bytes of the array per node (padded fields, two slowness
 * copies, block-face mailbox); larger grids -- beyond about 4 million nodes -- return
 * EIKX_ERR_INVALID without running.  All calls on a device share the array and it keeps
 * the last call's contents (each solve clears what must start at zero); calls that
 * overlap on the GPU race and must be serialised by the caller. */
eikx_status eikx_solve3d_noalloc(int nx, int ny, int nz, double dx, double dy, double dz,
                                 double x0, double y0, double z0, const float *slowness,
                                 const eikx_source3d *src, const eikx_options *opt,
                                 float *t_out, void *stream);

/* ---- learned warm start: the travel-time predictor -------------------------- */
/* No counterpart in the reference.  A 3D U-Net predicts the factored correction
 * tau = T / T0 - 1 of a travel-time field from its velocity model and source, where
 * T0 = s_src * |x - x_s| and s_src is the slowness (1/v) at the node nearest the source,
 * in FP32 (the offsets from the source are FP64 differences rounded to FP32).  Its
 * prediction, inflated, is an initial field for eikx_solve3d_warm.  Grids with 128 nodes
 * along x run the first level's convolutions on tcgen05 (TMA staging, TMEM accumulators),
 * the rest on mma.sync.
 *
 * Network (channels-last BF16 activations [sample][z][y][x][channel], BF16 weights,
 * FP32 accumulation on the tensor cores, FP32 master weights and Adam state):
 *   input features (16 channels, 6 used): s/s_src - 1, |x - x_s| / L, (x - x_s) / L,
 *     (y - y_s) / L, (z - z_s) / L, with L the length of the grid's diagonal, and the
 *     straight-ray estimate of tau: the mean of s/s_src - 1 at 32 midpoints of the
 *     segment from the source to the node (s trilinear in the nodal 1/v, FP32);
 *   encoder: two 3x3x3 convolutions + ReLU per level, 16, 32, 64 channels, 2x2x2 average
 *     pooling between levels; bottleneck: two convolutions with 128 channels;
 *   decoder: nearest 2x upsampling, concatenation with the encoder level, two
 *     convolutions + ReLU (64, 32, 16 channels); head: 1x1x1 convolution to tau.
 *   Zero padding at the grid's faces.  1,466,065 parameters.  The loss is the mean of
 *   (tau_pred - tau)^2 over the nodes with T0 > 0.
 * Parameters are one FP32 vector: per convolution (in the order above: E0a, E0b, E1a,
 * E1b, E2a, E2b, Ba, Bb, D2a, D2b, D1a, D1b, D0a, D0b) its weights [27 taps][out][in]
 * (tap = (dz*3 + dy)*3 + dx, the input node offset (dz-1, dy-1, dx-1)) then its biases
 * [out]; then the head's 16 weights and its bias.  E0a takes 16 input channels, of
 * which the last 10 are zero. */
typedef struct eikx_warmnet eikx_warmnet;

typedef struct {
    int nx, ny, nz;        /* node grid; each a multiple of 8 */
    double dx, dy, dz;     /* grid spacing (m); positive and finite */
    double x0, y0, z0;     /* origin (m); finite */
    int batch;             /* largest number of samples per call; at least 1 */
    unsigned long long seed;   /* initial weights (He-normal convolutions, zero biases and head) */
} eikx_warmnet_config;

/* One sample: DEVICE pointers to its nodal velocity model (nx*ny*nz FP32, m/s, natural
 * order) and, for training, its solved travel-time field (same layout; NULL when only
 * predicting), and the source position (m). */
typedef struct {
    const float *velocity;
    const float *travel_time;
    double x, y, z;
} eikx_warmnet_sample;

eikx_status eikx_warmnet_create(int device, const eikx_warmnet_config *cfg, eikx_warmnet **net);
eikx_status eikx_warmnet_destroy(eikx_warmnet *net);
eikx_status eikx_warmnet_num_params(const eikx_warmnet *net, long long *n);
/* Copy the FP32 parameter vector out of / into the network (host pointers).  Setting it
 * also resets the Adam state and its step count. */
eikx_status eikx_warmnet_get_params(eikx_warmnet *net, float *params);
eikx_status eikx_warmnet_set_params(eikx_warmnet *net, const float *params);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8, learning rate lr) on n samples
 * (1 <= n <= batch); loss: the loss before the step. */
eikx_status eikx_warmnet_train_step(eikx_warmnet *net, const eikx_warmnet_sample *s, int n, float lr,
                                    double *loss);
/* The loss and its gradient with respect to the parameter vector (host, num_params
 * floats) on n samples, without updating the network. */
eikx_status eikx_warmnet_gradients(eikx_warmnet *net, const eikx_warmnet_sample *s, int n, float *grads,
                                   double *loss);
/* Predicted travel times T0 * (1 + tau_pred) * inflate for n samples: n*nx*ny*nz FP32,
 * natural order, host or device (where).  Also the forward pass a loss evaluation uses:
 * loss (may be NULL) receives the loss when every sample has a travel_time. */
eikx_status eikx_warmnet_predict(eikx_warmnet *net, const eikx_warmnet_sample *s, int n, double inflate,
                                 float *t_out, int where, double *loss);
/* Device time (ms, CUDA events on the network's stream) of one training step on n
 * samples, split into forward convolutions, input-gradient convolutions, weight-gradient
 * kernels and everything else, and the algorithmic tensor-core FLOPs of each of the
 * first three (2 * nodes * 27 * in * out per convolution and sample).  The step updates
 * the network.  ms and flops: 4 and 3 doubles. */
eikx_status eikx_warmnet_profile_step(eikx_warmnet *net, const eikx_warmnet_sample *s, int n, float lr,
                                      double *ms, double *flops);
/* Test hook of the tcgen05 convolutions' bounded mbarrier waits (0, 0 in production).
 * spin_limit_log2: a wait gives up after 2^n polls (0 = the default, 2^24).  late = 1:
 * the first input chunk's operand barrier expects 16 bytes more than its copies bring,
 * and the kernel declares them complete only after the wait ran out; late = 2: the
 * first chunk's MMA completion is committed only after the wait ran out.  Either way
 * the wait runs out while every copy and MMA still completes: the kernel then drains
 * them (a second wait, 64 times as long) before it frees TMEM and leaves, and the call
 * returns EIKX_ERR_TIMEOUT; the next call on the network is correct.  Exercises failure
 * detection without a GPU fault. */
eikx_status eikx_warmnet_set_test_hooks(eikx_warmnet *net, int spin_limit_log2, int late);

/* Self-test of the 3D sweep's operator shortcuts on device `device`: n seeded random
 * stencils, built to sit at the shortcuts' edges (node times a few units in the last place
 * from the operator's value, neighbour differences at the 2D windows' limits, homogeneous
 * slowness, unreached neighbours), are evaluated by the uniform-grid Cartesian operator with
 * and without its lower-bound exits and gated operators, in precision EIKX_F32 or EIKX_F64.
 * counts[0] = stencils evaluated, counts[1] = stencils where min(t0, result) differs in any
 * bit (0 when the shortcuts are exact), counts[2] = results equal to t0, counts[3] = stencils
 * whose t0 is the operator's own value.  A test of the sweep kernels' arithmetic; it
 * allocates 32 bytes of device memory for the call. */
eikx_status eikx_selftest_operator3d(int device, int precision, long long n, unsigned long long seed,
                                     long long counts[4]);

#ifdef __cplusplus
}
#endif
#endif /* EIKX_C_H */
