// Kernel argument blocks and launchers of the sweep and field kernels.
// Included by the CUDA translation units and by the host runtime (capi.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "local_solver.cuh"

namespace eikx {

// Warp-block shape of the 3D kernel: LY3 x LZ3 x-pencils per warp.
constexpr int LY3 = 8, LZ3 = 4;
// 2D kernel: 32 x-rows per warp.
constexpr int LZ2 = 32;
constexpr int kWarpsPerBlock = 4;

// Device state shared by all sweeps of one solve (one entry per field unless noted).
struct SolveState {
    unsigned *queue[2];             // work-queue heads, double-buffered across sweeps
    unsigned long long *mbox;       // per warp block: its downstream faces, tagged words
    unsigned *epoch;                // [0] sweep-tag base, advanced by the reset of each solve
                                    // past the tags of the previous one; [1] tags it used
    int epochStride;                // tags this solve uses (sweep launches + 1)
    unsigned long long *residual;   // [field][sweep slot] largest decrease (double bits)
    int residualStride;             // slots per field
    int *converged;                 // 1 once a field's iteration decrease fell below tol
    int *sweepsRun;                 // refinement sweeps each field ran
    int *abortFlag;                 // raised when a bounded wait ran out
    const int4 *order;              // work queue: (field, by, bz, 0) sorted by start step
    int totalItems;                 // fields * warp blocks per field
    unsigned long long spinLimit;   // polls before a wait gives up
};

// Geometry of one work unit (one field on one model) of a multi-model batch: the grids of
// a batch may differ in size and spacing; a warp reads its unit's entry per work item.
template <class T> struct Grid3Unit {
    T *tt;                        // this field's travel times, row pitch Px
    const T *spPos, *spNeg;       // the model's padded slowness copies
    unsigned long long *mbox;     // this field's mailbox (tilesY * tilesZ warp blocks)
    long long spPlane;            // spPitch * (ny + 1)
    int spPitch, Px, nx, ny, nz, tilesY, tilesZ, pad;
    T h;                          // uniform spacing
    Spacing3<T> sp3;              // non-uniform constants
};

template <class T> struct Sweep3Args {
    T *tt;                    // travel-time fields, row pitch `pitch`, rows (y,z) natural
    long long fieldStride;    // elements per field
    int pitch;                // padded x extent Px (multiple of 4) = walk length
    const T *spPos;           // edge-replicated slowness, columns shifted by 3 (+x sweeps)
    const T *spNeg;           // edge-replicated slowness, unshifted (-x sweeps)
    int spPitch;              // row pitch of both (multiple of 4, >= Px + 8)
    long long spPlane;        // spPitch * (ny + 1)
    int nx, ny, nz;
    int tilesY, tilesZ;       // warp blocks per field along y', z'
    const SourceT<T> *srcs;   // per field
    SolveState st;
    int buf;                  // which queue head this sweep uses
    int sweepIndex;           // position of this sweep in the solve (its mailbox tag offset)
    int residualSlot;         // residual slot this sweep writes
    int sweep;                // 0..7 = Sweep1..Sweep8
    int init;                 // 1 = source-limited initialisation sweep
    int radius;               // factored-eikonal radius
    T h;                      // uniform spacing
    Spacing3<T> sp3;          // non-uniform constants
    const int2 *pairs;        // field pairs of the paired kernel (work items index pairs)
    const Grid3Unit<T> *units;  // multi-model batch: per-unit geometry (chunk-step kernel only)
    const SourceFp64 *srcs64; // per field, FP32 chunk-step only: set = the FP64 factored branch
                              // (eikx_options.near_fp64), its own kernel instances
    // A stream of sources through slots (chunk-step, one model; eikx_options.max_in_flight):
    // set = field f is a slot whose current source started at sweep slots[f].x of the stream
    // (-1 = idle) in field buffer slots[f].y; sweepIndex is this sweep's position in the
    // stream and `sweep` its ordering (sweepIndex mod 8).
    const int2 *slots;
    int initSweeps;           // 1 = a slot's first 8 sweeps are its initialisation pass
    // FP64 chunk-step kernel on a uniform grid, one model (required there): the padded
    // slowness copies multiplied by h (launchPadSlowness3 with h), laid out as spPos / spNeg,
    // and the model's natural-order cell slowness for the factored branch (FP64 cells, or FP32
    // cells with cells64 = 0)
    const T *hsPos, *hsNeg;
    const void *cells;
    int cells64;
};

template <class T> struct Sweep2Args {
    T *tt;
    long long fieldStride;
    int pitch;                // Px
    const T *spPos;           // (nz+1) x spPitch, columns shifted by 3 (+x sweeps)
    const T *spNeg;           // unshifted (-x sweeps)
    int spPitch;
    int nx, nz;
    int tilesZ;
    const SourceT<T> *srcs;
    SolveState st;
    int buf;
    int sweepIndex;
    int residualSlot;
    int sweep;                // 0..3 = Sweep1..Sweep4
    int init;
    int radius;
    T h;
    Spacing2<T> sp2;
};

// Launchers (sweep.cu).  blocks = persistent grid size.
template <class T>
cudaError_t launchSweep3(const Sweep3Args<T> &a, bool uniform, int blocks, cudaStream_t s);
template <class T>
cudaError_t launchSweep2(const Sweep2Args<T> &a, bool uniform, int blocks, cudaStream_t s);
// 2D grids of at most kMaxBlockRows2 rows: one CTA per field, one thread per row.
constexpr int kMaxBlockRows2 = 512;
template <class T>
cudaError_t launchSweep2Block(const Sweep2Args<T> &a, bool uniform, int nFields, cudaStream_t s);
// Chunk-step 3D kernel (sweep_chunk.cuh): a lane updates one 16-byte chunk of its pencil
// per wavefront step.  With a.units set, a work item's field index is a unit of a
// multi-model batch and the grid, slowness, mailbox and spacing come from a.units[unit].
// Warp-block shapes (pencils per warp along y' x z'), one translation unit each.
enum ChunkShape { kShape8x4 = 0, kShape4x8 = 1, kShape16x2 = 2, kNumShapes = 3 };
constexpr int shapeLY(int shape) { return shape == kShape4x8 ? 4 : shape == kShape16x2 ? 16 : 8; }
constexpr int shapeLZ(int shape) { return shape == kShape4x8 ? 8 : shape == kShape16x2 ? 2 : 4; }
#define EIKX_DECLARE_CHUNK_SHAPE(LY_, LZ_)                                                        \
    template <class T>                                                                            \
    cudaError_t launchSweep3Chunk_##LY_##x##LZ_(const Sweep3Args<T> &a, bool uniform, int blocks, \
                                                cudaStream_t s);                                  \
    template <class T> int sweep3ChunkBlocksPerSM_##LY_##x##LZ_(bool uniform, bool batch);
EIKX_DECLARE_CHUNK_SHAPE(8, 4)
EIKX_DECLARE_CHUNK_SHAPE(4, 8)
EIKX_DECLARE_CHUNK_SHAPE(16, 2)
#undef EIKX_DECLARE_CHUNK_SHAPE
template <class T>
inline cudaError_t launchSweep3Chunk(const Sweep3Args<T> &a, bool uniform, int shape, int blocks, cudaStream_t s) {
    if (shape == kShape4x8) return launchSweep3Chunk_4x8<T>(a, uniform, blocks, s);
    if (shape == kShape16x2) return launchSweep3Chunk_16x2<T>(a, uniform, blocks, s);
    return launchSweep3Chunk_8x4<T>(a, uniform, blocks, s);
}
template <class T> inline int sweep3ChunkBlocksPerSM(bool uniform, bool batch, int shape) {
    if (shape == kShape4x8) return sweep3ChunkBlocksPerSM_4x8<T>(uniform, batch);
    if (shape == kShape16x2) return sweep3ChunkBlocksPerSM_16x2<T>(uniform, batch);
    return sweep3ChunkBlocksPerSM_8x4<T>(uniform, batch);
}
// 3D sweep kernel variants (eikx_options.sweep_kernel).
enum Sweep3Variant { kNodeStep = 1, kChunkStep = 2 };
// Paired 3D kernel (sweep_pair.cu): FP32, uniform grid, two fields of one model per lane.
cudaError_t launchSweep3Pair(const Sweep3Args<float> &a, int blocks, cudaStream_t s);
int sweep3PairBlocksPerSM();
size_t sweep3PairSmemBytes();
// Resident blocks per SM of the sweep kernels (for the persistent grid size).
template <class T> int sweep3BlocksPerSM(bool uniform);
template <class T> int sweep2BlocksPerSM(bool uniform);
size_t sweep3SmemBytes(size_t elem);
size_t sweep2SmemBytes(size_t elem);

// Field kernels (fields.cu).
struct Corner3 {
    int isx, isy, isz;
    double xo, yo, zo, s;     // source offsets and source-cell slowness (FP64)
};
template <class T>
cudaError_t launchInit3(T *tt, int nFields, long long fieldStride, int pitch, int nx, int ny, int nz,
                        double dx, double dy, double dz, const Corner3 *corners, int fp64,
                        cudaStream_t s);
template <class T>
cudaError_t launchInit2(T *tt, int nFields, long long fieldStride, int pitch, int nx, int nz,
                        double dx, double dz, const Corner3 *corners, int fp64, cudaStream_t s);
// Edge-replicated slowness: element (pz, py, i) = S[clamp(pz-1), clamp(py-1), clamp(i-1-shift)],
// in T; with h > 0 each element is then multiplied by h (in T).
template <class T, class U>
cudaError_t launchPadSlowness3(T *sp, int spPitch, int shift, const U *s, int nx, int ny, int nz,
                               cudaStream_t st, T h = 0);
template <class T, class U>
cudaError_t launchPadSlowness2(T *sp, int spPitch, int shift, const U *s, int nx, int nz, cudaStream_t st);
template <class U>
cudaError_t launchNodalToCell3(double *slow, const U *v, int nx, int ny, int nz, int ordering,
                               cudaStream_t s);
template <class U>
cudaError_t launchNodalToCell2(double *slow, const U *v, int nx, int nz, int ordering, cudaStream_t s);
template <class U>
cudaError_t launchCellsToNatural3(double *slow, const U *c, int nx, int ny, int nz, int ordering,
                                  cudaStream_t s);
template <class U>
cudaError_t launchCellsToNatural2(double *slow, const U *c, int nx, int nz, int ordering, cudaStream_t s);
cudaError_t launchResetState(const SolveState &st, int nFields, int buf, cudaStream_t s);
// Warm start of a 3D solve: the initial fields (natural order) into the pitched fields,
// nodes the local solver shows underestimated reset to HUGE (count added to *nReset),
// the source cells' corners initialised analytically.
template <class T>
cudaError_t launchWarmInit3(T *tt, const T *init, int nFields, long long fieldStride, int pitch, int nx, int ny, int nz,
                            double dx, double dy, double dz, const Corner3 *corners, const SourceT<T> *srcs,
                            const double *slow, int radius, bool uniform, T h, const Spacing3<T> &g, double gateTol,
                            int twoSided, int fp64, const SourceFp64 *srcs64, unsigned long long *nReset,
                            cudaStream_t s);
// Fills the FP64 analytic-factor table of each field whose SourceFp64 has one.
cudaError_t launchFactorTables(const SourceFp64 *srcs, int nFields, cudaStream_t s);
// Box of a field's factor table: the nodes within `radius` of the source cell along every
// axis (the factored branch's nodes), clamped to the grid; false when 8 sweeps x the box
// exceed kMaxFactorTable entries.
inline bool factorBox(int isx, int isy, int isz, int radius, int nx, int ny, int nz, int (&o)[3], int (&e)[3]) {
    const int c[3] = {isx, isy, isz}, n[3] = {nx, ny, nz};
    const long long r = radius;
    long long vol = 8;
    for (int k = 0; k < 3; ++k) {
        const long long lo = c[k] - r < 0 ? 0 : c[k] - r;
        const long long hi = c[k] + r > n[k] - 1 ? n[k] - 1 : c[k] + r;
        o[k] = static_cast<int>(lo);
        e[k] = static_cast<int>(hi - lo + 1);
        vol *= e[k];
    }
    return vol <= kMaxFactorTable;
}
// Sets *flag (ORs 1) if any of the n slownesses is not positive and finite.
cudaError_t launchCheckPositive(const double *s, long long n, int *flag, cudaStream_t st);
cudaError_t launchCheckPositive(const float *s, long long n, int *flag, cudaStream_t st);
// After refinement sweep `sweepsDone - 1`: a field whose residual slots
// [firstSlot, firstSlot + nSlots) all fell below tol is frozen (later sweeps skip it).
// Stream mode (eikx_options.max_in_flight): the convergence test after sweep `sweepIndex`
// of the stream, per slot; and the refill of the listed slots with their new sources
// (field buffer := HUGE, source-cell corners, residual row, flag and sweep count cleared).
cudaError_t launchCheckStream(const SolveState &st, const int2 *slots, int nSlots, int sweepIndex, int initSweeps,
                              double tol, cudaStream_t s);
template <class T>
cudaError_t launchRefillSlots(T *tt, long long fieldStride, int pitch, int nx, int ny, int nz, double dx, double dy,
                              double dz, const SolveState &st, const int2 *slots, const int *list, int n,
                              const Corner3 *corners, int fp64, cudaStream_t s);
cudaError_t launchCheckConvergence(const SolveState &st, int nFields, int firstSlot, int nSlots,
                                   int sweepsDone, double tol, cudaStream_t s);
// 2D gradient ray tracing (rays.cu): grid, source, step rules and output capacity.
constexpr int kMaxRadii = 16;
struct RayTrace2Args {
    int nx, nz;
    double dx, dz, x0, z0;
    const double *slow;           // cell slowness (nz-1) x (nx-1), FP64, device
    int isx, isz;                 // source cell
    double xs, zs;                // source offsets from the origin
    int nRsf;                     // radius / scale pairs, ascending radius (the last applies beyond)
    int rsfRadius[kMaxRadii];
    double rsfScale[kMaxRadii];
    int maxSteps;                 // bound on the march (march points per station: maxSteps + 1)
    int capacity;                 // segments per station
};
template <class T>
cudaError_t launchTraceRays2(const RayTrace2Args &a, const T *grad, int n, const double *stations, double *pos,
                             double *segments, int *counts, cudaStream_t s);

// Products of a solved field (post.cu): the travel-time gradient (3 or 2 values per
// natural node) and travel times at stations (cells and origin offsets per station).
template <class T>
cudaError_t launchGradient(const T *tt, int dim, int Px, int nx, int ny, int nz, double dx, double dy, double dz,
                           const Corner3 &src, T *grad, cudaStream_t s);
template <class T>
cudaError_t launchStations(const T *tt, int dim, int Px, int ny, double dx, double dy, double dz, const Corner3 &src,
                           int n, const int *cells, const double *offs, double *out, cudaStream_t s);
cudaError_t launchAnalytic3(double *t, int nx, int ny, int nz, double dx, double dy, double dz,
                            double xs, double ys, double zs, double vTop, double vBottom, cudaStream_t s);
cudaError_t launchAnalytic2(double *t, int nx, int nz, double dx, double dz, double xs, double zs,
                            double vTop, double vBottom, cudaStream_t s);

// Self-test of the Cartesian operator's lower-bound shortcuts (post.cu): n random stencils
// at the shortcuts' edges; counts[0..3] += evaluated, mismatches of min(t0, .) against
// fd3UniformFar, shortcut results equal to t0, stencils whose t0 is the operator's value.
cudaError_t launchOperatorSelftest(int precision, long long n, unsigned long long seed, unsigned long long *counts,
                                   cudaStream_t s);

// Rows of `width` bytes from a pitched source to a pitched destination: one contiguous copy
// when neither has padding (a 2D copy of many short rows moves them row by row), else a 2D
// copy.
inline cudaError_t copyRows(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, size_t height,
                            cudaMemcpyKind kind, cudaStream_t s) {
    if (dpitch == width && spitch == width) return cudaMemcpyAsync(dst, src, width * height, kind, s);
    return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, kind, s);
}

}  // namespace eikx
