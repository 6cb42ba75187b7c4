// Host runtime behind the C ABI (include/eikx/eikx_c.h).
//
// A context holds the model (cell slowness, FP64 master copy on the device plus an
// edge-replicated copy in each sweep precision), the solve workspace and the CUDA
// graph of the last sweep schedule.  A solve is: upload the per-field source table,
// replay (or capture, then replay) the schedule graph -- reset, corner
// initialisation, the source-limited pass, nSweeps refinement iterations each
// followed by the convergence check -- and copy the fields out with one pitched copy.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <limits>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

#include "eikx/eikx_c.h"
#include "sweep.h"

namespace {

thread_local std::string gLastError;

eikx_status fail(eikx_status code, const std::string &msg) {
    gLastError = msg;
    return code;
}

#define EIKX_CUDA(expr)                                                                      \
    do {                                                                                      \
        cudaError_t e_ = (expr);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(e_ == cudaErrorMemoryAllocation ? EIKX_ERR_ALLOC : EIKX_ERR_CUDA,     \
                        std::string(#expr) + ": " + cudaGetErrorString(e_));                  \
    } while (0)

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&p, n ? n : 16);
        if (e == cudaSuccess) bytes = n; else p = nullptr;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class X> X *as() const { return static_cast<X *>(p); }
    ~DevBuf() { release(); }
};

struct PinnedBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMallocHost(&p, n ? n : 16);
        if (e == cudaSuccess) bytes = n; else p = nullptr;
        return e;
    }
    ~PinnedBuf() { if (p) cudaFreeHost(p); }
};

int roundUp(int v, int m) { return (v + m - 1) / m * m; }

// Cell index and offset of a coordinate, as Source3D::setLocationInX
// (src/source3d.cpp:161-185): offset = x - x0, cell = min(nCell-1, int(offset/dx)).
bool locate(double x, double x0, double d, int n, int *cell, double *offset) {
    const double x1 = x0 + static_cast<double>(n - 1) * d;
    if (!(x >= x0 && x <= x1)) return false;
    *offset = x - x0;
    *cell = std::min(n - 2, static_cast<int>(*offset / d));
    return true;
}

// Convergence test after refinement sweep j (counted over all refinement iterations from 0):
// a field stops once each of its last nSweepKinds refinement sweeps decreased no node by tol
// or more.  The window slides sweep by sweep and may span two iterations; the first full
// window ends with the first iteration.  Slot nSweepKinds + j holds sweep j's residual.
cudaError_t checkAfterSweep(const eikx::SolveState &st, int nFields, int nSweepKinds, int j, double tol,
                            cudaStream_t s) {
    const int lo = std::max(0, j - (nSweepKinds - 1));
    return eikx::launchCheckConvergence(st, nFields, nSweepKinds + lo, j - lo + 1, j + 1,
                                        j >= nSweepKinds - 1 ? tol : -1.0, s);
}

// The host's copy of a workspace's sweep-tag base.  The device's reset kernel advances the
// base by the previous solve's tag count at the start of every solve; the host repeats that
// step and, before a solve whose 32-bit tags would wrap (and so could meet words an early
// solve left in the mailbox), clears the mailbox and restarts the base at 1.
struct EpochMirror {
    unsigned long long base = 0, last = 0;
};

struct Workspace {
    DevBuf tt, mbox, epoch, queue, residual, converged, iterations, abortFlag, order, srcs, corners, pairs, init,
        resetCount, srcs64, factor;
    EpochMirror epochMirror;
    PinnedBuf stage;
    std::vector<int> orderKey;   // (tilesY, tilesZ, nFields, dim) of the uploaded order table
};

// Buffers of a stream of sources through slots (eikx_options.max_in_flight): field buffers
// for the slots plus those whose copy-out is in flight, per-slot mailbox and control words,
// the slot table, and the FP64 factor tables of every source of the stream.
struct StreamWorkspace {
    DevBuf tt, mbox, epoch, queue, residual, converged, iterations, abortFlag, order, srcs, corners, slots, list,
        srcs64, srcs64All, factor;
    EpochMirror epochMirror;
    PinnedBuf stage, flags;
    std::vector<int> orderKey;
    std::vector<cudaEvent_t> bufEv;   // per field buffer: its copy-out has finished
    cudaEvent_t boundary = nullptr;   // the end of an iteration on the solve stream
};

// Buffers of multi-model batches (eikx_solve3d_batch): every model's fields, padded
// slowness and mailbox packed into one allocation each, plus the cached schedule graph.
struct BatchWorkspace {
    DevBuf tt, sp, mbox, epoch, queue, residual, converged, iterations, abortFlag, order, srcs, corners, units,
        slow64, input, badFlag, srcs64, factor;
    EpochMirror epochMirror;
    PinnedBuf stage, srcCells, iterFlags;
    std::vector<double> key;                 // what the cached graph was captured for
    cudaGraphExec_t exec = nullptr;
    int launches = 0;
    void dropGraph() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        key.clear();
    }
    ~BatchWorkspace() { dropGraph(); }
};

struct ScheduleKey {
    int dim = 0, precision = -1, nFields = 0, nx = 0, ny = 0, nz = 0, nSweeps = -1, radius = 0,
        initSweeps = 0, initFp64 = 0, uniform = 0, blocks = 0, dropBlocks = 0, paired = 0, variant = 0, shape = 0,
        warm = 0, early = 0, nearFp64 = 0, warmGate = 0;
    double tol = 0, h = 0, dx = 0, dy = 0, dz = 0, gate = 0;
    unsigned long long spin = 0;
    const void *tt = nullptr, *sp = nullptr, *srcs = nullptr, *corners = nullptr, *flags = nullptr;
    bool operator==(const ScheduleKey &o) const { return std::memcmp(this, &o, sizeof(*this)) == 0; }
};

// Grid class of the tuning table: precision, uniform spacing, extents rounded up to
// multiples of 32, source count rounded up to a power of two.
struct TuneKey {
    int precision, uniform, nx, ny, nz, nsrc;
    bool operator<(const TuneKey &o) const {
        return std::tie(precision, uniform, nx, ny, nz, nsrc) < std::tie(o.precision, o.uniform, o.nx, o.ny, o.nz, o.nsrc);
    }
};
TuneKey tuneKey(int precision, bool uniform, int nx, int ny, int nz, int nSrc) {
    int p2 = 1;
    while (p2 < nSrc) p2 <<= 1;
    return TuneKey{precision, uniform ? 1 : 0, (nx + 31) / 32 * 32, (ny + 31) / 32 * 32, (nz + 31) / 32 * 32, p2};
}

}  // namespace

struct eikx_ctx {
    int device = 0;
    int numSMs = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // copying fields to the host as they converge: a second stream, one event per refinement
    // iteration of the schedule, and the converged flags read back after each iteration
    cudaStream_t copyStream = nullptr;
    cudaEvent_t copyDone = nullptr;
    std::vector<cudaEvent_t> iterEv;
    PinnedBuf iterFlags;
    std::vector<cudaEvent_t> sweepEv;   // per-sweep timing (profile_sweeps)
    StreamWorkspace sw;                 // stream mode (eikx_options.max_in_flight)
    // 3D model
    int nx = 0, ny = 0, nz = 0;
    double dx = 0, dy = 0, dz = 0, x0 = 0, y0 = 0, z0 = 0;
    bool haveGrid3 = false, haveSlow3 = false;
    DevBuf slow3;                  // natural-order cell slowness, FP64
    mutable std::vector<double> hostSlow3;   // host copy, fetched when first asked for
    mutable bool hostSlow3Valid = false;
    DevBuf spad3[2][2];            // [precision][0: shifted for +x sweeps, 1: unshifted]
    bool spadValid3[2] = {false, false};
    DevBuf shad3[2][2];            // the same multiplied by h (uniform grids, FP64 chunk-step kernel)
    bool shadValid3[2] = {false, false};
    // 2D model
    int nx2 = 0, nz2 = 0;
    double dx2 = 0, dz2 = 0, x02 = 0, z02 = 0;
    bool haveGrid2 = false, haveSlow2 = false;
    DevBuf slow2;
    mutable std::vector<double> hostSlow2;
    mutable bool hostSlow2Valid = false;
    DevBuf modelFlag;              // raised by the device checks of a new model
    DevBuf rayGrad, raySlow, raySt, rayPos, raySeg, rayCnt;   // eikx_trace_rays2d buffers
    PinnedBuf srcSlow;             // source-cell slownesses of a solve, read from the device
    DevBuf spad2[2][2];
    bool spadValid2[2] = {false, false};
    DevBuf scratch;                // staging for host inputs and analytic fields
    Workspace ws;
    BatchWorkspace bw;
    std::map<TuneKey, eikx_tuning> tuning;   // eikx_autotune3d results per grid class
    // the last eikx_solve3d / eikx_solve2d: its fields stay in ws.tt (row pitch Px)
    struct {
        bool valid = false;
        int dim = 0, precision = -1, nSrc = 0, nx = 0, ny = 0, nz = 0, Px = 0;
        long long fieldStride = 0;
        double dx = 0, dy = 0, dz = 0, x0 = 0, y0 = 0, z0 = 0;
        std::vector<eikx::Corner3> corners;      // source cell, offsets, source-cell slowness
    } last;
    DevBuf postBuf;                          // gradient / station staging
    DevBuf tuneOut;                          // fields written while tuning
    eikx_stats stats{};
    // cached schedule graph
    ScheduleKey graphKey;
    cudaGraphExec_t graphExec = nullptr;
    int graphLaunches = 0;
    bool useGraphs = true;
};

namespace {

// Before a solve using `stride` tags: the host's mirror of the reset kernel's update of the
// tag base, clearing the mailbox (and the base) when the tags would pass 2^32.
eikx_status advanceEpoch(EpochMirror &m, DevBuf &mbox, DevBuf &epoch, int stride, cudaStream_t s) {
    unsigned long long next = m.base + m.last + 1;
    if (next + static_cast<unsigned long long>(stride) >= (1ull << 32)) {
        EIKX_CUDA(cudaMemsetAsync(mbox.p, 0, mbox.bytes, s));
        EIKX_CUDA(cudaMemsetAsync(epoch.p, 0, 2 * sizeof(unsigned), s));
        m.base = m.last = 0;
        next = 1;
    }
    m.base = next;
    m.last = static_cast<unsigned long long>(stride);
    return EIKX_OK;
}

void dropGraph(eikx_ctx *c) {
    if (c->graphExec) cudaGraphExecDestroy(c->graphExec);
    c->graphExec = nullptr;
    c->graphKey = ScheduleKey{};
}

// Work-queue order: warp blocks of all fields sorted by the step at which they can start
// (by*LY + bz*LZ); every block's upstream blocks come before it.
std::vector<int> buildOrder(int tilesY, int tilesZ, int nFields, int ly, int lz) {
    struct Item { int key, f, b, c; };
    std::vector<Item> items;
    items.reserve(static_cast<size_t>(tilesY) * tilesZ * nFields);
    for (int c = 0; c < tilesZ; ++c)
        for (int b = 0; b < tilesY; ++b)
            for (int f = 0; f < nFields; ++f) items.push_back({b * ly + c * lz, f, b, c});
    std::stable_sort(items.begin(), items.end(), [](const Item &a, const Item &b) {
        if (a.key != b.key) return a.key < b.key;
        if (a.f != b.f) return a.f < b.f;
        return a.b < b.b;
    });
    std::vector<int> out(items.size() * 4);
    for (size_t i = 0; i < items.size(); ++i) {
        out[4 * i] = items[i].f;
        out[4 * i + 1] = items[i].b;
        out[4 * i + 2] = items[i].c;
        out[4 * i + 3] = 0;
    }
    return out;
}

eikx_status checkCtx(const eikx_ctx *c) {
    if (!c) return fail(EIKX_ERR_INVALID, "context is NULL");
    return EIKX_OK;
}

// Copies n elements of type U from `src` (host or device) into device buffer `dst`.
template <class U>
eikx_status toDevice(eikx_ctx *c, const U *src, size_t n, int where, const U **devPtr) {
    if (where == EIKX_DEVICE) {
        *devPtr = src;
        return EIKX_OK;
    }
    EIKX_CUDA(c->scratch.ensure(n * sizeof(U)));
    EIKX_CUDA(cudaMemcpyAsync(c->scratch.p, src, n * sizeof(U), cudaMemcpyHostToDevice, c->stream));
    *devPtr = c->scratch.as<U>();
    return EIKX_OK;
}

// A new model is checked on the device (the input was checked by setCells into the same
// flag): every cell slowness must be positive and finite.  Only the flag comes back; the
// host copy of the model is fetched when eikx_get_slowness asks for it.  The cached
// schedule graph stays valid: it holds buffer addresses, and the padded copies are rebuilt
// before the next launch.
eikx_status finishModel(eikx_ctx *c, int dim) {
    const size_t nCell = dim == 3 ? static_cast<size_t>(c->nx - 1) * (c->ny - 1) * (c->nz - 1)
                                  : static_cast<size_t>(c->nx2 - 1) * (c->nz2 - 1);
    const DevBuf &slow = dim == 3 ? c->slow3 : c->slow2;
    EIKX_CUDA(eikx::launchCheckPositive(slow.as<double>(), static_cast<long long>(nCell), c->modelFlag.as<int>(),
                                        c->stream));
    int bad = 0;
    EIKX_CUDA(cudaMemcpyAsync(&bad, c->modelFlag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    EIKX_CUDA(cudaStreamSynchronize(c->stream));
    if (dim == 3) {
        c->haveSlow3 = false;
        c->hostSlow3Valid = false;
        c->spadValid3[0] = c->spadValid3[1] = false;
        c->shadValid3[0] = c->shadValid3[1] = false;
    } else {
        c->haveSlow2 = false;
        c->hostSlow2Valid = false;
        c->spadValid2[0] = c->spadValid2[1] = false;
    }
    if (bad) return fail(EIKX_ERR_INVALID, "Non-positive velocities detected");
    (dim == 3 ? c->haveSlow3 : c->haveSlow2) = true;
    return EIKX_OK;
}

// The host copy of the cell slowness (natural order, FP64), fetched once per model.
eikx_status hostSlowness(const eikx_ctx *c, int dim, const std::vector<double> **out) {
    std::vector<double> &h = dim == 3 ? c->hostSlow3 : c->hostSlow2;
    bool &valid = dim == 3 ? c->hostSlow3Valid : c->hostSlow2Valid;
    if (!valid) {
        const size_t nCell = dim == 3 ? static_cast<size_t>(c->nx - 1) * (c->ny - 1) * (c->nz - 1)
                                      : static_cast<size_t>(c->nx2 - 1) * (c->nz2 - 1);
        h.resize(nCell);
        EIKX_CUDA(cudaSetDevice(c->device));
        EIKX_CUDA(cudaMemcpyAsync(h.data(), (dim == 3 ? c->slow3 : c->slow2).p, nCell * sizeof(double),
                                  cudaMemcpyDeviceToHost, c->stream));
        EIKX_CUDA(cudaStreamSynchronize(c->stream));
        valid = true;
    }
    *out = &h;
    return EIKX_OK;
}

template <class T> eikx::Spacing3<T> spacing3(double dx, double dy, double dz);
template <class T> int precOf();
template <> int precOf<float>() { return EIKX_F32; }
template <> int precOf<double>() { return EIKX_F64; }

// FP64 analytic factor of an FP32 sweep (eikx_options.near_fp64): the source offsets and
// the grid spacing in FP64, the model's unshifted padded FP32 slowness the table is filled
// from, and the field's factor-table box (its entries are laid out by assignFactorTables).
eikx::SourceFp64 sourceFp64(const std::array<double, 3> &off, int isx, int isy, int isz, int radius, int nx, int ny,
                            int nz, double dx, double dy, double dz, const float *spNeg, int spPitch) {
    eikx::SourceFp64 f{};
    f.xs = off[0]; f.ys = off[1]; f.zs = off[2];
    f.dx = dx; f.dy = dy; f.dz = dz;
    f.sp = spNeg;
    f.spPitch = spPitch;
    f.spPlane = static_cast<long long>(spPitch) * (ny + 1);
    f.ncx = nx - 1; f.ncy = ny - 1; f.ncz = nz - 1;
    int o[3], e[3];
    if (eikx::factorBox(isx, isy, isz, radius, nx, ny, nz, o, e)) {
        f.bx0 = o[0]; f.by0 = o[1]; f.bz0 = o[2];
        f.bnx = e[0]; f.bny = e[1]; f.bnz = e[2];
    }
    return f;
}
// Lays the fields' factor tables (8 sweep orderings x box) out in `buf`, grown as needed,
// and points each record at its table.  Records whose box is too large keep a null table.
cudaError_t assignFactorTables(std::vector<eikx::SourceFp64> &recs, DevBuf &buf) {
    size_t total = 0;
    for (const auto &f : recs) total += 8 * static_cast<size_t>(f.bnx) * f.bny * f.bnz;
    if (total == 0) return cudaSuccess;
    if (cudaError_t e = buf.ensure(total * sizeof(eikx::NearFactor)); e != cudaSuccess) return e;
    size_t off = 0;
    for (auto &f : recs) {
        const size_t n = 8 * static_cast<size_t>(f.bnx) * f.bny * f.bnz;
        f.table = n ? buf.as<eikx::NearFactor>() + off : nullptr;
        off += n;
    }
    return cudaSuccess;
}

// A stream of sources through S = o.max_in_flight slots (3D, chunk-step).  Each slot solves
// one source at a time in one of S + S/2 field buffers; the sweeps run iteration by
// iteration (8 launches, each followed by the per-slot convergence test), and at each
// iteration boundary the host reads the slots' flags: a field that converged (or ran
// n_sweeps iterations) is copied out on the copy stream, and its slot takes the next source
// in a free buffer.  A slot's sweep k of its own schedule runs ordering k mod 8 (sources
// start at iteration boundaries), so every field runs exactly the sweeps of a solve of its
// source alone.
template <class T>
eikx_status solveStream3(eikx_ctx *c, const eikx_options &o, int nSrc, const std::vector<eikx::SourceT<T>> &srcT,
                         const std::vector<eikx::SourceFp64> &srcT64In, const std::vector<eikx::Corner3> &corners,
                         bool uniform, int shape, void *tOut, int where, DevBuf *spad) {
    StreamWorkspace &w = c->sw;
    DevBuf *shad = c->shad3[sizeof(T) == 4 ? EIKX_F32 : EIKX_F64];   // uniform FP64 grids: the scaled copies
    const int nx = c->nx, ny = c->ny, nz = c->nz;
    const double dx = c->dx, dy = c->dy, dz = c->dz;
    const int Px = roundUp(nx, 4), spPitch = Px + 8;
    const long long fieldStride = static_cast<long long>(Px) * ny * nz;
    const int S = o.max_in_flight;
    const int nBufs = S + (S + 1) / 2;
    const int ly = eikx::shapeLY(shape), lz = eikx::shapeLZ(shape);
    const int tilesY = (ny + ly - 1) / ly, tilesZ = (nz + lz - 1) / lz;
    const long long nProgressL = static_cast<long long>(S) * tilesY * tilesZ;
    if (nProgressL > std::numeric_limits<int>::max()) return fail(EIKX_ERR_INVALID, "too many slots for this grid");
    const int nProgress = static_cast<int>(nProgressL);
    const int nSweeps = std::max(0, o.n_sweeps);
    const int initSweeps = o.init_sweeps ? 1 : 0;
    const int resStride = 8 * (1 + nSweeps);
    const int W = static_cast<int>(sizeof(T) / 4);
    // the stream's sweeps: every slot is busy until the sources run out, and a source takes
    // at most (init + n_sweeps) iterations
    const long long perSource = initSweeps + nSweeps;
    const long long maxIters = (static_cast<long long>(nSrc) * perSource + S - 1) / S + perSource + 1;
    if (8 * maxIters + 1 >= (1ll << 31)) return fail(EIKX_ERR_INVALID, "stream too long for one call");
    const int epochStride = static_cast<int>(8 * maxIters + 1);

    // buffers
    const size_t mboxBytes = static_cast<size_t>(nProgress) * (ly + lz) * Px * W * 8;
    EIKX_CUDA(w.tt.ensure(static_cast<size_t>(fieldStride) * nBufs * sizeof(T)));
    if (w.mbox.bytes < mboxBytes || !w.mbox.p) {
        EIKX_CUDA(w.mbox.ensure(mboxBytes));
        EIKX_CUDA(cudaMemsetAsync(w.mbox.p, 0, w.mbox.bytes, c->stream));
    }
    if (!w.epoch.p) {
        EIKX_CUDA(w.epoch.ensure(2 * sizeof(unsigned)));
        EIKX_CUDA(cudaMemsetAsync(w.epoch.p, 0, 2 * sizeof(unsigned), c->stream));
    }
    EIKX_CUDA(w.queue.ensure(2 * sizeof(unsigned)));
    EIKX_CUDA(w.residual.ensure(static_cast<size_t>(S) * resStride * 8));
    EIKX_CUDA(w.converged.ensure(static_cast<size_t>(S) * 4));
    EIKX_CUDA(w.iterations.ensure(static_cast<size_t>(S) * 4));
    EIKX_CUDA(w.abortFlag.ensure(sizeof(int)));
    EIKX_CUDA(w.order.ensure(static_cast<size_t>(nProgress) * 16));
    EIKX_CUDA(w.srcs.ensure(static_cast<size_t>(S) * sizeof(eikx::SourceT<T>)));
    EIKX_CUDA(w.corners.ensure(static_cast<size_t>(S) * sizeof(eikx::Corner3)));
    EIKX_CUDA(w.slots.ensure(static_cast<size_t>(S) * sizeof(int2)));
    EIKX_CUDA(w.list.ensure(static_cast<size_t>(S) * sizeof(int)));
    while (static_cast<int>(w.bufEv.size()) < nBufs) {
        cudaEvent_t e;
        EIKX_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        w.bufEv.push_back(e);
    }
    if (!w.boundary) EIKX_CUDA(cudaEventCreateWithFlags(&w.boundary, cudaEventDisableTiming));
    // FP64 factor tables of every source, filled once
    std::vector<eikx::SourceFp64> srcT64 = srcT64In;
    const bool near64 = !srcT64.empty();
    if (near64) {
        EIKX_CUDA(assignFactorTables(srcT64, w.factor));
        EIKX_CUDA(w.srcs64All.ensure(srcT64.size() * sizeof(eikx::SourceFp64)));
        EIKX_CUDA(w.srcs64.ensure(static_cast<size_t>(S) * sizeof(eikx::SourceFp64)));
    }
    // staging: the slot table, sources, corners, FP64 records and the refill list per
    // boundary; the flags read back per boundary
    const size_t srcB = sizeof(eikx::SourceT<T>), cornB = sizeof(eikx::Corner3), s64B = sizeof(eikx::SourceFp64);
    const size_t offSrc = static_cast<size_t>(S) * sizeof(int2), offCorn = offSrc + S * srcB,
                 offS64 = offCorn + S * cornB, offList = offS64 + S * s64B, offEnd = offList + S * sizeof(int);
    EIKX_CUDA(cudaStreamSynchronize(c->stream));
    EIKX_CUDA(w.stage.ensure(std::max(offEnd, near64 ? srcT64.size() * s64B : 0) + 64));
    EIKX_CUDA(w.flags.ensure(static_cast<size_t>(2 * S + 1) * sizeof(int)));
    char *stage = static_cast<char *>(w.stage.p);
    int *flags = static_cast<int *>(w.flags.p);
    if (near64) {
        std::memcpy(stage, srcT64.data(), srcT64.size() * s64B);
        EIKX_CUDA(cudaMemcpyAsync(w.srcs64All.p, stage, srcT64.size() * s64B, cudaMemcpyHostToDevice, c->stream));
        EIKX_CUDA(eikx::launchFactorTables(w.srcs64All.as<eikx::SourceFp64>(), nSrc, c->stream));
        EIKX_CUDA(cudaStreamSynchronize(c->stream));   // the staging buffer is reused below
    }
    std::vector<int> key = {tilesY, tilesZ, S, 3, ly};
    if (key != w.orderKey) {
        const std::vector<int> order = buildOrder(tilesY, tilesZ, S, ly, lz);
        EIKX_CUDA(cudaMemcpy(w.order.p, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice));
        w.orderKey = key;
    }

    eikx::SolveState st{};
    st.queue[0] = w.queue.as<unsigned>();
    st.queue[1] = w.queue.as<unsigned>() + 1;
    st.mbox = w.mbox.as<unsigned long long>();
    st.epoch = w.epoch.as<unsigned>();
    st.epochStride = epochStride;
    st.residual = w.residual.as<unsigned long long>();
    st.residualStride = resStride;
    st.converged = w.converged.as<int>();
    st.sweepsRun = w.iterations.as<int>();
    st.abortFlag = w.abortFlag.as<int>();
    const int drop = std::min(std::max(o.test_drop_blocks, 0), nProgress);
    st.order = w.order.as<int4>() + drop;
    st.totalItems = nProgress - drop;
    const int spinLog2 = o.spin_limit_log2 > 0 ? std::min(o.spin_limit_log2, 40) : 22;
    st.spinLimit = 1ull << spinLog2;
    int perSM = eikx::sweep3ChunkBlocksPerSM<T>(uniform, false, shape);
    if (o.blocks_per_sm > 0) perSM = std::min(perSM, o.blocks_per_sm);
    const int blocks = std::max(1, std::min(c->numSMs * perSM, (nProgress + eikx::kWarpsPerBlock - 1) / eikx::kWarpsPerBlock));

    // slots
    std::vector<int> slotSrc(S, -1), slotStart(S, -1), slotBuf(S, -1), bufBusy(nBufs, 0), freeBufs;
    std::vector<int> runOf(nSrc, 0);
    for (int b = nBufs - 1; b >= 0; --b) freeBufs.push_back(b);
    auto takeBuffer = [&](int *out) -> eikx_status {
        for (int b = 0; b < nBufs; ++b)
            if (bufBusy[b] && cudaEventQuery(w.bufEv[b]) == cudaSuccess) {
                bufBusy[b] = 0;
                freeBufs.push_back(b);
            }
        if (freeBufs.empty()) {
            // every spare buffer is still being copied out: wait for one
            for (int b = 0; b < nBufs; ++b)
                if (bufBusy[b]) {
                    EIKX_CUDA(cudaEventSynchronize(w.bufEv[b]));
                    bufBusy[b] = 0;
                    freeBufs.push_back(b);
                    break;
                }
        }
        *out = freeBufs.back();
        freeBufs.pop_back();
        return EIKX_OK;
    };
    int next = 0, active = 0, launches = 0, sweepsRun = 0, profiled = 0;
    std::vector<int> list;
    for (int f = 0; f < S && next < nSrc; ++f) {
        slotSrc[f] = next++;
        slotStart[f] = 0;
        if (eikx_status r = takeBuffer(&slotBuf[f]); r != EIKX_OK) return r;
        list.push_back(f);
        ++active;
    }
    // the slot table and the new slots' sources, then their fields
    auto upload = [&]() -> eikx_status {
        int2 *tab = reinterpret_cast<int2 *>(stage);
        for (int f = 0; f < S; ++f) tab[f] = make_int2(slotStart[f], slotBuf[f]);
        for (int f : list) {
            std::memcpy(stage + offSrc + f * srcB, &srcT[slotSrc[f]], srcB);
            std::memcpy(stage + offCorn + f * cornB, &corners[slotSrc[f]], cornB);
            if (near64) std::memcpy(stage + offS64 + f * s64B, &srcT64[slotSrc[f]], s64B);
        }
        std::memcpy(stage + offList, list.data(), list.size() * sizeof(int));
        EIKX_CUDA(cudaMemcpyAsync(w.slots.p, stage, S * sizeof(int2), cudaMemcpyHostToDevice, c->stream));
        for (int f : list) {
            EIKX_CUDA(cudaMemcpyAsync(w.srcs.as<char>() + f * srcB, stage + offSrc + f * srcB, srcB,
                                      cudaMemcpyHostToDevice, c->stream));
            EIKX_CUDA(cudaMemcpyAsync(w.corners.as<char>() + f * cornB, stage + offCorn + f * cornB, cornB,
                                      cudaMemcpyHostToDevice, c->stream));
            if (near64)
                EIKX_CUDA(cudaMemcpyAsync(w.srcs64.as<char>() + f * s64B, stage + offS64 + f * s64B, s64B,
                                          cudaMemcpyHostToDevice, c->stream));
        }
        if (!list.empty()) {
            EIKX_CUDA(cudaMemcpyAsync(w.list.p, stage + offList, list.size() * sizeof(int), cudaMemcpyHostToDevice,
                                      c->stream));
            EIKX_CUDA(eikx::launchRefillSlots<T>(w.tt.as<T>(), fieldStride, Px, nx, ny, nz, dx, dy, dz, st,
                                                 w.slots.as<int2>(), w.list.as<int>(), static_cast<int>(list.size()),
                                                 w.corners.as<eikx::Corner3>(), o.init_fp64 ? 1 : 0, c->stream));
            launches += 2;
        }
        return EIKX_OK;
    };

    const bool profile = o.profile_sweeps != 0;
    if (eikx_status r = advanceEpoch(w.epochMirror, w.mbox, w.epoch, epochStride, c->stream); r != EIKX_OK) return r;
    EIKX_CUDA(cudaEventRecord(c->ev0, c->stream));
    EIKX_CUDA(eikx::launchResetState(st, S, 0, c->stream));
    ++launches;
    if (eikx_status r = upload(); r != EIKX_OK) return r;
    const eikx::Spacing3<T> g = spacing3<T>(dx, dy, dz);
    const cudaMemcpyKind kind = where == EIKX_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const long long nodes = static_cast<long long>(nx) * ny * nz;
    int buf = 0, aborted = 0;
    long long refineUpdates = 0;
    std::vector<int> iterOf(nSrc, 0);
    while (active > 0) {
        for (int e = 0; e < 8; ++e) {
            if (sweepsRun + 1 >= epochStride) return fail(EIKX_ERR_STATE, "stream ran past its sweep bound");
            if (profile) {
                while (static_cast<int>(c->sweepEv.size()) < 2 * (profiled + 1)) {
                    cudaEvent_t ev;
                    EIKX_CUDA(cudaEventCreate(&ev));
                    c->sweepEv.push_back(ev);
                }
                EIKX_CUDA(cudaEventRecord(c->sweepEv[2 * profiled], c->stream));
            }
            eikx::Sweep3Args<T> a{};
            a.tt = w.tt.as<T>(); a.fieldStride = fieldStride; a.pitch = Px;
            a.spPos = spad[0].as<T>(); a.spNeg = spad[1].as<T>(); a.spPitch = spPitch;
            a.spPlane = static_cast<long long>(spPitch) * (ny + 1);
            a.nx = nx; a.ny = ny; a.nz = nz; a.tilesY = tilesY; a.tilesZ = tilesZ;
            a.srcs = w.srcs.as<eikx::SourceT<T>>(); a.st = st; a.buf = buf; a.residualSlot = 0;
            a.sweepIndex = sweepsRun; a.sweep = e; a.init = 0; a.radius = o.factored_radius;
            a.h = static_cast<T>(dx); a.sp3 = g;
            a.srcs64 = near64 ? w.srcs64.as<eikx::SourceFp64>() : nullptr;
            a.slots = w.slots.as<int2>();
            a.initSweeps = initSweeps;
            if (uniform && sizeof(T) == 8) {
                a.hsPos = shad[0].as<T>(); a.hsNeg = shad[1].as<T>();
                a.cells = c->slow3.p; a.cells64 = 1;
            }
            EIKX_CUDA(eikx::launchSweep3Chunk<T>(a, uniform, shape, blocks, c->stream));
            EIKX_CUDA(eikx::launchCheckStream(st, w.slots.as<int2>(), S, sweepsRun, initSweeps, o.tolerance, c->stream));
            if (profile) EIKX_CUDA(cudaEventRecord(c->sweepEv[2 * profiled + 1], c->stream));
            ++profiled;
            launches += 2;
            buf ^= 1;
            ++sweepsRun;
        }
        // iteration boundary: the slots' flags and sweep counts
        EIKX_CUDA(cudaMemcpyAsync(flags, w.converged.p, S * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        EIKX_CUDA(cudaMemcpyAsync(flags + S, w.iterations.p, S * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        EIKX_CUDA(cudaMemcpyAsync(flags + 2 * S, w.abortFlag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        EIKX_CUDA(cudaEventRecord(w.boundary, c->stream));
        EIKX_CUDA(cudaStreamSynchronize(c->stream));
        if (flags[2 * S]) {
            aborted = 1;
            break;
        }
        list.clear();
        bool changed = false;
        for (int f = 0; f < S; ++f) {
            if (slotSrc[f] < 0) continue;
            const int refined = sweepsRun - slotStart[f] - 8 * initSweeps;
            if (!flags[f] && refined < 8 * nSweeps) continue;
            // finished: copy the field out, after this iteration's sweeps
            const int src = slotSrc[f], b = slotBuf[f];
            iterOf[src] = flags[S + f];
            refineUpdates += nodes * flags[S + f];
            EIKX_CUDA(cudaStreamWaitEvent(c->copyStream, w.boundary, 0));
            EIKX_CUDA(eikx::copyRows(static_cast<char *>(tOut) + static_cast<size_t>(src) * nodes * sizeof(T),
                                        static_cast<size_t>(nx) * sizeof(T),
                                        w.tt.as<T>() + static_cast<size_t>(b) * fieldStride,
                                        static_cast<size_t>(Px) * sizeof(T), static_cast<size_t>(nx) * sizeof(T),
                                        static_cast<size_t>(ny) * nz, kind, c->copyStream));
            EIKX_CUDA(cudaEventRecord(w.bufEv[b], c->copyStream));
            bufBusy[b] = 1;
            changed = true;
            if (next < nSrc) {
                slotSrc[f] = next++;
                slotStart[f] = sweepsRun;
                if (eikx_status r = takeBuffer(&slotBuf[f]); r != EIKX_OK) return r;
                list.push_back(f);
            } else {
                slotSrc[f] = slotStart[f] = slotBuf[f] = -1;
                --active;
            }
        }
        if (changed && active > 0)
            if (eikx_status r = upload(); r != EIKX_OK) return r;
    }
    // the copies, then the end of the solve
    EIKX_CUDA(cudaEventRecord(c->copyDone, c->copyStream));
    EIKX_CUDA(cudaStreamWaitEvent(c->stream, c->copyDone, 0));
    EIKX_CUDA(cudaEventRecord(c->ev1, c->stream));
    EIKX_CUDA(cudaStreamSynchronize(c->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    eikx_stats s{};
    s.n_fields = nSrc;
    s.iterations_max = 0;
    s.iterations_min = 1 << 30;
    for (int i = 0; i < nSrc; ++i) {
        const int it = (iterOf[i] + 7) / 8;
        s.iterations_max = std::max(s.iterations_max, it);
        s.iterations_min = std::min(s.iterations_min, it);
    }
    s.refine_node_updates = refineUpdates;
    s.residual_last = 0;
    s.sweeps_launched = sweepsRun;
    s.sweep_ms = -1;
    if (profile) {
        double tot = 0;
        for (int i = 0; i < profiled; ++i) {
            float m = 0;
            cudaEventElapsedTime(&m, c->sweepEv[2 * i], c->sweepEv[2 * i + 1]);
            tot += m;
        }
        s.sweep_ms = tot;
    }
    s.kernel_launches = launches;
    s.device_ms = ms;
    s.reset_nodes = 0;
    c->stats = s;
    c->last.valid = false;   // the fields of a stream do not stay on the device
    if (aborted) return fail(EIKX_ERR_TIMEOUT, "a bounded inter-tile wait ran out; the fields are not valid");
    return EIKX_OK;
}

// Shared solve driver for 2D and 3D.

template <class T, int DIM>
eikx_status solveImpl(eikx_ctx *c, const double *srcXYZ, int nSrc, eikx_options o, void *tOut,
                      int where, const void *tInit = nullptr, int initWhere = EIKX_HOST, double gateTol = 0) {
    const bool warm = DIM == 3 && tInit != nullptr;
    if (warm) o.init_sweeps = 0;   // the initial field replaces the initialisation pass
    const int P = precOf<T>();
    const int nx = DIM == 3 ? c->nx : c->nx2;
    const int ny = DIM == 3 ? c->ny : 1;
    const int nz = DIM == 3 ? c->nz : c->nz2;
    const double dx = DIM == 3 ? c->dx : c->dx2, dy = DIM == 3 ? c->dy : 1.0, dz = DIM == 3 ? c->dz : c->dz2;
    const double x0 = DIM == 3 ? c->x0 : c->x02, y0 = DIM == 3 ? c->y0 : 0.0, z0 = DIM == 3 ? c->z0 : c->z02;
    const int Px = roundUp(nx, 4);
    const int spPitch = Px + 8;
    const long long fieldStride = static_cast<long long>(Px) * ny * nz;
    // sources: cell, offsets, source-cell slowness (reference Source3D / Solver3D::solve);
    // the slownesses are read from the device model, one value per source
    std::vector<eikx::SourceT<T>> srcT(nSrc);
    std::vector<eikx::SourceFp64> srcT64;
    std::vector<eikx::Corner3> corners(nSrc);
    std::vector<size_t> srcCells(nSrc);
    std::vector<std::array<double, 3>> srcOffs(nSrc);
    for (int i = 0; i < nSrc; ++i) {
        const double x = srcXYZ[3 * i], y = srcXYZ[3 * i + 1], z = srcXYZ[3 * i + 2];
        int cx, cy = 0, cz;
        double ox, oy = 0, oz;
        if (!locate(x, x0, dx, nx, &cx, &ox))
            return fail(EIKX_ERR_INVALID, "x source position = " + std::to_string(x) + " must be in range [" +
                                              std::to_string(x0) + "," + std::to_string(x0 + (nx - 1) * dx) + "]");
        if (DIM == 3 && !locate(y, y0, dy, ny, &cy, &oy))
            return fail(EIKX_ERR_INVALID, "y source position = " + std::to_string(y) + " must be in range [" +
                                              std::to_string(y0) + "," + std::to_string(y0 + (ny - 1) * dy) + "]");
        if (!locate(z, z0, dz, nz, &cz, &oz))
            return fail(EIKX_ERR_INVALID, "z source position = " + std::to_string(z) + " must be in range [" +
                                              std::to_string(z0) + "," + std::to_string(z0 + (nz - 1) * dz) + "]");
        srcCells[i] = DIM == 3 ? (static_cast<size_t>(cz) * (ny - 1) + cy) * (nx - 1) + cx
                               : static_cast<size_t>(cz) * (nx - 1) + cx;
        srcOffs[i] = {ox, oy, oz};
        srcT[i].isx = cx; srcT[i].isy = cy; srcT[i].isz = cz;
        srcT[i].xs = static_cast<T>(ox); srcT[i].ys = static_cast<T>(oy); srcT[i].zs = static_cast<T>(oz);
    }
    EIKX_CUDA(c->srcSlow.ensure(static_cast<size_t>(nSrc) * sizeof(double)));
    double *srcSlow = static_cast<double *>(c->srcSlow.p);
    const double *slowDev = (DIM == 3 ? c->slow3 : c->slow2).as<double>();
    EIKX_CUDA(cudaStreamSynchronize(c->stream));   // the pinned values of a previous call are free
    for (int i = 0; i < nSrc; ++i)
        EIKX_CUDA(cudaMemcpyAsync(srcSlow + i, slowDev + srcCells[i], sizeof(double), cudaMemcpyDeviceToHost,
                                  c->stream));
    EIKX_CUDA(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < nSrc; ++i) {
        const double s = srcSlow[i];
        srcT[i].sSrc = static_cast<T>(s);
        if (DIM == 3 && P == EIKX_F32 && o.near_fp64)
            srcT64.push_back(sourceFp64(srcOffs[i], srcT[i].isx, srcT[i].isy, srcT[i].isz, std::max(0, o.factored_radius),
                                        nx, ny, nz, dx, dy, dz, nullptr, spPitch));
        // corner init: slowness as the field type holds it, offsets in FP64
        corners[i] = eikx::Corner3{srcT[i].isx, srcT[i].isy, srcT[i].isz, srcOffs[i][0], srcOffs[i][1], srcOffs[i][2],
                                   static_cast<double>(static_cast<T>(s))};
    }

    // edge-replicated slowness in the sweep precision: one copy shifted by V-1 columns
    // (16-byte chunks of V elements) for +x sweeps, one unshifted for -x sweeps
    DevBuf *spad = DIM == 3 ? c->spad3[P] : c->spad2[P];
    bool &spadValid = DIM == 3 ? c->spadValid3[P] : c->spadValid2[P];
    const size_t spElems = static_cast<size_t>(spPitch) * (DIM == 3 ? ny + 1 : 1) * (nz + 1);
    if (!spadValid || spad[0].bytes < spElems * sizeof(T)) {
        if (spad[0].bytes < spElems * sizeof(T)) dropGraph(c);
        for (int k = 0; k < 2; ++k) {
            EIKX_CUDA(spad[k].ensure(spElems * sizeof(T)));
            const int shift = k == 0 ? static_cast<int>(16 / sizeof(T)) - 1 : 0;
            if (DIM == 3)
                EIKX_CUDA((eikx::launchPadSlowness3<T, double>(spad[k].as<T>(), spPitch, shift, c->slow3.as<double>(),
                                                               nx, ny, nz, c->stream)));
            else
                EIKX_CUDA((eikx::launchPadSlowness2<T, double>(spad[k].as<T>(), spPitch, shift, c->slow2.as<double>(),
                                                               nx, nz, c->stream)));
        }
        spadValid = true;
    }

    // the factor tables are filled from the unshifted padded copy (FP32 sweeps)
    for (auto &f : srcT64) {
        if (f.bnx == 0)
            return fail(EIKX_ERR_UNSUPPORTED, "near_fp64: the factored region of radius " +
                                                  std::to_string(o.factored_radius) + " needs more than " +
                                                  std::to_string(eikx::kMaxFactorTable) + " table entries");
        f.sp = static_cast<const float *>(spad[1].p);
    }

    // geometry in the sweep type (include/private/solver3d.hpp:31-44, solver2d.hpp:29-46)
    const double eps = std::numeric_limits<T>::epsilon() * 100;
    const bool uniform = DIM == 3 ? (std::abs(dx - dy) < eps && std::abs(dx - dz) < eps) : (std::abs(dx - dz) < eps);
    // uniform 3D grids in FP64: the padded copies multiplied by h, which the chunk-step kernel reads
    DevBuf *shad = c->shad3[P];
    if (DIM == 3 && sizeof(T) == 8 && uniform && (!c->shadValid3[P] || shad[0].bytes < spElems * sizeof(T))) {
        if (shad[0].bytes < spElems * sizeof(T)) dropGraph(c);
        for (int k = 0; k < 2; ++k) {
            EIKX_CUDA(shad[k].ensure(spElems * sizeof(T)));
            const int shift = k == 0 ? static_cast<int>(16 / sizeof(T)) - 1 : 0;
            EIKX_CUDA((eikx::launchPadSlowness3<T, double>(shad[k].as<T>(), spPitch, shift, c->slow3.as<double>(),
                                                           nx, ny, nz, c->stream, static_cast<T>(dx))));
        }
        c->shadValid3[P] = true;
    }
    // options left at "auto" take the tuned configuration of this grid class
    if (DIM == 3 && o.sweep_kernel == 0 && o.block_shape == 0 && o.blocks_per_sm == 0 && !o.pair_fields) {
        // a stream launches its slots' fields, not all of its sources
        const int perLaunch = o.max_in_flight > 0 && o.max_in_flight < nSrc ? o.max_in_flight : nSrc;
        auto it = c->tuning.find(tuneKey(P, uniform, nx, ny, nz, perLaunch));
        if (it != c->tuning.end()) {
            o.sweep_kernel = it->second.sweep_kernel;
            o.pair_fields = it->second.pair_fields;
            o.block_shape = it->second.block_shape;
            o.blocks_per_sm = it->second.blocks_per_sm;
        }
    }
    // the FP64 factored branch runs in the chunk-step kernel (its own instances)
    if (DIM == 3 && P == EIKX_F32 && o.near_fp64) {
        o.sweep_kernel = eikx::kChunkStep;
        o.pair_fields = 0;
    }
    // a stream of the sources through max_in_flight slots (chunk-step)
    if constexpr (DIM == 3) {
        if (!warm && o.max_in_flight > 0 && o.max_in_flight < nSrc && (o.init_sweeps || o.n_sweeps > 0))
            return solveStream3<T>(c, o, nSrc, srcT, srcT64, corners, uniform,
                                   o.block_shape > 0 ? o.block_shape - 1 : eikx::kShape8x4, tOut, where, spad);
    }
    // FP32 uniform 3D batches run two fields per lane (the paired kernel)
    const bool paired = DIM == 3 && P == EIKX_F32 && uniform && nSrc >= 2 && o.pair_fields;
    const int nUnits = paired ? (nSrc + 1) / 2 : nSrc;   // work units: fields or field pairs

    // sweep kernel and warp-block shape
    const int variant = o.sweep_kernel == eikx::kNodeStep ? eikx::kNodeStep : eikx::kChunkStep;
    const bool chunkStep = DIM == 3 && !paired && variant == eikx::kChunkStep;
    // 2D grids of up to 512 rows can run one CTA per field (sweep_kernel = 2); the warp-block
    // kernel is the default: measured faster on GB300 for 1 to 512 fields of 501 x 251 nodes
    const bool block2 = DIM == 2 && nz <= eikx::kMaxBlockRows2 && o.sweep_kernel == eikx::kChunkStep;
    const int shape = chunkStep && o.block_shape > 0 ? o.block_shape - 1 : eikx::kShape8x4;

    // workspace
    const int ly = DIM == 3 ? eikx::shapeLY(shape) : 1, lz = DIM == 3 ? eikx::shapeLZ(shape) : eikx::LZ2;
    const int tilesY = DIM == 3 ? (ny + ly - 1) / ly : 1;
    const int tilesZ = (nz + lz - 1) / lz;
    const int nProgress = nUnits * tilesY * tilesZ;
    const int nSweepKinds = DIM == 3 ? 8 : 4;
    const int nSweeps = std::max(0, o.n_sweeps);
    const int resStride = nSweepKinds * (1 + nSweeps);
    Workspace &w = c->ws;
    const size_t ttBytes = static_cast<size_t>(fieldStride) * nSrc * sizeof(T);
    const int mailWords = paired ? 2 : static_cast<int>(sizeof(T) / 4);   // tagged 64-bit words per unit
    const size_t mboxBytes = static_cast<size_t>(nProgress) * (DIM == 3 ? ly + lz : 1) * Px * mailWords * 8;
    const void *before[] = {w.tt.p, w.mbox.p, w.epoch.p, w.residual.p, w.converged.p,
                            w.iterations.p, w.order.p, w.srcs.p, w.corners.p, w.srcs64.p, w.factor.p};
    EIKX_CUDA(w.tt.ensure(ttBytes));
    if (w.mbox.bytes < mboxBytes || !w.mbox.p) {
        // fresh words carry tag 0, which no sweep uses
        EIKX_CUDA(w.mbox.ensure(mboxBytes));
        EIKX_CUDA(cudaMemsetAsync(w.mbox.p, 0, w.mbox.bytes, c->stream));
    }
    if (!w.epoch.p) {
        EIKX_CUDA(w.epoch.ensure(2 * sizeof(unsigned)));
        EIKX_CUDA(cudaMemsetAsync(w.epoch.p, 0, 2 * sizeof(unsigned), c->stream));
    }
    EIKX_CUDA(w.queue.ensure(2 * sizeof(unsigned)));
    EIKX_CUDA(w.residual.ensure(static_cast<size_t>(nSrc) * resStride * 8));
    EIKX_CUDA(w.converged.ensure(static_cast<size_t>(nSrc) * 4));
    EIKX_CUDA(w.iterations.ensure(static_cast<size_t>(nSrc) * 4));
    EIKX_CUDA(w.abortFlag.ensure(sizeof(int)));
    EIKX_CUDA(w.order.ensure(static_cast<size_t>(nProgress) * 16));
    EIKX_CUDA(w.srcs.ensure(static_cast<size_t>(nSrc) * sizeof(eikx::SourceT<T>)));
    EIKX_CUDA(w.corners.ensure(static_cast<size_t>(nSrc) * sizeof(eikx::Corner3)));
    EIKX_CUDA(w.pairs.ensure(static_cast<size_t>(nUnits) * sizeof(int2)));
    if (!srcT64.empty()) {
        EIKX_CUDA(w.srcs64.ensure(srcT64.size() * sizeof(eikx::SourceFp64)));
        EIKX_CUDA(assignFactorTables(srcT64, w.factor));
    }
    const void *after[] = {w.tt.p, w.mbox.p, w.epoch.p, w.residual.p, w.converged.p,
                           w.iterations.p, w.order.p, w.srcs.p, w.corners.p, w.srcs64.p, w.factor.p};
    if (std::memcmp(before, after, sizeof(before)) != 0) dropGraph(c);

    // small uploads through pinned staging
    std::vector<int> key = {tilesY, tilesZ, nUnits, DIM, ly};
    const bool newOrder = key != w.orderKey;
    std::vector<int> order;
    if (newOrder) order = buildOrder(tilesY, tilesZ, nUnits, ly, lz);
    std::vector<int> pairs;
    if (paired) {
        for (int i = 0; i < nUnits; ++i) {
            pairs.push_back(2 * i);
            pairs.push_back(std::min(2 * i + 1, nSrc - 1));   // an odd batch pairs its last field with itself
        }
    }
    const size_t pairBytes = pairs.size() * sizeof(int);
    const size_t srcBytes = srcT.size() * sizeof(eikx::SourceT<T>);
    const size_t cornerBytes = corners.size() * sizeof(eikx::Corner3);
    const size_t orderBytes = order.size() * sizeof(int);
    const size_t src64Bytes = srcT64.size() * sizeof(eikx::SourceFp64);
    EIKX_CUDA(cudaStreamSynchronize(c->stream));  // staging buffer reuse
    EIKX_CUDA(w.stage.ensure(srcBytes + cornerBytes + orderBytes + pairBytes + src64Bytes + 64));
    char *stage = static_cast<char *>(w.stage.p);
    std::memcpy(stage, srcT.data(), srcBytes);
    std::memcpy(stage + srcBytes, corners.data(), cornerBytes);
    EIKX_CUDA(cudaMemcpyAsync(w.srcs.p, stage, srcBytes, cudaMemcpyHostToDevice, c->stream));
    EIKX_CUDA(cudaMemcpyAsync(w.corners.p, stage + srcBytes, cornerBytes, cudaMemcpyHostToDevice, c->stream));
    if (newOrder) {
        std::memcpy(stage + srcBytes + cornerBytes, order.data(), orderBytes);
        EIKX_CUDA(cudaMemcpyAsync(w.order.p, stage + srcBytes + cornerBytes, orderBytes, cudaMemcpyHostToDevice,
                                  c->stream));
        w.orderKey = key;
    }
    if (paired) {
        char *pstage = stage + srcBytes + cornerBytes + orderBytes;
        std::memcpy(pstage, pairs.data(), pairBytes);
        EIKX_CUDA(cudaMemcpyAsync(w.pairs.p, pstage, pairBytes, cudaMemcpyHostToDevice, c->stream));
    }
    const eikx::SourceFp64 *srcs64 = nullptr;
    if (!srcT64.empty()) {
        char *qstage = stage + srcBytes + cornerBytes + orderBytes + pairBytes;
        std::memcpy(qstage, srcT64.data(), src64Bytes);
        EIKX_CUDA(cudaMemcpyAsync(w.srcs64.p, qstage, src64Bytes, cudaMemcpyHostToDevice, c->stream));
        srcs64 = w.srcs64.as<eikx::SourceFp64>();
    }

    if (warm) {
        const size_t initBytes = static_cast<size_t>(nx) * ny * nz * nSrc * sizeof(T);
        const void *initBefore = w.init.p;
        EIKX_CUDA(w.init.ensure(initBytes));
        EIKX_CUDA(w.resetCount.ensure(sizeof(unsigned long long)));
        if (w.init.p != initBefore) dropGraph(c);
        EIKX_CUDA(cudaMemcpyAsync(w.init.p, tInit, initBytes,
                                  initWhere == EIKX_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                  c->stream));
    }
    const int nSweepLaunches = nSweepKinds * ((o.init_sweeps ? 1 : 0) + nSweeps);
    eikx::SolveState st{};
    st.queue[0] = w.queue.as<unsigned>();
    st.queue[1] = w.queue.as<unsigned>() + 1;
    st.mbox = w.mbox.as<unsigned long long>();
    st.epoch = w.epoch.as<unsigned>();
    st.epochStride = nSweepLaunches + 1;
    st.residual = w.residual.as<unsigned long long>();
    st.residualStride = resStride;
    st.converged = w.converged.as<int>();
    st.sweepsRun = w.iterations.as<int>();
    st.abortFlag = w.abortFlag.as<int>();
    // test hook: leave the first blocks of the queue out (their dependants time out)
    const int drop = std::min(std::max(o.test_drop_blocks, 0), nProgress);
    st.order = w.order.as<int4>() + drop;
    st.totalItems = nProgress - drop;
    const int spinLog2 = o.spin_limit_log2 > 0 ? std::min(o.spin_limit_log2, 40) : 22;
    st.spinLimit = 1ull << spinLog2;

    int perSM = paired ? eikx::sweep3PairBlocksPerSM()
                : DIM == 2 ? eikx::sweep2BlocksPerSM<T>(uniform)
                : chunkStep ? eikx::sweep3ChunkBlocksPerSM<T>(uniform, false, shape)
                            : eikx::sweep3BlocksPerSM<T>(uniform);
    if (o.blocks_per_sm > 0) perSM = std::min(perSM, o.blocks_per_sm);
    int blocks = std::min(c->numSMs * perSM, (nProgress + eikx::kWarpsPerBlock - 1) / eikx::kWarpsPerBlock);
    blocks = std::max(blocks, 1);

    // Host output: a field that has converged is not written again, so it is copied out on
    // a second stream at the end of the iteration in which it converged, while the sweeps
    // go on for the others; the rest are copied after the schedule.
    const bool early = where == EIKX_HOST && nSrc > 1 && nSweeps > 1 && o.tolerance > 0 && o.profile_sweeps == 0;
    int *iterFlags = nullptr;
    if (early) {
        while (static_cast<int>(c->iterEv.size()) < nSweeps) {
            cudaEvent_t e;
            EIKX_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            c->iterEv.push_back(e);
        }
        const void *fb = c->iterFlags.p;
        EIKX_CUDA(c->iterFlags.ensure(static_cast<size_t>(nSweeps) * nSrc * sizeof(int)));
        if (c->iterFlags.p != fb) dropGraph(c);
        iterFlags = static_cast<int *>(c->iterFlags.p);
    }

    ScheduleKey sk;
    sk.dim = DIM; sk.precision = P; sk.nFields = nSrc; sk.nx = nx; sk.ny = ny; sk.nz = nz;
    sk.nSweeps = nSweeps; sk.radius = o.factored_radius; sk.initSweeps = o.init_sweeps ? 1 : 0;
    sk.initFp64 = o.init_fp64 ? 1 : 0; sk.uniform = uniform; sk.blocks = blocks; sk.tol = o.tolerance;
    sk.h = dx; sk.dx = dx; sk.dy = dy; sk.dz = dz; sk.spin = st.spinLimit; sk.dropBlocks = drop;
    sk.paired = paired ? 1 : 0;
    sk.warm = warm ? 1 : 0;
    sk.gate = gateTol;
    sk.nearFp64 = DIM == 3 && P == EIKX_F32 && o.near_fp64 ? 1 : 0;
    sk.warmGate = warm ? o.warm_gate : 0;
    sk.variant = variant;
    sk.shape = shape;
    sk.tt = w.tt.p; sk.sp = spad[0].p; sk.srcs = w.srcs.p; sk.corners = w.corners.p;
    sk.early = early ? 1 : 0;
    sk.flags = iterFlags;

    int launches = 0;
    int sweepsLaunched = 0;
    const bool profile = o.profile_sweeps != 0;
    if (profile) {
        while (static_cast<int>(c->sweepEv.size()) < 2 * nSweepLaunches) {
            cudaEvent_t e;
            EIKX_CUDA(cudaEventCreate(&e));
            c->sweepEv.push_back(e);
        }
    }
    auto enqueue = [&]() -> eikx_status {
        launches = 0;
        sweepsLaunched = 0;
        int buf = 0;
        EIKX_CUDA(eikx::launchResetState(st, nSrc, buf, c->stream));
        ++launches;
        if (srcs64) {
            EIKX_CUDA(eikx::launchFactorTables(srcs64, nSrc, c->stream));
            ++launches;
        }
        if (warm) {
            EIKX_CUDA(cudaMemsetAsync(w.resetCount.p, 0, sizeof(unsigned long long), c->stream));
            EIKX_CUDA(eikx::launchWarmInit3<T>(w.tt.as<T>(), w.init.as<T>(), nSrc, fieldStride, Px, nx, ny, nz, dx, dy,
                                               dz, w.corners.as<eikx::Corner3>(), w.srcs.as<eikx::SourceT<T>>(),
                                               c->slow3.as<double>(), o.factored_radius, uniform, static_cast<T>(dx),
                                               spacing3<T>(dx, dy, dz), gateTol, o.warm_gate == 1 ? 1 : 0,
                                               o.init_fp64 ? 1 : 0, srcs64,
                                               w.resetCount.as<unsigned long long>(), c->stream));
        } else if (DIM == 3)
            EIKX_CUDA(eikx::launchInit3<T>(w.tt.as<T>(), nSrc, fieldStride, Px, nx, ny, nz, dx, dy, dz,
                                           w.corners.as<eikx::Corner3>(), o.init_fp64 ? 1 : 0, c->stream));
        else
            EIKX_CUDA(eikx::launchInit2<T>(w.tt.as<T>(), nSrc, fieldStride, Px, nx, nz, dx, dz,
                                           w.corners.as<eikx::Corner3>(), o.init_fp64 ? 1 : 0, c->stream));
        // 3D: the fill and the corner kernel; a warm start: its gate and the pitch padding
        launches += warm ? 1 + (Px > nx ? 1 : 0) : DIM == 3 ? 2 : 1;
        auto sweep = [&](int e, int init, int slot) -> eikx_status {
            if (profile) EIKX_CUDA(cudaEventRecord(c->sweepEv[2 * sweepsLaunched], c->stream));
            if (DIM == 3) {
                eikx::Sweep3Args<T> a{};
                a.tt = w.tt.as<T>(); a.fieldStride = fieldStride; a.pitch = Px;
                a.spPos = spad[0].as<T>(); a.spNeg = spad[1].as<T>(); a.spPitch = spPitch;
                a.spPlane = static_cast<long long>(spPitch) * (ny + 1);
                a.nx = nx; a.ny = ny; a.nz = nz; a.tilesY = tilesY; a.tilesZ = tilesZ;
                a.srcs = w.srcs.as<eikx::SourceT<T>>(); a.st = st; a.buf = buf; a.residualSlot = slot;
                a.sweepIndex = sweepsLaunched;
                a.sweep = e; a.init = init; a.radius = o.factored_radius; a.h = static_cast<T>(dx);
                a.srcs64 = srcs64;
                if (uniform && sizeof(T) == 8) {
                    a.hsPos = shad[0].as<T>(); a.hsNeg = shad[1].as<T>();
                    a.cells = c->slow3.p; a.cells64 = 1;
                }
                const T tdx = static_cast<T>(dx), tdy = static_cast<T>(dy), tdz = static_cast<T>(dz);
                eikx::Spacing3<T> g;
                g.dx = tdx; g.dy = tdy; g.dz = tdz;
                g.dxInv = 1 / tdx; g.dyInv = 1 / tdy; g.dzInv = 1 / tdz;
                g.dx2Inv = 1 / (tdx * tdx); g.dy2Inv = 1 / (tdy * tdy); g.dz2Inv = 1 / (tdz * tdz);
                g.dx_dz = tdx / tdz; g.dz_dx = tdz / tdx; g.dy_dz = tdy / tdz; g.dz_dy = tdz / tdy;
                g.dx_dy = tdx / tdy; g.dy_dx = tdy / tdx;
                g.dx2_p_dz2_inv = 1 / (tdx * tdx + tdz * tdz);
                g.dy2_p_dz2_inv = 1 / (tdy * tdy + tdz * tdz);
                g.dx2_p_dy2_inv = 1 / (tdx * tdx + tdy * tdy);
                a.sp3 = g;
                a.pairs = w.pairs.as<int2>();
                bool done = false;
                if constexpr (std::is_same<T, float>::value) {
                    if (paired) {
                        EIKX_CUDA(eikx::launchSweep3Pair(a, blocks, c->stream));
                        done = true;
                    }
                }
                if (!done) {
                    if (chunkStep) EIKX_CUDA(eikx::launchSweep3Chunk<T>(a, uniform, shape, blocks, c->stream));
                    else EIKX_CUDA(eikx::launchSweep3<T>(a, uniform, blocks, c->stream));
                }
            } else {
                eikx::Sweep2Args<T> a{};
                a.tt = w.tt.as<T>(); a.fieldStride = fieldStride; a.pitch = Px;
                a.spPos = spad[0].as<T>(); a.spNeg = spad[1].as<T>(); a.spPitch = spPitch;
                a.nx = nx; a.nz = nz; a.tilesZ = tilesZ;
                a.srcs = w.srcs.as<eikx::SourceT<T>>(); a.st = st; a.buf = buf; a.residualSlot = slot;
                a.sweepIndex = sweepsLaunched;
                a.sweep = e; a.init = init; a.radius = o.factored_radius; a.h = static_cast<T>(dx);
                eikx::Spacing2<T> g;
                g.dx = static_cast<T>(dx); g.dz = static_cast<T>(dz);
                g.dx_dz = static_cast<T>(dx / dz); g.dz_dx = static_cast<T>(dz / dx);
                g.cosTheta = static_cast<T>(dx / std::hypot(dx, dz));
                g.sinTheta = static_cast<T>(dz / std::hypot(dx, dz));
                a.sp2 = g;
                if (block2) EIKX_CUDA(eikx::launchSweep2Block<T>(a, uniform, nSrc, c->stream));
                else EIKX_CUDA(eikx::launchSweep2<T>(a, uniform, blocks, c->stream));
            }
            if (profile) EIKX_CUDA(cudaEventRecord(c->sweepEv[2 * sweepsLaunched + 1], c->stream));
            buf ^= 1;
            ++launches;
            ++sweepsLaunched;
            return EIKX_OK;
        };
        if (o.init_sweeps)
            for (int e = 0; e < nSweepKinds; ++e)
                if (eikx_status r = sweep(e, 1, e); r != EIKX_OK) return r;
        for (int k = 0; k < nSweeps; ++k) {
            for (int e = 0; e < nSweepKinds; ++e) {
                if (eikx_status r = sweep(e, 0, nSweepKinds * (1 + k) + e); r != EIKX_OK) return r;
                EIKX_CUDA(checkAfterSweep(st, nSrc, nSweepKinds, nSweepKinds * k + e, o.tolerance, c->stream));
                ++launches;
            }
            if (early) {
                EIKX_CUDA(cudaMemcpyAsync(iterFlags + static_cast<size_t>(k) * nSrc, w.converged.p, nSrc * sizeof(int),
                                          cudaMemcpyDeviceToHost, c->stream));
                // external: captured into the graph as a real record the host can wait on
                EIKX_CUDA(cudaEventRecordWithFlags(c->iterEv[k], c->stream, cudaEventRecordExternal));
            }
        }
        return EIKX_OK;
    };

    if (o.test_tag_margin > 0 && w.epochMirror.base == 0 && w.epochMirror.last == 0) {
        // test hook: put the tag base just below the 32-bit wrap-around
        const unsigned start[2] = {static_cast<unsigned>((1ull << 32) - static_cast<unsigned long long>(o.test_tag_margin)), 0u};
        EIKX_CUDA(cudaMemcpyAsync(w.epoch.p, start, sizeof(start), cudaMemcpyHostToDevice, c->stream));
        EIKX_CUDA(cudaStreamSynchronize(c->stream));
        w.epochMirror.base = start[0];
        w.epochMirror.last = 0;
    }
    if (eikx_status r = advanceEpoch(w.epochMirror, w.mbox, w.epoch, st.epochStride, c->stream); r != EIKX_OK)
        return r;
    EIKX_CUDA(cudaEventRecord(c->ev0, c->stream));
    if (c->useGraphs && !profile) {
        if (!(c->graphExec && c->graphKey == sk)) {
            dropGraph(c);
            cudaGraph_t graph = nullptr;
            EIKX_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            eikx_status r = enqueue();
            cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
            if (r != EIKX_OK) {
                if (graph) cudaGraphDestroy(graph);
                return r;
            }
            EIKX_CUDA(ce);
            cudaError_t ie = cudaGraphInstantiate(&c->graphExec, graph, 0);
            cudaGraphDestroy(graph);
            EIKX_CUDA(ie);
            c->graphKey = sk;
            c->graphLaunches = launches;
        }
        EIKX_CUDA(cudaGraphLaunch(c->graphExec, c->stream));
        launches = c->graphLaunches;
        sweepsLaunched = nSweepKinds * ((o.init_sweeps ? 1 : 0) + nSweeps);
    } else {
        if (eikx_status r = enqueue(); r != EIKX_OK) return r;
    }
    // pitched copies: rows of nx values out of rows of Px, one per run of consecutive fields
    const cudaMemcpyKind kind = where == EIKX_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const long long nodesPerField = static_cast<long long>(nx) * ny * nz;
    auto copyFields = [&](int f0, int f1, cudaStream_t s) -> cudaError_t {
        return eikx::copyRows(static_cast<char *>(tOut) + static_cast<size_t>(f0) * nodesPerField * sizeof(T),
                                 static_cast<size_t>(nx) * sizeof(T),
                                 static_cast<char *>(w.tt.p) + static_cast<size_t>(f0) * fieldStride * sizeof(T),
                                 static_cast<size_t>(Px) * sizeof(T), static_cast<size_t>(nx) * sizeof(T),
                                 static_cast<size_t>(ny) * nz * (f1 - f0), kind, s);
    };
    std::vector<char> copied(nSrc, 0);
    if (early) {
        int left = nSrc;
        for (int k = 0; k < nSweeps && left > 0; ++k) {
            EIKX_CUDA(cudaEventSynchronize(c->iterEv[k]));
            const int *fl = iterFlags + static_cast<size_t>(k) * nSrc;
            bool waited = false;
            for (int f = 0; f < nSrc;) {
                if (!fl[f] || copied[f]) {
                    ++f;
                    continue;
                }
                int g = f;
                while (g < nSrc && fl[g] && !copied[g]) copied[g++] = 1;
                if (!waited) EIKX_CUDA(cudaStreamWaitEvent(c->copyStream, c->iterEv[k], 0));
                waited = true;
                EIKX_CUDA(copyFields(f, g, c->copyStream));
                left -= g - f;
                f = g;
            }
        }
    }
    for (int f = 0; f < nSrc;) {
        if (copied[f]) {
            ++f;
            continue;
        }
        int g = f;
        while (g < nSrc && !copied[g]) ++g;
        EIKX_CUDA(copyFields(f, g, c->stream));
        f = g;
    }
    if (early) {
        EIKX_CUDA(cudaEventRecord(c->copyDone, c->copyStream));
        EIKX_CUDA(cudaStreamWaitEvent(c->stream, c->copyDone, 0));
    }
    EIKX_CUDA(cudaEventRecord(c->ev1, c->stream));
    std::vector<int> iters(nSrc);
    int aborted = 0;
    unsigned long long resets = 0;
    if (warm)
        EIKX_CUDA(cudaMemcpyAsync(&resets, w.resetCount.p, sizeof(resets), cudaMemcpyDeviceToHost, c->stream));
    EIKX_CUDA(cudaMemcpyAsync(iters.data(), w.iterations.p, nSrc * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    EIKX_CUDA(cudaMemcpyAsync(&aborted, w.abortFlag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    std::vector<unsigned long long> lastRes;
    if (nSweeps > 0) {
        lastRes.resize(static_cast<size_t>(nSrc) * resStride);
        EIKX_CUDA(cudaMemcpyAsync(lastRes.data(), w.residual.p, lastRes.size() * 8, cudaMemcpyDeviceToHost, c->stream));
    }
    EIKX_CUDA(cudaStreamSynchronize(c->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    eikx_stats s{};
    s.n_fields = nSrc;
    s.iterations_max = 0;
    s.iterations_min = nSrc ? 1 << 30 : 0;
    double rl = 0;
    const long long nodes = static_cast<long long>(nx) * ny * nz;
    for (int i = 0; i < nSrc; ++i) {
        // iters[i] holds the refinement sweeps the field ran; report iterations begun
        const int sweepsRun = iters[i], it = (sweepsRun + nSweepKinds - 1) / nSweepKinds;
        s.iterations_max = std::max(s.iterations_max, it);
        s.iterations_min = std::min(s.iterations_min, it);
        s.refine_node_updates += nodes * sweepsRun;
        if (sweepsRun > 0) {
            // the residual window: the last nSweepKinds refinement sweeps the field ran
            for (int j = std::max(0, sweepsRun - nSweepKinds); j < sweepsRun; ++j) {
                unsigned long long bits = lastRes[static_cast<size_t>(i) * resStride + nSweepKinds + j];
                double r;
                std::memcpy(&r, &bits, sizeof(r));
                rl = std::max(rl, r);
            }
        }
    }
    s.residual_last = rl;
    s.sweeps_launched = sweepsLaunched;
    s.sweep_ms = -1;
    if (profile) {
        double tot = 0;
        for (int i = 0; i < sweepsLaunched; ++i) {
            float m = 0;
            cudaEventElapsedTime(&m, c->sweepEv[2 * i], c->sweepEv[2 * i + 1]);
            tot += m;
        }
        s.sweep_ms = tot;
    }
    s.kernel_launches = launches;
    s.device_ms = ms;
    s.reset_nodes = static_cast<long long>(resets);
    c->stats = s;
    c->last.valid = false;
    if (aborted) return fail(EIKX_ERR_TIMEOUT, "a bounded inter-tile wait ran out; the fields are not valid");
    c->last.valid = true;
    c->last.dim = DIM;
    c->last.precision = P;
    c->last.nSrc = nSrc;
    c->last.nx = nx; c->last.ny = ny; c->last.nz = nz; c->last.Px = Px;
    c->last.fieldStride = fieldStride;
    c->last.dx = dx; c->last.dy = dy; c->last.dz = dz;
    c->last.x0 = x0; c->last.y0 = y0; c->last.z0 = z0;
    c->last.corners = corners;
    return EIKX_OK;
}

// Spacing constants of the non-uniform 3D solver in the field type
// (include/private/solver3d.hpp:247-261).
template <class T> eikx::Spacing3<T> spacing3(double dx, double dy, double dz) {
    const T tdx = static_cast<T>(dx), tdy = static_cast<T>(dy), tdz = static_cast<T>(dz);
    eikx::Spacing3<T> g;
    g.dx = tdx; g.dy = tdy; g.dz = tdz;
    g.dxInv = 1 / tdx; g.dyInv = 1 / tdy; g.dzInv = 1 / tdz;
    g.dx2Inv = 1 / (tdx * tdx); g.dy2Inv = 1 / (tdy * tdy); g.dz2Inv = 1 / (tdz * tdz);
    g.dx_dz = tdx / tdz; g.dz_dx = tdz / tdx; g.dy_dz = tdy / tdz; g.dz_dy = tdz / tdy;
    g.dx_dy = tdx / tdy; g.dy_dx = tdy / tdx;
    g.dx2_p_dz2_inv = 1 / (tdx * tdx + tdz * tdz);
    g.dy2_p_dz2_inv = 1 / (tdy * tdy + tdz * tdz);
    g.dx2_p_dy2_inv = 1 / (tdx * tdx + tdy * tdy);
    return g;
}

bool uniformSpacing3(double dx, double dy, double dz, double eps) {
    return std::abs(dx - dy) < eps && std::abs(dx - dz) < eps;
}

// Checks one model of a batch; returns an error message or "".
std::string checkModel(const eikx_model3d &m, int i) {
    const std::string who = "model " + std::to_string(i) + ": ";
    if (m.nx < 3 || m.ny < 3 || m.nz < 3) return who + "grid needs at least 3 points in each direction";
    if (!(m.dx > 0) || !(m.dy > 0) || !(m.dz > 0)) return who + "grid spacing must be positive";
    if (!m.model) return who + "model is NULL";
    if (m.model_kind != EIKX_CELL_SLOWNESS && m.model_kind != EIKX_NODAL_VELOCITY)
        return who + "model_kind must be EIKX_CELL_SLOWNESS or EIKX_NODAL_VELOCITY";
    if (m.dtype != EIKX_F32 && m.dtype != EIKX_F64) return who + "dtype must be EIKX_F32 or EIKX_F64";
    if (m.ordering != 0 && m.ordering != 1) return who + "ordering must be 0 (natural) or 1";
    if (m.where != EIKX_HOST && m.where != EIKX_DEVICE) return who + "where must be EIKX_HOST or EIKX_DEVICE";
    if (m.n_src < 1 || !m.src) return who + "needs at least one source";
    if (!m.t_out) return who + "t_out is NULL";
    if (m.t_where != EIKX_HOST && m.t_where != EIKX_DEVICE) return who + "t_where must be EIKX_HOST or EIKX_DEVICE";
    return "";
}

// One schedule over the selected models of a batch (all with uniform or all with
// non-uniform spacing).  Statistics are accumulated into `agg`.
template <class T>
eikx_status solveBatch3(eikx_ctx *c, const eikx_model3d *models, const std::vector<int> &sel, bool uniform,
                        const eikx_options &o, eikx_stats &agg) {
    BatchWorkspace &w = c->bw;
    constexpr int V = 16 / sizeof(T);
    constexpr int W = sizeof(T) / 4;
    const int shape = o.block_shape > 0 ? o.block_shape - 1 : eikx::kShape8x4;
    const int ly = eikx::shapeLY(shape), lz = eikx::shapeLZ(shape);
    const int nM = static_cast<int>(sel.size());
    struct Layout {
        int nx, ny, nz, Px, spPitch, tilesY, tilesZ, firstUnit, nSrc;
        long long fieldStride, spPlane, spElems, faceWords;
        size_t ttOff, spOff, mboxOff;
    };
    std::vector<Layout> L(nM);
    size_t ttElems = 0, spElems = 0, mboxWords = 0, maxCells = 0, maxInBytes = 0, nItems = 0;
    int nUnits = 0;
    for (int i = 0; i < nM; ++i) {
        const eikx_model3d &m = models[sel[i]];
        Layout &l = L[i];
        l.nx = m.nx; l.ny = m.ny; l.nz = m.nz;
        l.Px = roundUp(m.nx, 4);
        l.spPitch = l.Px + 8;
        l.tilesY = (m.ny + ly - 1) / ly;
        l.tilesZ = (m.nz + lz - 1) / lz;
        l.nSrc = m.n_src;
        l.firstUnit = nUnits;
        l.fieldStride = static_cast<long long>(l.Px) * m.ny * m.nz;
        l.spPlane = static_cast<long long>(l.spPitch) * (m.ny + 1);
        l.spElems = l.spPlane * (m.nz + 1);
        l.faceWords = static_cast<long long>(ly + lz) * l.Px * W;
        l.ttOff = ttElems;
        ttElems += static_cast<size_t>(l.fieldStride) * m.n_src;
        l.spOff = spElems;
        spElems += 2 * static_cast<size_t>(l.spElems);
        l.mboxOff = mboxWords;
        mboxWords += static_cast<size_t>(m.n_src) * l.tilesY * l.tilesZ * l.faceWords;
        nUnits += m.n_src;
        nItems += static_cast<size_t>(m.n_src) * l.tilesY * l.tilesZ;
        const size_t cells = static_cast<size_t>(m.nx - 1) * (m.ny - 1) * (m.nz - 1);
        const size_t nIn = m.model_kind == EIKX_NODAL_VELOCITY ? static_cast<size_t>(m.nx) * m.ny * m.nz : cells;
        maxCells = std::max(maxCells, cells);
        maxInBytes = std::max(maxInBytes, nIn * (m.dtype == EIKX_F64 ? 8 : 4));
    }
    if (nItems > static_cast<size_t>(std::numeric_limits<int>::max()))
        return fail(EIKX_ERR_INVALID, "batch has too many warp blocks");
    const int nSweepKinds = 8;
    const int nSweeps = std::max(0, o.n_sweeps);
    const int resStride = nSweepKinds * (1 + nSweeps);

    const bool near64 = sizeof(T) == 4 && o.near_fp64;
    const void *before[] = {w.tt.p, w.sp.p, w.mbox.p, w.epoch.p, w.residual.p, w.converged.p, w.iterations.p,
                            w.order.p, w.srcs.p, w.corners.p, w.units.p, w.srcs64.p, w.factor.p};
    EIKX_CUDA(w.tt.ensure(ttElems * sizeof(T)));
    EIKX_CUDA(w.sp.ensure(spElems * sizeof(T)));
    if (w.mbox.bytes < mboxWords * 8 || !w.mbox.p) {
        // fresh words carry tag 0, which no sweep uses
        EIKX_CUDA(w.mbox.ensure(mboxWords * 8));
        EIKX_CUDA(cudaMemsetAsync(w.mbox.p, 0, w.mbox.bytes, c->stream));
    }
    if (!w.epoch.p) {
        EIKX_CUDA(w.epoch.ensure(2 * sizeof(unsigned)));
        EIKX_CUDA(cudaMemsetAsync(w.epoch.p, 0, 2 * sizeof(unsigned), c->stream));
    }
    EIKX_CUDA(w.queue.ensure(2 * sizeof(unsigned)));
    EIKX_CUDA(w.residual.ensure(static_cast<size_t>(nUnits) * resStride * 8));
    EIKX_CUDA(w.converged.ensure(static_cast<size_t>(nUnits) * 4));
    EIKX_CUDA(w.iterations.ensure(static_cast<size_t>(nUnits) * 4));
    EIKX_CUDA(w.abortFlag.ensure(sizeof(int)));
    EIKX_CUDA(w.order.ensure(nItems * 16));
    EIKX_CUDA(w.srcs.ensure(static_cast<size_t>(nUnits) * sizeof(eikx::SourceT<T>)));
    EIKX_CUDA(w.corners.ensure(static_cast<size_t>(nUnits) * sizeof(eikx::Corner3)));
    EIKX_CUDA(w.units.ensure(static_cast<size_t>(nUnits) * sizeof(eikx::Grid3Unit<T>)));
    EIKX_CUDA(w.slow64.ensure(maxCells * sizeof(double)));
    EIKX_CUDA(w.input.ensure(maxInBytes));
    EIKX_CUDA(w.badFlag.ensure(sizeof(int)));
    EIKX_CUDA(w.srcCells.ensure(static_cast<size_t>(nUnits) * sizeof(double) + sizeof(int)));
    if (near64) EIKX_CUDA(w.srcs64.ensure(static_cast<size_t>(nUnits) * sizeof(eikx::SourceFp64)));
    // the factor tables are laid out below, once the sources are located; a grown buffer
    // drops the cached graph there
    const void *after[] = {w.tt.p, w.sp.p, w.mbox.p, w.epoch.p, w.residual.p, w.converged.p, w.iterations.p,
                           w.order.p, w.srcs.p, w.corners.p, w.units.p, w.srcs64.p, w.factor.p};
    if (std::memcmp(before, after, sizeof(before)) != 0) w.dropGraph();

    // models -> cell slowness (FP64, natural) -> two padded copies in the sweep precision;
    // sources located on each model as eikx_solve3d does.  The whole batch is one stream
    // of work with a single synchronisation: positivity is checked on the device into one
    // flag and only the source cells' slowness comes back to the host.
    std::vector<eikx::SourceT<T>> srcT(nUnits);
    std::vector<eikx::Corner3> corners(nUnits);
    std::vector<eikx::Grid3Unit<T>> units(nUnits);
    std::vector<std::array<double, 3>> offs(nUnits), unitSpacing(nUnits);
    std::vector<std::array<int, 3>> unitGrid(nUnits);
    T *ttBase = w.tt.as<T>();
    T *spBase = w.sp.as<T>();
    unsigned long long *mbBase = w.mbox.as<unsigned long long>();
    double *srcCell = static_cast<double *>(w.srcCells.p);
    EIKX_CUDA(cudaStreamSynchronize(c->stream));   // pinned staging of a previous call is free
    EIKX_CUDA(cudaMemsetAsync(w.badFlag.p, 0, sizeof(int), c->stream));
    for (int i = 0; i < nM; ++i) {
        const eikx_model3d &m = models[sel[i]];
        const Layout &l = L[i];
        // locate the sources first: the cell slowness they need is copied out below
        for (int j = 0; j < m.n_src; ++j) {
            const int u = l.firstUnit + j;
            int cx, cy, cz;
            double ox, oy, oz;
            if (!locate(m.src[j].x, m.x0, m.dx, m.nx, &cx, &ox) || !locate(m.src[j].y, m.y0, m.dy, m.ny, &cy, &oy) ||
                !locate(m.src[j].z, m.z0, m.dz, m.nz, &cz, &oz))
                return fail(EIKX_ERR_INVALID, "model " + std::to_string(sel[i]) + ": source " + std::to_string(j) +
                                                  " lies outside the grid");
            srcT[u].isx = cx; srcT[u].isy = cy; srcT[u].isz = cz;
            offs[u] = {ox, oy, oz};
            unitSpacing[u] = {m.dx, m.dy, m.dz};
            unitGrid[u] = {m.nx, m.ny, m.nz};
        }
        const bool nodal = m.model_kind == EIKX_NODAL_VELOCITY;
        const size_t nCell = static_cast<size_t>(m.nx - 1) * (m.ny - 1) * (m.nz - 1);
        const size_t nIn = nodal ? static_cast<size_t>(m.nx) * m.ny * m.nz : nCell;
        const size_t inBytes = nIn * (m.dtype == EIKX_F64 ? 8 : 4);
        const void *d = m.model;
        if (m.where == EIKX_HOST) {
            EIKX_CUDA(cudaMemcpyAsync(w.input.p, m.model, inBytes, cudaMemcpyHostToDevice, c->stream));
            d = w.input.p;
        }
        double *slow = w.slow64.as<double>();
        if (m.dtype == EIKX_F32) {
            const float *f = static_cast<const float *>(d);
            if (nodal) EIKX_CUDA(eikx::launchNodalToCell3<float>(slow, f, m.nx, m.ny, m.nz, m.ordering, c->stream));
            else EIKX_CUDA(eikx::launchCellsToNatural3<float>(slow, f, m.nx, m.ny, m.nz, m.ordering, c->stream));
        } else {
            const double *f = static_cast<const double *>(d);
            if (nodal) EIKX_CUDA(eikx::launchNodalToCell3<double>(slow, f, m.nx, m.ny, m.nz, m.ordering, c->stream));
            else EIKX_CUDA(eikx::launchCellsToNatural3<double>(slow, f, m.nx, m.ny, m.nz, m.ordering, c->stream));
        }
        EIKX_CUDA(eikx::launchCheckPositive(slow, static_cast<long long>(nCell), w.badFlag.as<int>(), c->stream));
        EIKX_CUDA((eikx::launchPadSlowness3<T, double>(spBase + l.spOff, l.spPitch, V - 1, slow, m.nx, m.ny, m.nz,
                                                       c->stream)));
        EIKX_CUDA((eikx::launchPadSlowness3<T, double>(spBase + l.spOff + l.spElems, l.spPitch, 0, slow, m.nx, m.ny,
                                                       m.nz, c->stream)));
        for (int j = 0; j < m.n_src; ++j) {
            const int u = l.firstUnit + j;
            const size_t cell = (static_cast<size_t>(srcT[u].isz) * (m.ny - 1) + srcT[u].isy) * (m.nx - 1) + srcT[u].isx;
            EIKX_CUDA(cudaMemcpyAsync(srcCell + u, slow + cell, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        }
        const eikx::Spacing3<T> g = spacing3<T>(m.dx, m.dy, m.dz);
        for (int j = 0; j < m.n_src; ++j) {
            eikx::Grid3Unit<T> &gu = units[l.firstUnit + j];
            gu.tt = ttBase + l.ttOff + static_cast<size_t>(j) * l.fieldStride;
            gu.spPos = spBase + l.spOff;
            gu.spNeg = spBase + l.spOff + l.spElems;
            gu.mbox = mbBase + l.mboxOff + static_cast<size_t>(j) * l.tilesY * l.tilesZ * l.faceWords;
            gu.spPlane = l.spPlane;
            gu.spPitch = l.spPitch;
            gu.Px = l.Px; gu.nx = m.nx; gu.ny = m.ny; gu.nz = m.nz;
            gu.tilesY = l.tilesY; gu.tilesZ = l.tilesZ; gu.pad = 0;
            gu.h = static_cast<T>(m.dx);
            gu.sp3 = g;
        }
    }
    int *bad = reinterpret_cast<int *>(srcCell + nUnits);
    EIKX_CUDA(cudaMemcpyAsync(bad, w.badFlag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    EIKX_CUDA(cudaStreamSynchronize(c->stream));
    if (*bad) return fail(EIKX_ERR_INVALID, "Non-positive velocities detected");
    std::vector<eikx::SourceFp64> srcT64;
    for (int u = 0; u < nUnits; ++u) {
        const double sc = srcCell[u];
        srcT[u].xs = static_cast<T>(offs[u][0]);
        srcT[u].ys = static_cast<T>(offs[u][1]);
        srcT[u].zs = static_cast<T>(offs[u][2]);
        srcT[u].sSrc = static_cast<T>(sc);
        if (near64)
            srcT64.push_back(sourceFp64(offs[u], srcT[u].isx, srcT[u].isy, srcT[u].isz,
                                        std::max(0, o.factored_radius), unitGrid[u][0], unitGrid[u][1],
                                        unitGrid[u][2], unitSpacing[u][0], unitSpacing[u][1], unitSpacing[u][2],
                                        reinterpret_cast<const float *>(units[u].spNeg), units[u].spPitch));
        corners[u] = eikx::Corner3{srcT[u].isx, srcT[u].isy, srcT[u].isz, offs[u][0], offs[u][1], offs[u][2],
                                   static_cast<double>(static_cast<T>(sc))};
    }

    if (near64) {
        for (const auto &f : srcT64)
            if (f.bnx == 0)
                return fail(EIKX_ERR_UNSUPPORTED, "near_fp64: the factored region of radius " +
                                                      std::to_string(o.factored_radius) + " needs more than " +
                                                      std::to_string(eikx::kMaxFactorTable) + " table entries");
        const void *fb = w.factor.p;
        EIKX_CUDA(assignFactorTables(srcT64, w.factor));
        if (w.factor.p != fb) w.dropGraph();
    }

    // work order: every unit's warp blocks, sorted by the step at which they can start
    struct Item { int key, u, b, c; };
    std::vector<Item> items;
    items.reserve(nItems);
    for (int i = 0; i < nM; ++i)
        for (int j = 0; j < L[i].nSrc; ++j)
            for (int cc = 0; cc < L[i].tilesZ; ++cc)
                for (int bb = 0; bb < L[i].tilesY; ++bb) items.push_back({bb * ly + cc * lz, L[i].firstUnit + j, bb, cc});
    std::stable_sort(items.begin(), items.end(), [](const Item &a, const Item &b) {
        if (a.key != b.key) return a.key < b.key;
        if (a.u != b.u) return a.u < b.u;
        return a.b < b.b;
    });
    const size_t srcBytes = srcT.size() * sizeof(eikx::SourceT<T>);
    const size_t cornerBytes = corners.size() * sizeof(eikx::Corner3);
    const size_t unitBytes = units.size() * sizeof(eikx::Grid3Unit<T>);
    const size_t orderBytes = items.size() * 16;
    const size_t src64Bytes = srcT64.size() * sizeof(eikx::SourceFp64);
    EIKX_CUDA(w.stage.ensure(srcBytes + cornerBytes + unitBytes + orderBytes + src64Bytes + 64));
    char *stage = static_cast<char *>(w.stage.p);
    std::memcpy(stage, srcT.data(), srcBytes);
    std::memcpy(stage + srcBytes, corners.data(), cornerBytes);
    std::memcpy(stage + srcBytes + cornerBytes, units.data(), unitBytes);
    int *ord = reinterpret_cast<int *>(stage + srcBytes + cornerBytes + unitBytes);
    for (size_t k = 0; k < items.size(); ++k) {
        ord[4 * k] = items[k].u; ord[4 * k + 1] = items[k].b; ord[4 * k + 2] = items[k].c; ord[4 * k + 3] = 0;
    }
    EIKX_CUDA(cudaMemcpyAsync(w.srcs.p, stage, srcBytes, cudaMemcpyHostToDevice, c->stream));
    EIKX_CUDA(cudaMemcpyAsync(w.corners.p, stage + srcBytes, cornerBytes, cudaMemcpyHostToDevice, c->stream));
    EIKX_CUDA(cudaMemcpyAsync(w.units.p, stage + srcBytes + cornerBytes, unitBytes, cudaMemcpyHostToDevice, c->stream));
    EIKX_CUDA(cudaMemcpyAsync(w.order.p, ord, orderBytes, cudaMemcpyHostToDevice, c->stream));
    if (near64) {
        char *qstage = stage + srcBytes + cornerBytes + unitBytes + orderBytes;
        std::memcpy(qstage, srcT64.data(), src64Bytes);
        EIKX_CUDA(cudaMemcpyAsync(w.srcs64.p, qstage, src64Bytes, cudaMemcpyHostToDevice, c->stream));
    }

    const int nSweepLaunches = nSweepKinds * ((o.init_sweeps ? 1 : 0) + nSweeps);
    eikx::SolveState st{};
    st.queue[0] = w.queue.as<unsigned>();
    st.queue[1] = w.queue.as<unsigned>() + 1;
    st.mbox = w.mbox.as<unsigned long long>();
    st.epoch = w.epoch.as<unsigned>();
    st.epochStride = nSweepLaunches + 1;
    st.residual = w.residual.as<unsigned long long>();
    st.residualStride = resStride;
    st.converged = w.converged.as<int>();
    st.sweepsRun = w.iterations.as<int>();
    st.abortFlag = w.abortFlag.as<int>();
    st.order = w.order.as<int4>();
    st.totalItems = static_cast<int>(nItems);
    const int spinLog2 = o.spin_limit_log2 > 0 ? std::min(o.spin_limit_log2, 40) : 22;
    st.spinLimit = 1ull << spinLog2;
    int perSM = eikx::sweep3ChunkBlocksPerSM<T>(uniform, true, shape);
    if (o.blocks_per_sm > 0) perSM = std::min(perSM, o.blocks_per_sm);
    const int blocks = std::max(1, static_cast<int>(std::min<size_t>(
                                       static_cast<size_t>(c->numSMs) * perSM,
                                       (nItems + eikx::kWarpsPerBlock - 1) / eikx::kWarpsPerBlock)));

    int launches = 0, sweepsLaunched = 0;
    const bool profile = o.profile_sweeps != 0;
    if (profile) {
        while (static_cast<int>(c->sweepEv.size()) < 2 * nSweepLaunches) {
            cudaEvent_t e;
            EIKX_CUDA(cudaEventCreate(&e));
            c->sweepEv.push_back(e);
        }
    }
    // models with host output are copied out, on a second stream, at the end of the iteration
    // in which all their fields have converged (see solveImpl)
    bool anyHost = false;
    for (int i = 0; i < nM; ++i) anyHost = anyHost || models[sel[i]].t_where == EIKX_HOST;
    const bool early = anyHost && nSweeps > 1 && o.tolerance > 0 && o.profile_sweeps == 0;
    int *iterFlags = nullptr;
    if (early) {
        while (static_cast<int>(c->iterEv.size()) < nSweeps) {
            cudaEvent_t e;
            EIKX_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            c->iterEv.push_back(e);
        }
        EIKX_CUDA(w.iterFlags.ensure(static_cast<size_t>(nSweeps) * nUnits * sizeof(int)));
        iterFlags = static_cast<int *>(w.iterFlags.p);
    }
    auto enqueue = [&]() -> eikx_status {
        launches = 0;
        sweepsLaunched = 0;
        int buf = 0;
        EIKX_CUDA(eikx::launchResetState(st, nUnits, buf, c->stream));
        ++launches;
        if (near64) {
            EIKX_CUDA(eikx::launchFactorTables(w.srcs64.as<eikx::SourceFp64>(), nUnits, c->stream));
            ++launches;
        }
        for (int i = 0; i < nM; ++i) {
            const eikx_model3d &m = models[sel[i]];
            EIKX_CUDA(eikx::launchInit3<T>(ttBase + L[i].ttOff, L[i].nSrc, L[i].fieldStride, L[i].Px, m.nx, m.ny, m.nz,
                                           m.dx, m.dy, m.dz, w.corners.as<eikx::Corner3>() + L[i].firstUnit,
                                           o.init_fp64 ? 1 : 0, c->stream));
            launches += 2;   // the fill and the corner kernel
        }
        auto sweep = [&](int e, int init, int slot) -> eikx_status {
            if (profile) EIKX_CUDA(cudaEventRecord(c->sweepEv[2 * sweepsLaunched], c->stream));
            eikx::Sweep3Args<T> a{};
            a.srcs = w.srcs.as<eikx::SourceT<T>>(); a.st = st; a.buf = buf; a.residualSlot = slot;
            a.sweepIndex = sweepsLaunched;
            a.sweep = e; a.init = init; a.radius = o.factored_radius;
            a.units = w.units.as<eikx::Grid3Unit<T>>();
            a.srcs64 = near64 ? w.srcs64.as<eikx::SourceFp64>() : nullptr;
            EIKX_CUDA(eikx::launchSweep3Chunk<T>(a, uniform, shape, blocks, c->stream));
            if (profile) EIKX_CUDA(cudaEventRecord(c->sweepEv[2 * sweepsLaunched + 1], c->stream));
            buf ^= 1;
            ++launches;
            ++sweepsLaunched;
            return EIKX_OK;
        };
        if (o.init_sweeps)
            for (int e = 0; e < nSweepKinds; ++e)
                if (eikx_status r = sweep(e, 1, e); r != EIKX_OK) return r;
        for (int k = 0; k < nSweeps; ++k) {
            for (int e = 0; e < nSweepKinds; ++e) {
                if (eikx_status r = sweep(e, 0, nSweepKinds * (1 + k) + e); r != EIKX_OK) return r;
                EIKX_CUDA(checkAfterSweep(st, nUnits, nSweepKinds, nSweepKinds * k + e, o.tolerance, c->stream));
                ++launches;
            }
            if (early) {
                EIKX_CUDA(cudaMemcpyAsync(iterFlags + static_cast<size_t>(k) * nUnits, w.converged.p,
                                          nUnits * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
                EIKX_CUDA(cudaEventRecordWithFlags(c->iterEv[k], c->stream, cudaEventRecordExternal));
            }
        }
        return EIKX_OK;
    };

    // graph key: everything the captured launches depend on
    std::vector<double> key = {static_cast<double>(sizeof(T)), uniform ? 1.0 : 0.0, static_cast<double>(nM),
                               static_cast<double>(o.n_sweeps), static_cast<double>(o.factored_radius),
                               static_cast<double>(o.init_sweeps), static_cast<double>(o.init_fp64), o.tolerance,
                               static_cast<double>(st.spinLimit), static_cast<double>(blocks),
                               static_cast<double>(shape), static_cast<double>(o.near_fp64 ? 1 : 0)};
    for (int i = 0; i < nM; ++i) {
        const eikx_model3d &m = models[sel[i]];
        for (double v : {static_cast<double>(m.nx), static_cast<double>(m.ny), static_cast<double>(m.nz), m.dx, m.dy,
                         m.dz, static_cast<double>(m.n_src)})
            key.push_back(v);
    }
    for (const void *p : after) key.push_back(static_cast<double>(reinterpret_cast<uintptr_t>(p)));
    key.push_back(early ? 1.0 : 0.0);
    key.push_back(static_cast<double>(reinterpret_cast<uintptr_t>(iterFlags)));

    if (eikx_status r = advanceEpoch(w.epochMirror, w.mbox, w.epoch, st.epochStride, c->stream); r != EIKX_OK)
        return r;
    EIKX_CUDA(cudaEventRecord(c->ev0, c->stream));
    if (c->useGraphs && !profile) {
        if (!(w.exec && w.key == key)) {
            w.dropGraph();
            cudaGraph_t graph = nullptr;
            EIKX_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            eikx_status r = enqueue();
            cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
            if (r != EIKX_OK) {
                if (graph) cudaGraphDestroy(graph);
                return r;
            }
            EIKX_CUDA(ce);
            cudaError_t ie = cudaGraphInstantiate(&w.exec, graph, 0);
            cudaGraphDestroy(graph);
            EIKX_CUDA(ie);
            w.key = key;
            w.launches = launches;
        }
        EIKX_CUDA(cudaGraphLaunch(w.exec, c->stream));
        launches = w.launches;
        sweepsLaunched = nSweepLaunches;
    } else {
        if (eikx_status r = enqueue(); r != EIKX_OK) return r;
    }
    auto copyModel = [&](int i, cudaStream_t s) -> cudaError_t {
        const eikx_model3d &m = models[sel[i]];
        const cudaMemcpyKind kind = m.t_where == EIKX_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        return eikx::copyRows(m.t_out, static_cast<size_t>(m.nx) * sizeof(T), ttBase + L[i].ttOff,
                                 static_cast<size_t>(L[i].Px) * sizeof(T), static_cast<size_t>(m.nx) * sizeof(T),
                                 static_cast<size_t>(m.ny) * m.nz * m.n_src, kind, s);
    };
    std::vector<char> copied(nM, 0);
    if (early) {
        int left = 0;
        for (int i = 0; i < nM; ++i) left += models[sel[i]].t_where == EIKX_HOST;
        for (int k = 0; k < nSweeps && left > 0; ++k) {
            EIKX_CUDA(cudaEventSynchronize(c->iterEv[k]));
            const int *fl = iterFlags + static_cast<size_t>(k) * nUnits;
            bool waited = false;
            for (int i = 0; i < nM; ++i) {
                if (copied[i] || models[sel[i]].t_where != EIKX_HOST) continue;
                bool all = true;
                for (int j = 0; j < L[i].nSrc && all; ++j) all = fl[L[i].firstUnit + j] != 0;
                if (!all) continue;
                if (!waited) EIKX_CUDA(cudaStreamWaitEvent(c->copyStream, c->iterEv[k], 0));
                waited = true;
                EIKX_CUDA(copyModel(i, c->copyStream));
                copied[i] = 1;
                --left;
            }
        }
    }
    for (int i = 0; i < nM; ++i)
        if (!copied[i]) EIKX_CUDA(copyModel(i, c->stream));
    if (early) {
        EIKX_CUDA(cudaEventRecord(c->copyDone, c->copyStream));
        EIKX_CUDA(cudaStreamWaitEvent(c->stream, c->copyDone, 0));
    }
    EIKX_CUDA(cudaEventRecord(c->ev1, c->stream));
    std::vector<int> iters(nUnits);
    int aborted = 0;
    EIKX_CUDA(cudaMemcpyAsync(iters.data(), w.iterations.p, nUnits * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    EIKX_CUDA(cudaMemcpyAsync(&aborted, w.abortFlag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    std::vector<unsigned long long> res;
    if (nSweeps > 0) {
        res.resize(static_cast<size_t>(nUnits) * resStride);
        EIKX_CUDA(cudaMemcpyAsync(res.data(), w.residual.p, res.size() * 8, cudaMemcpyDeviceToHost, c->stream));
    }
    EIKX_CUDA(cudaStreamSynchronize(c->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    std::vector<long long> unitNodes(nUnits);
    for (int i = 0; i < nM; ++i)
        for (int j = 0; j < L[i].nSrc; ++j)
            unitNodes[L[i].firstUnit + j] = static_cast<long long>(L[i].nx) * L[i].ny * L[i].nz;
    for (int u = 0; u < nUnits; ++u) {
        // iters[u] holds the refinement sweeps the unit ran; report iterations begun
        const int sweepsRun = iters[u], it = (sweepsRun + nSweepKinds - 1) / nSweepKinds;
        agg.iterations_max = std::max(agg.iterations_max, it);
        agg.iterations_min = std::min(agg.iterations_min, it);
        agg.refine_node_updates += unitNodes[u] * sweepsRun;
        if (sweepsRun > 0)
            for (int j = std::max(0, sweepsRun - nSweepKinds); j < sweepsRun; ++j) {
                double r;
                std::memcpy(&r, &res[static_cast<size_t>(u) * resStride + nSweepKinds + j], sizeof(r));
                agg.residual_last = std::max(agg.residual_last, r);
            }
    }
    agg.n_fields += nUnits;
    agg.sweeps_launched += sweepsLaunched;
    agg.kernel_launches += launches;
    agg.device_ms += ms;
    if (profile) {
        double tot = 0;
        for (int i = 0; i < sweepsLaunched; ++i) {
            float m = 0;
            cudaEventElapsedTime(&m, c->sweepEv[2 * i], c->sweepEv[2 * i + 1]);
            tot += m;
        }
        agg.sweep_ms = (agg.sweep_ms < 0 ? 0 : agg.sweep_ms) + tot;
    }
    if (aborted) return fail(EIKX_ERR_TIMEOUT, "a bounded inter-tile wait ran out; the fields are not valid");
    return EIKX_OK;
}

template <class T>
eikx_status autotune3(eikx_ctx *c, const std::vector<double> &xyz, int nSrc, eikx_tuning *res) {
    const int P = precOf<T>();
    const size_t n = static_cast<size_t>(c->nx) * c->ny * c->nz;
    EIKX_CUDA(c->tuneOut.ensure(n * nSrc * sizeof(T)));
    const double eps = std::numeric_limits<T>::epsilon() * 100;
    const bool uniform = uniformSpacing3(c->dx, c->dy, c->dz, eps);
    eikx_options base;
    eikx_options_default(&base);
    base.n_sweeps = 1;
    base.tolerance = -1;
    base.profile_sweeps = 1;
    std::vector<eikx_options> cands;
    auto add = [&](int kernel, int pair, int shape, int perSM) {
        eikx_options o = base;
        o.sweep_kernel = kernel;
        o.pair_fields = pair;
        o.block_shape = shape;
        o.blocks_per_sm = perSM;
        cands.push_back(o);
    };
    for (int shape = 0; shape < eikx::kNumShapes; ++shape) {
        const int mx = eikx::sweep3ChunkBlocksPerSM<T>(uniform, false, shape);
        add(eikx::kChunkStep, 0, shape + 1, mx);
        if (mx / 2 >= 1 && mx / 2 < mx) add(eikx::kChunkStep, 0, shape + 1, mx / 2);
    }
    add(eikx::kNodeStep, 0, 1, eikx::sweep3BlocksPerSM<T>(uniform));
    if (std::is_same<T, float>::value && uniform && nSrc >= 2) add(eikx::kChunkStep, 1, 1, eikx::sweep3PairBlocksPerSM());
    double best = 1e300, dflt = -1;
    eikx_tuning pick{};
    for (size_t i = 0; i < cands.size(); ++i) {
        double ms = 0;
        for (int rep = 0; rep < 2; ++rep) {
            if (eikx_status r = solveImpl<T, 3>(c, xyz.data(), nSrc, cands[i], c->tuneOut.p, EIKX_DEVICE); r)
                return r;
            ms = c->stats.sweep_ms / std::max(1, c->stats.sweeps_launched);
        }
        if (i == 0) dflt = ms;   // chunk-step, 8x4, full grid: the untuned default
        if (ms < best) {
            best = ms;
            pick.sweep_kernel = cands[i].sweep_kernel;
            pick.pair_fields = cands[i].pair_fields;
            pick.block_shape = cands[i].block_shape;
            pick.blocks_per_sm = cands[i].blocks_per_sm;
        }
    }
    pick.ms_per_sweep = best;
    pick.default_ms_per_sweep = dflt;
    pick.candidates = static_cast<int>(cands.size());
    c->tuning[tuneKey(P, uniform, c->nx, c->ny, c->nz, nSrc)] = pick;
    if (res) *res = pick;
    return EIKX_OK;
}

eikx_status fillOptions(const eikx_options *in, eikx_options *out) {
    if (in) *out = *in; else eikx_options_default(out);
    if (out->n_sweeps < 0) return fail(EIKX_ERR_INVALID, "n_sweeps must be non-negative");
    if (out->factored_radius < 0) out->factored_radius = 0;
    if (out->block_shape < 0 || out->block_shape > eikx::kNumShapes)
        return fail(EIKX_ERR_INVALID, "block_shape must be 0..3");
    if (out->sweep_kernel < 0 || out->sweep_kernel > 2) return fail(EIKX_ERR_INVALID, "sweep_kernel must be 0..2");
    if (out->blocks_per_sm < 0) return fail(EIKX_ERR_INVALID, "blocks_per_sm must be >= 0");
    if (out->test_tag_margin < 0) return fail(EIKX_ERR_INVALID, "test_tag_margin must be >= 0");
    if (out->near_fp64 < 0 || out->near_fp64 > 1) return fail(EIKX_ERR_INVALID, "near_fp64 must be 0 or 1");
    if (out->warm_gate < 0 || out->warm_gate > 1) return fail(EIKX_ERR_INVALID, "warm_gate must be 0 or 1");
    if (out->max_in_flight < 0) return fail(EIKX_ERR_INVALID, "max_in_flight must be >= 0");
    return EIKX_OK;
}

}  // namespace

extern "C" {

void eikx_options_default(eikx_options *opt) {
    if (!opt) return;
    std::memset(opt, 0, sizeof(*opt));
    opt->n_sweeps = 5;            // src/solverOptions.cpp:7
    opt->tolerance = 1.e-5;       // src/solverOptions.cpp:5
    opt->factored_radius = 3;     // src/solverOptions.cpp:6
    opt->init_sweeps = 1;
    opt->init_fp64 = 1;
    opt->spin_limit_log2 = 22;
    opt->pair_fields = 0;
}

const char *eikx_last_error(void) { return gLastError.c_str(); }

eikx_status eikx_create(eikx_ctx **ctx, int device) {
    if (!ctx) return fail(EIKX_ERR_INVALID, "ctx is NULL");
    *ctx = nullptr;
    int n = 0;
    EIKX_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(EIKX_ERR_INVALID, "device " + std::to_string(device) + " not present");
    EIKX_CUDA(cudaSetDevice(device));
    std::unique_ptr<eikx_ctx> c(new eikx_ctx());
    c->device = device;
    EIKX_CUDA(cudaDeviceGetAttribute(&c->numSMs, cudaDevAttrMultiProcessorCount, device));
    EIKX_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    EIKX_CUDA(cudaEventCreate(&c->ev0));
    EIKX_CUDA(cudaEventCreate(&c->ev1));
    EIKX_CUDA(cudaStreamCreateWithFlags(&c->copyStream, cudaStreamNonBlocking));
    EIKX_CUDA(cudaEventCreateWithFlags(&c->copyDone, cudaEventDisableTiming));
    if (const char *g = std::getenv("EIKX_GRAPHS")) c->useGraphs = std::atoi(g) != 0;
    *ctx = c.release();
    return EIKX_OK;
}

eikx_status eikx_destroy(eikx_ctx *c) {
    if (!c) return EIKX_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    dropGraph(c);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->copyStream) {
        cudaStreamSynchronize(c->copyStream);
        cudaStreamDestroy(c->copyStream);
    }
    if (c->copyDone) cudaEventDestroy(c->copyDone);
    for (cudaEvent_t e : c->iterEv) cudaEventDestroy(e);
    for (cudaEvent_t e : c->sweepEv) cudaEventDestroy(e);
    for (cudaEvent_t e : c->sw.bufEv) cudaEventDestroy(e);
    if (c->sw.boundary) cudaEventDestroy(c->sw.boundary);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return EIKX_OK;
}

eikx_status eikx_get_stats(const eikx_ctx *c, eikx_stats *s) {
    if (eikx_status r = checkCtx(c); r) return r;
    if (!s) return fail(EIKX_ERR_INVALID, "stats is NULL");
    *s = c->stats;
    return EIKX_OK;
}

eikx_status eikx_set_grid3d(eikx_ctx *c, int nx, int ny, int nz, double dx, double dy, double dz, double x0,
                            double y0, double z0) {
    if (eikx_status r = checkCtx(c); r) return r;
    // Geometry3D setters, src/geometry3d.cpp:73-80 etc.
    if (nx < 3) return fail(EIKX_ERR_INVALID, "Number of grid points in x = " + std::to_string(nx) + " must be at least 3");
    if (ny < 3) return fail(EIKX_ERR_INVALID, "Number of grid points in y = " + std::to_string(ny) + " must be at least 3");
    if (nz < 3) return fail(EIKX_ERR_INVALID, "Number of grid points in z = " + std::to_string(nz) + " must be at least 3");
    if (!(dx > 0)) return fail(EIKX_ERR_INVALID, "Grid spacing in x = " + std::to_string(dx) + " must be positive");
    if (!(dy > 0)) return fail(EIKX_ERR_INVALID, "Grid spacing in y = " + std::to_string(dy) + " must be positive");
    if (!(dz > 0)) return fail(EIKX_ERR_INVALID, "Grid spacing in z = " + std::to_string(dz) + " must be positive");
    const long long n = static_cast<long long>(nx) * ny * nz;
    if (n > (1LL << 31) - 1) return fail(EIKX_ERR_INVALID, "grid has more than 2^31-1 points");
    EIKX_CUDA(cudaSetDevice(c->device));
    c->nx = nx; c->ny = ny; c->nz = nz;
    c->dx = dx; c->dy = dy; c->dz = dz;
    c->x0 = x0; c->y0 = y0; c->z0 = z0;
    c->haveGrid3 = true;
    c->haveSlow3 = false;
    c->spadValid3[0] = c->spadValid3[1] = false;
    c->shadValid3[0] = c->shadValid3[1] = false;
    dropGraph(c);
    return EIKX_OK;
}

eikx_status eikx_set_grid2d(eikx_ctx *c, int nx, int nz, double dx, double dz, double x0, double z0) {
    if (eikx_status r = checkCtx(c); r) return r;
    if (nx < 3) return fail(EIKX_ERR_INVALID, "Number of grid points in x = " + std::to_string(nx) + " must be at least 3");
    if (nz < 3) return fail(EIKX_ERR_INVALID, "Number of grid points in z = " + std::to_string(nz) + " must be at least 3");
    if (!(dx > 0)) return fail(EIKX_ERR_INVALID, "Grid spacing in x = " + std::to_string(dx) + " must be positive");
    if (!(dz > 0)) return fail(EIKX_ERR_INVALID, "Grid spacing in z = " + std::to_string(dz) + " must be positive");
    EIKX_CUDA(cudaSetDevice(c->device));
    c->nx2 = nx; c->nz2 = nz; c->dx2 = dx; c->dz2 = dz; c->x02 = x0; c->z02 = z0;
    c->haveGrid2 = true;
    c->haveSlow2 = false;
    c->spadValid2[0] = c->spadValid2[1] = false;
    dropGraph(c);
    return EIKX_OK;
}

static eikx_status setCells(eikx_ctx *c, int dim, const void *v, int dtype, int ordering, int where, bool nodal) {
    if (eikx_status r = checkCtx(c); r) return r;
    if (dim == 3 ? !c->haveGrid3 : !c->haveGrid2) return fail(EIKX_ERR_STATE, "Class not initialized");
    if (!v) return fail(EIKX_ERR_INVALID, "velocities is NULL");
    if (dtype != EIKX_F32 && dtype != EIKX_F64) return fail(EIKX_ERR_INVALID, "dtype must be EIKX_F32 or EIKX_F64");
    if (ordering != 0 && ordering != 1) return fail(EIKX_ERR_INVALID, "ordering must be 0 (natural) or 1");
    if (where != EIKX_HOST && where != EIKX_DEVICE) return fail(EIKX_ERR_INVALID, "where must be EIKX_HOST or EIKX_DEVICE");
    EIKX_CUDA(cudaSetDevice(c->device));
    const int nx = dim == 3 ? c->nx : c->nx2, ny = dim == 3 ? c->ny : 2, nz = dim == 3 ? c->nz : c->nz2;
    const size_t nIn = nodal ? static_cast<size_t>(nx) * (dim == 3 ? ny : 1) * nz
                             : static_cast<size_t>(nx - 1) * (ny - 1) * (nz - 1);
    // Model3D/Model2D reject non-positive velocities (src/model3d.cpp:301-305): the input
    // and the resulting cell slowness are checked on the device, into one flag
    EIKX_CUDA(c->modelFlag.ensure(sizeof(int)));
    EIKX_CUDA(cudaMemsetAsync(c->modelFlag.p, 0, sizeof(int), c->stream));
    const size_t nCell = static_cast<size_t>(nx - 1) * (ny - 1) * (nz - 1);
    DevBuf &dst = dim == 3 ? c->slow3 : c->slow2;
    EIKX_CUDA(dst.ensure(nCell * sizeof(double)));
    if (dtype == EIKX_F32) {
        const float *d = nullptr;
        if (eikx_status r = toDevice<float>(c, static_cast<const float *>(v), nIn, where, &d); r) return r;
        EIKX_CUDA(eikx::launchCheckPositive(d, static_cast<long long>(nIn), c->modelFlag.as<int>(), c->stream));
        if (nodal) {
            if (dim == 3) EIKX_CUDA(eikx::launchNodalToCell3<float>(dst.as<double>(), d, nx, ny, nz, ordering, c->stream));
            else EIKX_CUDA(eikx::launchNodalToCell2<float>(dst.as<double>(), d, nx, nz, ordering, c->stream));
        } else {
            if (dim == 3) EIKX_CUDA(eikx::launchCellsToNatural3<float>(dst.as<double>(), d, nx, ny, nz, ordering, c->stream));
            else EIKX_CUDA(eikx::launchCellsToNatural2<float>(dst.as<double>(), d, nx, nz, ordering, c->stream));
        }
    } else {
        const double *d = nullptr;
        if (eikx_status r = toDevice<double>(c, static_cast<const double *>(v), nIn, where, &d); r) return r;
        EIKX_CUDA(eikx::launchCheckPositive(d, static_cast<long long>(nIn), c->modelFlag.as<int>(), c->stream));
        if (nodal) {
            if (dim == 3) EIKX_CUDA(eikx::launchNodalToCell3<double>(dst.as<double>(), d, nx, ny, nz, ordering, c->stream));
            else EIKX_CUDA(eikx::launchNodalToCell2<double>(dst.as<double>(), d, nx, nz, ordering, c->stream));
        } else {
            if (dim == 3) EIKX_CUDA(eikx::launchCellsToNatural3<double>(dst.as<double>(), d, nx, ny, nz, ordering, c->stream));
            else EIKX_CUDA(eikx::launchCellsToNatural2<double>(dst.as<double>(), d, nx, nz, ordering, c->stream));
        }
    }
    return finishModel(c, dim);
}

eikx_status eikx_set_slowness3d(eikx_ctx *c, const void *s, int dtype, int ordering, int where) {
    return setCells(c, 3, s, dtype, ordering, where, false);
}
eikx_status eikx_set_nodal_velocity3d(eikx_ctx *c, const void *v, int dtype, int ordering, int where) {
    return setCells(c, 3, v, dtype, ordering, where, true);
}
eikx_status eikx_set_slowness2d(eikx_ctx *c, const void *s, int dtype, int ordering, int where) {
    return setCells(c, 2, s, dtype, ordering, where, false);
}
eikx_status eikx_set_nodal_velocity2d(eikx_ctx *c, const void *v, int dtype, int ordering, int where) {
    return setCells(c, 2, v, dtype, ordering, where, true);
}

eikx_status eikx_get_slowness3d(const eikx_ctx *c, void *out, int dtype) {
    if (eikx_status r = checkCtx(c); r) return r;
    if (!c->haveSlow3) return fail(EIKX_ERR_STATE, "Velocity model not set");
    if (!out) return fail(EIKX_ERR_INVALID, "output is NULL");
    if (dtype != EIKX_F64 && dtype != EIKX_F32) return fail(EIKX_ERR_INVALID, "dtype must be EIKX_F32 or EIKX_F64");
    const std::vector<double> *hs = nullptr;
    if (eikx_status r = hostSlowness(c, 3, &hs); r) return r;
    if (dtype == EIKX_F64) {
        std::memcpy(out, hs->data(), hs->size() * sizeof(double));
    } else {
        float *o = static_cast<float *>(out);
        for (size_t i = 0; i < hs->size(); ++i) o[i] = static_cast<float>((*hs)[i]);
    }
    return EIKX_OK;
}

eikx_status eikx_solve3d(eikx_ctx *c, const eikx_source3d *src, int nSrc, const eikx_options *opt, int precision,
                         void *tOut, int where) {
    if (eikx_status r = checkCtx(c); r) return r;
    if (!c->haveGrid3) return fail(EIKX_ERR_STATE, "Class not initialized");
    if (!c->haveSlow3) return fail(EIKX_ERR_STATE, "Velocity model not set");
    if (!src || nSrc <= 0) return fail(EIKX_ERR_STATE, "Source location not set");
    if (!tOut) return fail(EIKX_ERR_INVALID, "output is NULL");
    if (where != EIKX_HOST && where != EIKX_DEVICE) return fail(EIKX_ERR_INVALID, "where must be EIKX_HOST or EIKX_DEVICE");
    eikx_options o;
    if (eikx_status r = fillOptions(opt, &o); r) return r;
    EIKX_CUDA(cudaSetDevice(c->device));
    std::vector<double> xyz(3 * static_cast<size_t>(nSrc));
    for (int i = 0; i < nSrc; ++i) { xyz[3 * i] = src[i].x; xyz[3 * i + 1] = src[i].y; xyz[3 * i + 2] = src[i].z; }
    if (precision == EIKX_F32) return solveImpl<float, 3>(c, xyz.data(), nSrc, o, tOut, where);
    if (precision == EIKX_F64) return solveImpl<double, 3>(c, xyz.data(), nSrc, o, tOut, where);
    return fail(EIKX_ERR_INVALID, "precision must be EIKX_F32 or EIKX_F64");
}

eikx_status eikx_solve3d_warm(eikx_ctx *c, const eikx_source3d *src, int nSrc, const eikx_options *opt, int precision,
                              const void *tInit, int initWhere, double gateTol, void *tOut, int where) {
    if (eikx_status r = checkCtx(c); r) return r;
    if (!c->haveGrid3) return fail(EIKX_ERR_STATE, "Class not initialized");
    if (!c->haveSlow3) return fail(EIKX_ERR_STATE, "Velocity model not set");
    if (!src || nSrc <= 0) return fail(EIKX_ERR_STATE, "Source location not set");
    if (!tOut || !tInit) return fail(EIKX_ERR_INVALID, "initial field or output is NULL");
    if (where != EIKX_HOST && where != EIKX_DEVICE) return fail(EIKX_ERR_INVALID, "where must be EIKX_HOST or EIKX_DEVICE");
    if (initWhere != EIKX_HOST && initWhere != EIKX_DEVICE)
        return fail(EIKX_ERR_INVALID, "init_where must be EIKX_HOST or EIKX_DEVICE");
    if (!(gateTol >= 0)) return fail(EIKX_ERR_INVALID, "gate_tol must be >= 0");
    eikx_options o;
    if (eikx_status r = fillOptions(opt, &o); r) return r;
    EIKX_CUDA(cudaSetDevice(c->device));
    std::vector<double> xyz(3 * static_cast<size_t>(nSrc));
    for (int i = 0; i < nSrc; ++i) { xyz[3 * i] = src[i].x; xyz[3 * i + 1] = src[i].y; xyz[3 * i + 2] = src[i].z; }
    if (precision == EIKX_F32) return solveImpl<float, 3>(c, xyz.data(), nSrc, o, tOut, where, tInit, initWhere, gateTol);
    if (precision == EIKX_F64) return solveImpl<double, 3>(c, xyz.data(), nSrc, o, tOut, where, tInit, initWhere, gateTol);
    return fail(EIKX_ERR_INVALID, "precision must be EIKX_F32 or EIKX_F64");
}

eikx_status eikx_solve3d_batch(eikx_ctx *c, const eikx_model3d *models, int nModels, const eikx_options *opt,
                               int precision) {
    if (eikx_status r = checkCtx(c); r) return r;
    if (!models || nModels <= 0) return fail(EIKX_ERR_INVALID, "batch has no models");
    if (precision != EIKX_F32 && precision != EIKX_F64)
        return fail(EIKX_ERR_INVALID, "precision must be EIKX_F32 or EIKX_F64");
    eikx_options o;
    if (eikx_status r = fillOptions(opt, &o); r) return r;
    for (int i = 0; i < nModels; ++i)
        if (std::string e = checkModel(models[i], i); !e.empty()) return fail(EIKX_ERR_INVALID, e);
    EIKX_CUDA(cudaSetDevice(c->device));
    // uniform-grid and non-uniform-grid models run different local solvers: one schedule each
    const double eps = (precision == EIKX_F32 ? std::numeric_limits<float>::epsilon()
                                              : std::numeric_limits<double>::epsilon()) * 100;
    std::vector<int> uni, non;
    for (int i = 0; i < nModels; ++i)
        (uniformSpacing3(models[i].dx, models[i].dy, models[i].dz, eps) ? uni : non).push_back(i);
    eikx_stats agg{};
    agg.iterations_min = 1 << 30;
    agg.sweep_ms = -1;
    for (int pass = 0; pass < 2; ++pass) {
        const std::vector<int> &sel = pass == 0 ? uni : non;
        if (sel.empty()) continue;
        eikx_status r = precision == EIKX_F32 ? solveBatch3<float>(c, models, sel, pass == 0, o, agg)
                                              : solveBatch3<double>(c, models, sel, pass == 0, o, agg);
        if (r != EIKX_OK) return r;
    }
    c->stats = agg;
    return EIKX_OK;
}

eikx_status eikx_autotune3d(eikx_ctx *c, const eikx_source3d *src, int nSrc, int precision, eikx_tuning *out) {
    if (eikx_status r = checkCtx(c); r) return r;
    if (!c->haveGrid3) return fail(EIKX_ERR_STATE, "Class not initialized");
    if (!c->haveSlow3) return fail(EIKX_ERR_STATE, "Velocity model not set");
    if (!src || nSrc <= 0) return fail(EIKX_ERR_STATE, "Source location not set");
    EIKX_CUDA(cudaSetDevice(c->device));
    std::vector<double> xyz(3 * static_cast<size_t>(nSrc));
    for (int i = 0; i < nSrc; ++i) { xyz[3 * i] = src[i].x; xyz[3 * i + 1] = src[i].y; xyz[3 * i + 2] = src[i].z; }
    if (precision == EIKX_F32) return autotune3<float>(c, xyz, nSrc, out);
    if (precision == EIKX_F64) return autotune3<double>(c, xyz, nSrc, out);
    return fail(EIKX_ERR_INVALID, "precision must be EIKX_F32 or EIKX_F64");
}

eikx_status eikx_tuning_save(const eikx_ctx *c, const char *path) {
    if (eikx_status r = checkCtx(c); r) return r;
    if (!path) return fail(EIKX_ERR_INVALID, "path is NULL");
    std::ofstream f(path);
    if (!f) return fail(EIKX_ERR_INVALID, std::string("cannot write ") + path);
    for (const auto &kv : c->tuning) {
        const TuneKey &k = kv.first;
        const eikx_tuning &t = kv.second;
        f << "{\"precision\": " << k.precision << ", \"uniform\": " << k.uniform << ", \"nx\": " << k.nx
          << ", \"ny\": " << k.ny << ", \"nz\": " << k.nz << ", \"nsrc\": " << k.nsrc
          << ", \"sweep_kernel\": " << t.sweep_kernel << ", \"pair_fields\": " << t.pair_fields
          << ", \"block_shape\": " << t.block_shape << ", \"blocks_per_sm\": " << t.blocks_per_sm
          << ", \"ms_per_sweep\": " << t.ms_per_sweep << ", \"default_ms_per_sweep\": " << t.default_ms_per_sweep
          << ", \"candidates\": " << t.candidates << "}\n";
    }
    return f ? EIKX_OK : fail(EIKX_ERR_INVALID, std::string("cannot write ") + path);
}

eikx_status eikx_tuning_load(eikx_ctx *c, const char *path) {
    if (eikx_status r = checkCtx(c); r) return r;
    if (!path) return fail(EIKX_ERR_INVALID, "path is NULL");
    std::ifstream f(path);
    if (!f) return fail(EIKX_ERR_INVALID, std::string("cannot read ") + path);
    std::string line;
    int lineNo = 0;
    std::map<TuneKey, eikx_tuning> add;
    while (std::getline(f, line)) {
        ++lineNo;
        if (line.find_first_not_of(" \t\r") == std::string::npos) continue;
        TuneKey k{};
        eikx_tuning t{};
        const int got = std::sscanf(line.c_str(),
                                    " {\"precision\": %d, \"uniform\": %d, \"nx\": %d, \"ny\": %d, \"nz\": %d, "
                                    "\"nsrc\": %d, \"sweep_kernel\": %d, \"pair_fields\": %d, \"block_shape\": %d, "
                                    "\"blocks_per_sm\": %d, \"ms_per_sweep\": %lf, \"default_ms_per_sweep\": %lf, "
                                    "\"candidates\": %d}",
                                    &k.precision, &k.uniform, &k.nx, &k.ny, &k.nz, &k.nsrc, &t.sweep_kernel,
                                    &t.pair_fields, &t.block_shape, &t.blocks_per_sm, &t.ms_per_sweep,
                                    &t.default_ms_per_sweep, &t.candidates);
        if (got != 13 || t.sweep_kernel < 1 || t.sweep_kernel > 2 || t.block_shape < 1 ||
            t.block_shape > eikx::kNumShapes || t.blocks_per_sm < 0)
            return fail(EIKX_ERR_INVALID, std::string(path) + ":" + std::to_string(lineNo) + ": not a tuning entry");
        add[k] = t;
    }
    for (const auto &kv : add) c->tuning[kv.first] = kv.second;
    return EIKX_OK;
}

static eikx_status checkLast(const eikx_ctx *c, int dim, int field) {
    if (eikx_status r = checkCtx(c); r) return r;
    if (!c->last.valid || c->last.dim != dim)
        return fail(EIKX_ERR_STATE, "Travel time field not yet computed");
    if (field < 0 || field >= c->last.nSrc) return fail(EIKX_ERR_INVALID, "field index out of range");
    return EIKX_OK;
}

static eikx_status gradientImpl(eikx_ctx *c, int dim, int field, void *grad, int where) {
    if (eikx_status r = checkLast(c, dim, field); r) return r;
    if (!grad) return fail(EIKX_ERR_INVALID, "gradient output is NULL");
    if (where != EIKX_HOST && where != EIKX_DEVICE) return fail(EIKX_ERR_INVALID, "where must be EIKX_HOST or EIKX_DEVICE");
    EIKX_CUDA(cudaSetDevice(c->device));
    const auto &L = c->last;
    const size_t nodes = static_cast<size_t>(L.nx) * L.ny * L.nz;
    const size_t elem = L.precision == EIKX_F32 ? 4 : 8;
    const size_t bytes = nodes * dim * elem;
    void *dst = grad;
    if (where == EIKX_HOST) {
        EIKX_CUDA(c->postBuf.ensure(bytes));
        dst = c->postBuf.p;
    }
    if (L.precision == EIKX_F32)
        EIKX_CUDA(eikx::launchGradient<float>(c->ws.tt.as<float>() + field * L.fieldStride, dim, L.Px, L.nx, L.ny, L.nz,
                                              L.dx, L.dy, L.dz, L.corners[field], static_cast<float *>(dst), c->stream));
    else
        EIKX_CUDA(eikx::launchGradient<double>(c->ws.tt.as<double>() + field * L.fieldStride, dim, L.Px, L.nx, L.ny,
                                               L.nz, L.dx, L.dy, L.dz, L.corners[field], static_cast<double *>(dst),
                                               c->stream));
    if (where == EIKX_HOST) EIKX_CUDA(cudaMemcpyAsync(grad, dst, bytes, cudaMemcpyDeviceToHost, c->stream));
    EIKX_CUDA(cudaStreamSynchronize(c->stream));
    return EIKX_OK;
}

static eikx_status stationsImpl(eikx_ctx *c, int dim, int field, const double *xyz, int n, double *times) {
    if (eikx_status r = checkLast(c, dim, field); r) return r;
    if (n < 0 || (n > 0 && (!xyz || !times))) return fail(EIKX_ERR_INVALID, "stations or output is NULL");
    if (n == 0) return EIKX_OK;
    EIKX_CUDA(cudaSetDevice(c->device));
    const auto &L = c->last;
    std::vector<int> cells(static_cast<size_t>(n) * dim);
    std::vector<double> offs(static_cast<size_t>(n) * dim);
    for (int i = 0; i < n; ++i) {
        int cx, cy = 0, cz;
        double ox, oy = 0, oz;
        const double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
        if (!locate(x, L.x0, L.dx, L.nx, &cx, &ox) || (dim == 3 && !locate(y, L.y0, L.dy, L.ny, &cy, &oy)) ||
            !locate(z, L.z0, L.dz, L.nz, &cz, &oz))
            return fail(EIKX_ERR_INVALID, "station " + std::to_string(i) + " lies outside the grid");
        if (dim == 3) {
            cells[3 * i] = cx; cells[3 * i + 1] = cy; cells[3 * i + 2] = cz;
            offs[3 * i] = ox; offs[3 * i + 1] = oy; offs[3 * i + 2] = oz;
        } else {
            cells[2 * i] = cx; cells[2 * i + 1] = cz;
            offs[2 * i] = ox; offs[2 * i + 1] = oz;
        }
    }
    const size_t cb = cells.size() * sizeof(int), ob = offs.size() * sizeof(double), tb = static_cast<size_t>(n) * 8;
    EIKX_CUDA(c->postBuf.ensure(cb + ob + tb + 32));
    char *base = static_cast<char *>(c->postBuf.p);
    int *dCells = reinterpret_cast<int *>(base);
    double *dOffs = reinterpret_cast<double *>(base + (cb + 15) / 16 * 16);
    double *dOut = dOffs + offs.size();
    EIKX_CUDA(cudaMemcpyAsync(dCells, cells.data(), cb, cudaMemcpyHostToDevice, c->stream));
    EIKX_CUDA(cudaMemcpyAsync(dOffs, offs.data(), ob, cudaMemcpyHostToDevice, c->stream));
    if (L.precision == EIKX_F32)
        EIKX_CUDA(eikx::launchStations<float>(c->ws.tt.as<float>() + field * L.fieldStride, dim, L.Px, L.ny, L.dx, L.dy,
                                              L.dz, L.corners[field], n, dCells, dOffs, dOut, c->stream));
    else
        EIKX_CUDA(eikx::launchStations<double>(c->ws.tt.as<double>() + field * L.fieldStride, dim, L.Px, L.ny, L.dx,
                                               L.dy, L.dz, L.corners[field], n, dCells, dOffs, dOut, c->stream));
    EIKX_CUDA(cudaMemcpyAsync(times, dOut, tb, cudaMemcpyDeviceToHost, c->stream));
    EIKX_CUDA(cudaStreamSynchronize(c->stream));
    return EIKX_OK;
}

eikx_status eikx_gradient3d(eikx_ctx *c, int field, void *grad, int where) { return gradientImpl(c, 3, field, grad, where); }
eikx_status eikx_gradient2d(eikx_ctx *c, int field, void *grad, int where) { return gradientImpl(c, 2, field, grad, where); }

eikx_status eikx_station_times3d(eikx_ctx *c, int field, const eikx_source3d *st, int n, double *times) {
    std::vector<double> xyz(3 * static_cast<size_t>(std::max(n, 0)));
    for (int i = 0; i < n && st; ++i) { xyz[3 * i] = st[i].x; xyz[3 * i + 1] = st[i].y; xyz[3 * i + 2] = st[i].z; }
    return stationsImpl(c, 3, field, st ? xyz.data() : nullptr, n, times);
}
eikx_status eikx_station_times2d(eikx_ctx *c, int field, const eikx_source2d *st, int n, double *times) {
    std::vector<double> xyz(3 * static_cast<size_t>(std::max(n, 0)));
    for (int i = 0; i < n && st; ++i) { xyz[3 * i] = st[i].x; xyz[3 * i + 1] = 0; xyz[3 * i + 2] = st[i].z; }
    return stationsImpl(c, 2, field, st ? xyz.data() : nullptr, n, times);
}

eikx_status eikx_selftest_operator3d(int device, int precision, long long n, unsigned long long seed,
                                     long long counts[4]) {
    if (!counts || n < 0) return fail(EIKX_ERR_INVALID, "counts must not be NULL and n must be >= 0");
    if (precision != EIKX_F32 && precision != EIKX_F64) return fail(EIKX_ERR_INVALID, "precision must be F32 or F64");
    EIKX_CUDA(cudaSetDevice(device));
    unsigned long long *d = nullptr;
    EIKX_CUDA(cudaMalloc(&d, 4 * sizeof(unsigned long long)));
    unsigned long long h[4] = {0, 0, 0, 0};
    cudaError_t e = cudaMemset(d, 0, sizeof(h));
    if (e == cudaSuccess) e = eikx::launchOperatorSelftest(precision == EIKX_F32 ? 0 : 1, n, seed, d, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    EIKX_CUDA(e);
    for (int k = 0; k < 4; ++k) counts[k] = static_cast<long long>(h[k]);
    return EIKX_OK;
}

void eikx_ray_options_default(eikx_ray_options *opt) {
    if (!opt) return;
    std::memset(opt, 0, sizeof(*opt));
    // GradientTracerOptions defaults, src/ray/gradientTracerOptions.cpp
    const int r[5] = {1, 2, 3, 5, std::numeric_limits<int>::max()};
    const double s[5] = {0.05, 0.10, 0.20, 0.30, 0.45};
    opt->n_radii = 5;
    for (int k = 0; k < 5; ++k) { opt->radius[k] = r[k]; opt->scale[k] = s[k]; }
    opt->max_steps = 0;
}

eikx_status eikx_trace_rays2d(eikx_ctx *c, int nx, int nz, double dx, double dz, double x0, double z0,
                              const void *gradient, int dtype, const double *slowness, double sourceX,
                              double sourceZ, const double *stations, int n, const eikx_ray_options *opt,
                              int capacity, eikx_ray_segment2d *segments, int *counts) {
    if (eikx_status r = checkCtx(c); r) return r;
    if (nx < 3 || nz < 3) return fail(EIKX_ERR_INVALID, "grid needs at least 3 points in each direction");
    if (!(dx > 0) || !(dz > 0)) return fail(EIKX_ERR_INVALID, "grid spacing must be positive");
    if (!gradient || !slowness) return fail(EIKX_ERR_INVALID, "Travel time gradient field not set");
    if (dtype != EIKX_F32 && dtype != EIKX_F64) return fail(EIKX_ERR_INVALID, "dtype must be EIKX_F32 or EIKX_F64");
    if (n <= 0 || !stations) return fail(EIKX_ERR_STATE, "No stations were set");
    if (capacity < 1 || !segments || !counts) return fail(EIKX_ERR_INVALID, "segment output is NULL or empty");
    eikx_ray_options o;
    if (opt) o = *opt; else eikx_ray_options_default(&o);
    // GradientTracerOptions::setRadiusScaleFactor (src/ray/gradientTracerOptions.cpp): radii
    // non-negative and distinct, scales in (eps, 1), sorted by radius, extended to INT_MAX
    if (o.n_radii < 1 || o.n_radii > 16) return fail(EIKX_ERR_INVALID, "Input vector cannot be empty");
    std::vector<std::pair<int, double>> rsf;
    for (int k = 0; k < o.n_radii; ++k) {
        if (o.radius[k] < 0) return fail(EIKX_ERR_INVALID, "All radii must be non-negative");
        if (o.scale[k] <= std::numeric_limits<double>::epsilon())
            return fail(EIKX_ERR_INVALID, "All scale factors must be non-negative");
        if (o.scale[k] >= 1) return fail(EIKX_ERR_INVALID, "All scale factors must be less than 1");
        rsf.emplace_back(o.radius[k], o.scale[k]);
    }
    std::stable_sort(rsf.begin(), rsf.end(), [](const auto &a, const auto &b) { return a.first < b.first; });
    for (size_t k = 0; k + 1 < rsf.size(); ++k)
        if (rsf[k].first == rsf[k + 1].first) return fail(EIKX_ERR_INVALID, "Duplicate radii");
    if (rsf.back().first < std::numeric_limits<int>::max()) {
        if (rsf.size() == eikx::kMaxRadii) return fail(EIKX_ERR_INVALID, "at most 15 radii below INT_MAX");
        rsf.emplace_back(std::numeric_limits<int>::max(), rsf.back().second);
    }
    eikx::RayTrace2Args a{};
    a.nx = nx; a.nz = nz; a.dx = dx; a.dz = dz; a.x0 = x0; a.z0 = z0;
    if (!locate(sourceX, x0, dx, nx, &a.isx, &a.xs) || !locate(sourceZ, z0, dz, nz, &a.isz, &a.zs))
        return fail(EIKX_ERR_INVALID, "source position outside the grid");
    for (int i = 0; i < n; ++i) {
        int cx, cz;
        double ox, oz;
        if (!locate(stations[2 * i], x0, dx, nx, &cx, &ox) || !locate(stations[2 * i + 1], z0, dz, nz, &cz, &oz))
            return fail(EIKX_ERR_INVALID, "station " + std::to_string(i) + " outside the grid");
    }
    a.nRsf = static_cast<int>(rsf.size());
    double minScale = 1;
    for (int k = 0; k < a.nRsf; ++k) {
        a.rsfRadius[k] = rsf[k].first;
        a.rsfScale[k] = rsf[k].second;
        minScale = std::min(minScale, rsf[k].second);
    }
    a.maxSteps = o.max_steps > 0 ? o.max_steps
                                 : static_cast<int>(std::min(1.e8, std::ceil(4.0 * (nx + nz) / minScale)) + 16);
    a.capacity = capacity;
    const size_t nNode = static_cast<size_t>(nx) * nz, nCell = static_cast<size_t>(nx - 1) * (nz - 1);
    const size_t gradBytes = 2 * nNode * (dtype == EIKX_F64 ? 8 : 4);
    const size_t posBytes = static_cast<size_t>(n) * (a.maxSteps + 1) * 2 * sizeof(double);
    const size_t segBytes = static_cast<size_t>(n) * capacity * 6 * sizeof(double);
    EIKX_CUDA(cudaSetDevice(c->device));
    EIKX_CUDA(c->rayGrad.ensure(gradBytes));
    EIKX_CUDA(c->raySlow.ensure(nCell * sizeof(double)));
    EIKX_CUDA(c->raySt.ensure(2 * static_cast<size_t>(n) * sizeof(double)));
    EIKX_CUDA(c->rayPos.ensure(posBytes));
    EIKX_CUDA(c->raySeg.ensure(segBytes));
    EIKX_CUDA(c->rayCnt.ensure(static_cast<size_t>(n) * sizeof(int)));
    EIKX_CUDA(cudaMemcpyAsync(c->rayGrad.p, gradient, gradBytes, cudaMemcpyHostToDevice, c->stream));
    EIKX_CUDA(cudaMemcpyAsync(c->raySlow.p, slowness, nCell * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    EIKX_CUDA(cudaMemcpyAsync(c->raySt.p, stations, 2 * static_cast<size_t>(n) * sizeof(double),
                              cudaMemcpyHostToDevice, c->stream));
    a.slow = c->raySlow.as<double>();
    if (dtype == EIKX_F64)
        EIKX_CUDA(eikx::launchTraceRays2<double>(a, c->rayGrad.as<double>(), n, c->raySt.as<double>(),
                                                 c->rayPos.as<double>(), c->raySeg.as<double>(), c->rayCnt.as<int>(),
                                                 c->stream));
    else
        EIKX_CUDA(eikx::launchTraceRays2<float>(a, c->rayGrad.as<float>(), n, c->raySt.as<double>(),
                                                c->rayPos.as<double>(), c->raySeg.as<double>(), c->rayCnt.as<int>(),
                                                c->stream));
    std::vector<double> seg(static_cast<size_t>(n) * capacity * 6);
    EIKX_CUDA(cudaMemcpyAsync(counts, c->rayCnt.p, static_cast<size_t>(n) * sizeof(int), cudaMemcpyDeviceToHost,
                              c->stream));
    EIKX_CUDA(cudaMemcpyAsync(seg.data(), c->raySeg.p, segBytes, cudaMemcpyDeviceToHost, c->stream));
    EIKX_CUDA(cudaStreamSynchronize(c->stream));
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < std::max(0, counts[i]); ++k) {
            const double *s = &seg[(static_cast<size_t>(i) * capacity + k) * 6];
            eikx_ray_segment2d &d = segments[static_cast<size_t>(i) * capacity + k];
            d.x0 = s[0]; d.z0 = s[1]; d.x1 = s[2]; d.z1 = s[3]; d.slowness = s[4];
            d.cell = static_cast<int>(s[5]);
            d.reserved = 0;
        }
    return EIKX_OK;
}

eikx_status eikx_solve2d(eikx_ctx *c, const eikx_source2d *src, int nSrc, const eikx_options *opt, int precision,
                         void *tOut, int where) {
    if (eikx_status r = checkCtx(c); r) return r;
    if (!c->haveGrid2) return fail(EIKX_ERR_STATE, "Class not initialized");
    if (!c->haveSlow2) return fail(EIKX_ERR_STATE, "Velocity model not set");
    if (!src || nSrc <= 0) return fail(EIKX_ERR_STATE, "Source location not set");
    if (!tOut) return fail(EIKX_ERR_INVALID, "output is NULL");
    if (where != EIKX_HOST && where != EIKX_DEVICE) return fail(EIKX_ERR_INVALID, "where must be EIKX_HOST or EIKX_DEVICE");
    eikx_options o;
    if (eikx_status r = fillOptions(opt, &o); r) return r;
    EIKX_CUDA(cudaSetDevice(c->device));
    std::vector<double> xyz(3 * static_cast<size_t>(nSrc));
    for (int i = 0; i < nSrc; ++i) { xyz[3 * i] = src[i].x; xyz[3 * i + 1] = 0; xyz[3 * i + 2] = src[i].z; }
    if (precision == EIKX_F32) return solveImpl<float, 2>(c, xyz.data(), nSrc, o, tOut, where);
    if (precision == EIKX_F64) return solveImpl<double, 2>(c, xyz.data(), nSrc, o, tOut, where);
    return fail(EIKX_ERR_INVALID, "precision must be EIKX_F32 or EIKX_F64");
}

eikx_status eikx_analytic3d(eikx_ctx *c, const eikx_source3d *src, double vTop, double vBottom, double *tOut,
                            int where) {
    if (eikx_status r = checkCtx(c); r) return r;
    if (!c->haveGrid3) return fail(EIKX_ERR_STATE, "Class not initialized");
    if (!src || !tOut) return fail(EIKX_ERR_INVALID, "source or output is NULL");
    if (!(vTop > 0) || !(vBottom > 0)) return fail(EIKX_ERR_INVALID, "velocities must be positive");
    int cx, cy, cz;
    double ox, oy, oz;
    if (!locate(src->x, c->x0, c->dx, c->nx, &cx, &ox) || !locate(src->y, c->y0, c->dy, c->ny, &cy, &oy) ||
        !locate(src->z, c->z0, c->dz, c->nz, &cz, &oz))
        return fail(EIKX_ERR_INVALID, "source position outside the grid");
    EIKX_CUDA(cudaSetDevice(c->device));
    const size_t n = static_cast<size_t>(c->nx) * c->ny * c->nz;
    double *dst = tOut;
    if (where != EIKX_DEVICE) {
        EIKX_CUDA(c->scratch.ensure(n * sizeof(double)));
        dst = c->scratch.as<double>();
    }
    EIKX_CUDA(eikx::launchAnalytic3(dst, c->nx, c->ny, c->nz, c->dx, c->dy, c->dz, ox, oy, oz, vTop, vBottom, c->stream));
    if (where != EIKX_DEVICE)
        EIKX_CUDA(cudaMemcpyAsync(tOut, dst, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    EIKX_CUDA(cudaStreamSynchronize(c->stream));
    return EIKX_OK;
}

eikx_status eikx_analytic2d(eikx_ctx *c, const eikx_source2d *src, double vTop, double vBottom, double *tOut,
                            int where) {
    if (eikx_status r = checkCtx(c); r) return r;
    if (!c->haveGrid2) return fail(EIKX_ERR_STATE, "Class not initialized");
    if (!src || !tOut) return fail(EIKX_ERR_INVALID, "source or output is NULL");
    if (!(vTop > 0) || !(vBottom > 0)) return fail(EIKX_ERR_INVALID, "velocities must be positive");
    int cx, cz;
    double ox, oz;
    if (!locate(src->x, c->x02, c->dx2, c->nx2, &cx, &ox) || !locate(src->z, c->z02, c->dz2, c->nz2, &cz, &oz))
        return fail(EIKX_ERR_INVALID, "source position outside the grid");
    EIKX_CUDA(cudaSetDevice(c->device));
    const size_t n = static_cast<size_t>(c->nx2) * c->nz2;
    double *dst = tOut;
    if (where != EIKX_DEVICE) {
        EIKX_CUDA(c->scratch.ensure(n * sizeof(double)));
        dst = c->scratch.as<double>();
    }
    EIKX_CUDA(eikx::launchAnalytic2(dst, c->nx2, c->nz2, c->dx2, c->dz2, ox, oz, vTop, vBottom, c->stream));
    if (where != EIKX_DEVICE)
        EIKX_CUDA(cudaMemcpyAsync(tOut, dst, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    EIKX_CUDA(cudaStreamSynchronize(c->stream));
    return EIKX_OK;
}

}  // extern "C"

// Lets other translation units of the library report through eikx_last_error().
eikx_status eikxSetLastError(eikx_status code, const char *msg) { return fail(code, msg); }
