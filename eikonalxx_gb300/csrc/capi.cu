// Host runtime behind the C ABI (include/eikx/eikx_c.h).
//
// A context holds the model (cell slowness, FP64 master copy on the device plus an
// edge-replicated copy in each sweep precision), the solve workspace and the CUDA
// graph of the last sweep schedule.  A solve is: upload the per-field source table,
// replay (or capture, then replay) the schedule graph -- reset, corner
// initialisation, the source-limited pass, nSweeps refinement iterations each
// followed by the convergence check -- and copy the fields out with one pitched copy.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
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

struct Workspace {
    DevBuf tt, mbox, epoch, queue, residual, converged, iterations, abortFlag, order, srcs, corners, pairs;
    PinnedBuf stage;
    std::vector<int> orderKey;   // (tilesY, tilesZ, nFields, dim) of the uploaded order table
};

struct ScheduleKey {
    int dim = 0, precision = -1, nFields = 0, nx = 0, ny = 0, nz = 0, nSweeps = -1, radius = 0,
        initSweeps = 0, initFp64 = 0, uniform = 0, blocks = 0, dropBlocks = 0, paired = 0, variant = 0;
    double tol = 0, h = 0, dx = 0, dy = 0, dz = 0;
    unsigned long long spin = 0;
    const void *tt = nullptr, *sp = nullptr, *srcs = nullptr, *corners = nullptr;
    bool operator==(const ScheduleKey &o) const { return std::memcmp(this, &o, sizeof(*this)) == 0; }
};

}  // namespace

struct eikx_ctx {
    int device = 0;
    int numSMs = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<cudaEvent_t> sweepEv;   // per-sweep timing (profile_sweeps)
    // 3D model
    int nx = 0, ny = 0, nz = 0;
    double dx = 0, dy = 0, dz = 0, x0 = 0, y0 = 0, z0 = 0;
    bool haveGrid3 = false, haveSlow3 = false;
    DevBuf slow3;                  // natural-order cell slowness, FP64
    std::vector<double> hostSlow3; // host mirror (source-cell slowness lookups)
    DevBuf spad3[2][2];            // [precision][0: shifted for +x sweeps, 1: unshifted]
    bool spadValid3[2] = {false, false};
    // 2D model
    int nx2 = 0, nz2 = 0;
    double dx2 = 0, dz2 = 0, x02 = 0, z02 = 0;
    bool haveGrid2 = false, haveSlow2 = false;
    DevBuf slow2;
    std::vector<double> hostSlow2;
    DevBuf spad2[2][2];
    bool spadValid2[2] = {false, false};
    DevBuf scratch;                // staging for host inputs and analytic fields
    Workspace ws;
    eikx_stats stats{};
    // cached schedule graph
    ScheduleKey graphKey;
    cudaGraphExec_t graphExec = nullptr;
    int graphLaunches = 0;
    bool useGraphs = true;
};

namespace {

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

eikx_status finishModel3(eikx_ctx *c) {
    const size_t nCell = static_cast<size_t>(c->nx - 1) * (c->ny - 1) * (c->nz - 1);
    c->hostSlow3.resize(nCell);
    EIKX_CUDA(cudaMemcpyAsync(c->hostSlow3.data(), c->slow3.p, nCell * sizeof(double), cudaMemcpyDeviceToHost,
                              c->stream));
    EIKX_CUDA(cudaStreamSynchronize(c->stream));
    for (double s : c->hostSlow3)
        if (!(s > 0) || !std::isfinite(s))
            return fail(EIKX_ERR_INVALID, "Non-positive velocities detected");
    c->spadValid3[0] = c->spadValid3[1] = false;
    c->haveSlow3 = true;
    dropGraph(c);
    return EIKX_OK;
}

eikx_status finishModel2(eikx_ctx *c) {
    const size_t nCell = static_cast<size_t>(c->nx2 - 1) * (c->nz2 - 1);
    c->hostSlow2.resize(nCell);
    EIKX_CUDA(cudaMemcpyAsync(c->hostSlow2.data(), c->slow2.p, nCell * sizeof(double), cudaMemcpyDeviceToHost,
                              c->stream));
    EIKX_CUDA(cudaStreamSynchronize(c->stream));
    for (double s : c->hostSlow2)
        if (!(s > 0) || !std::isfinite(s))
            return fail(EIKX_ERR_INVALID, "Non-positive velocities detected");
    c->spadValid2[0] = c->spadValid2[1] = false;
    c->haveSlow2 = true;
    dropGraph(c);
    return EIKX_OK;
}

template <class T> int precOf();
template <> int precOf<float>() { return EIKX_F32; }
template <> int precOf<double>() { return EIKX_F64; }

// Shared solve driver for 2D and 3D.
template <class T, int DIM>
eikx_status solveImpl(eikx_ctx *c, const double *srcXYZ, int nSrc, const eikx_options &o, void *tOut,
                      int where) {
    const int P = precOf<T>();
    const int nx = DIM == 3 ? c->nx : c->nx2;
    const int ny = DIM == 3 ? c->ny : 1;
    const int nz = DIM == 3 ? c->nz : c->nz2;
    const double dx = DIM == 3 ? c->dx : c->dx2, dy = DIM == 3 ? c->dy : 1.0, dz = DIM == 3 ? c->dz : c->dz2;
    const double x0 = DIM == 3 ? c->x0 : c->x02, y0 = DIM == 3 ? c->y0 : 0.0, z0 = DIM == 3 ? c->z0 : c->z02;
    const int Px = roundUp(nx, 4);
    const int spPitch = Px + 8;
    const long long fieldStride = static_cast<long long>(Px) * ny * nz;
    const std::vector<double> &hs = DIM == 3 ? c->hostSlow3 : c->hostSlow2;

    // sources: cell, offsets, source-cell slowness (reference Source3D / Solver3D::solve)
    std::vector<eikx::SourceT<T>> srcT(nSrc);
    std::vector<eikx::Corner3> corners(nSrc);
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
        const size_t cell = DIM == 3 ? (static_cast<size_t>(cz) * (ny - 1) + cy) * (nx - 1) + cx
                                     : static_cast<size_t>(cz) * (nx - 1) + cx;
        const double s = hs[cell];
        srcT[i].isx = cx; srcT[i].isy = cy; srcT[i].isz = cz;
        srcT[i].xs = static_cast<T>(ox); srcT[i].ys = static_cast<T>(oy); srcT[i].zs = static_cast<T>(oz);
        srcT[i].sSrc = static_cast<T>(s);
        // corner init: slowness as the field type holds it, offsets in FP64
        corners[i] = eikx::Corner3{cx, cy, cz, ox, oy, oz, static_cast<double>(static_cast<T>(s))};
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

    // geometry in the sweep type (include/private/solver3d.hpp:31-44, solver2d.hpp:29-46)
    const double eps = std::numeric_limits<T>::epsilon() * 100;
    const bool uniform = DIM == 3 ? (std::abs(dx - dy) < eps && std::abs(dx - dz) < eps) : (std::abs(dx - dz) < eps);
    // FP32 uniform 3D batches run two fields per lane (the paired kernel)
    const bool paired = DIM == 3 && P == EIKX_F32 && uniform && nSrc >= 2 && o.pair_fields;
    const int nUnits = paired ? (nSrc + 1) / 2 : nSrc;   // work units: fields or field pairs

    // workspace
    const int ly = DIM == 3 ? eikx::LY3 : 1, lz = DIM == 3 ? eikx::LZ3 : eikx::LZ2;
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
                            w.iterations.p, w.order.p, w.srcs.p, w.corners.p};
    EIKX_CUDA(w.tt.ensure(ttBytes));
    if (w.mbox.bytes < mboxBytes || !w.mbox.p) {
        // fresh words carry tag 0, which no sweep uses
        EIKX_CUDA(w.mbox.ensure(mboxBytes));
        EIKX_CUDA(cudaMemsetAsync(w.mbox.p, 0, w.mbox.bytes, c->stream));
    }
    if (!w.epoch.p) {
        EIKX_CUDA(w.epoch.ensure(sizeof(unsigned)));
        EIKX_CUDA(cudaMemsetAsync(w.epoch.p, 0, sizeof(unsigned), c->stream));
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
    const void *after[] = {w.tt.p, w.mbox.p, w.epoch.p, w.residual.p, w.converged.p,
                           w.iterations.p, w.order.p, w.srcs.p, w.corners.p};
    if (std::memcmp(before, after, sizeof(before)) != 0) dropGraph(c);

    // small uploads through pinned staging
    std::vector<int> key = {tilesY, tilesZ, nUnits, DIM};
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
    EIKX_CUDA(cudaStreamSynchronize(c->stream));  // staging buffer reuse
    EIKX_CUDA(w.stage.ensure(srcBytes + cornerBytes + orderBytes + pairBytes + 64));
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
    st.iterations = w.iterations.as<int>();
    st.abortFlag = w.abortFlag.as<int>();
    // test hook: leave the first blocks of the queue out (their dependants time out)
    const int drop = std::min(std::max(o.test_drop_blocks, 0), nProgress);
    st.order = w.order.as<int4>() + drop;
    st.totalItems = nProgress - drop;
    const int spinLog2 = o.spin_limit_log2 > 0 ? std::min(o.spin_limit_log2, 40) : 22;
    st.spinLimit = 1ull << spinLog2;

    const int variant = o.sweep_kernel == eikx::kNodeStep ? eikx::kNodeStep : eikx::kChunkStep;
    const int perSM = paired ? eikx::sweep3PairBlocksPerSM()
                      : DIM == 2 ? eikx::sweep2BlocksPerSM<T>(uniform)
                      : variant == eikx::kChunkStep ? eikx::sweep3ChunkBlocksPerSM<T>(uniform)
                                                    : eikx::sweep3BlocksPerSM<T>(uniform);
    int blocks = std::min(c->numSMs * perSM, (nProgress + eikx::kWarpsPerBlock - 1) / eikx::kWarpsPerBlock);
    blocks = std::max(blocks, 1);

    ScheduleKey sk;
    sk.dim = DIM; sk.precision = P; sk.nFields = nSrc; sk.nx = nx; sk.ny = ny; sk.nz = nz;
    sk.nSweeps = nSweeps; sk.radius = o.factored_radius; sk.initSweeps = o.init_sweeps ? 1 : 0;
    sk.initFp64 = o.init_fp64 ? 1 : 0; sk.uniform = uniform; sk.blocks = blocks; sk.tol = o.tolerance;
    sk.h = dx; sk.dx = dx; sk.dy = dy; sk.dz = dz; sk.spin = st.spinLimit; sk.dropBlocks = drop;
    sk.paired = paired ? 1 : 0;
    sk.variant = variant;
    sk.tt = w.tt.p; sk.sp = spad[0].p; sk.srcs = w.srcs.p; sk.corners = w.corners.p;

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
        if (DIM == 3)
            EIKX_CUDA(eikx::launchInit3<T>(w.tt.as<T>(), nSrc, fieldStride, Px, nx, ny, nz, dx, dy, dz,
                                           w.corners.as<eikx::Corner3>(), o.init_fp64 ? 1 : 0, c->stream));
        else
            EIKX_CUDA(eikx::launchInit2<T>(w.tt.as<T>(), nSrc, fieldStride, Px, nx, nz, dx, dz,
                                           w.corners.as<eikx::Corner3>(), o.init_fp64 ? 1 : 0, c->stream));
        ++launches;
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
                    if (variant == eikx::kChunkStep) EIKX_CUDA(eikx::launchSweep3Chunk<T>(a, uniform, blocks, c->stream));
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
                EIKX_CUDA(eikx::launchSweep2<T>(a, uniform, blocks, c->stream));
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
            for (int e = 0; e < nSweepKinds; ++e)
                if (eikx_status r = sweep(e, 0, nSweepKinds * (1 + k) + e); r != EIKX_OK) return r;
            EIKX_CUDA(eikx::launchCheckConvergence(st, nSrc, nSweepKinds * (1 + k), nSweepKinds, k, o.tolerance,
                                                   c->stream));
            ++launches;
        }
        return EIKX_OK;
    };

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
    // one pitched copy for all fields: rows of nx values out of rows of Px
    const cudaMemcpyKind kind = where == EIKX_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    EIKX_CUDA(cudaMemcpy2DAsync(tOut, static_cast<size_t>(nx) * sizeof(T), w.tt.p, static_cast<size_t>(Px) * sizeof(T),
                                static_cast<size_t>(nx) * sizeof(T), static_cast<size_t>(ny) * nz * nSrc, kind,
                                c->stream));
    EIKX_CUDA(cudaEventRecord(c->ev1, c->stream));
    std::vector<int> iters(nSrc);
    int aborted = 0;
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
    for (int i = 0; i < nSrc; ++i) {
        s.iterations_max = std::max(s.iterations_max, iters[i]);
        s.iterations_min = std::min(s.iterations_min, iters[i]);
        if (iters[i] > 0) {
            for (int e = 0; e < nSweepKinds; ++e) {
                unsigned long long bits = lastRes[static_cast<size_t>(i) * resStride + nSweepKinds * iters[i] + e];
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
    c->stats = s;
    if (aborted) return fail(EIKX_ERR_TIMEOUT, "a bounded inter-tile wait ran out; the fields are not valid");
    return EIKX_OK;
}

eikx_status fillOptions(const eikx_options *in, eikx_options *out) {
    if (in) *out = *in; else eikx_options_default(out);
    if (out->n_sweeps < 0) return fail(EIKX_ERR_INVALID, "n_sweeps must be non-negative");
    if (out->factored_radius < 0) out->factored_radius = 0;
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
    for (cudaEvent_t e : c->sweepEv) cudaEventDestroy(e);
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
    // Model3D/Model2D reject non-positive velocities (src/model3d.cpp:301-305); host
    // inputs are checked before upload, device inputs through the resulting slowness.
    if (where == EIKX_HOST) {
        bool bad = false;
        if (dtype == EIKX_F32) {
            const float *p = static_cast<const float *>(v);
            for (size_t i = 0; i < nIn && !bad; ++i) bad = !(p[i] > 0);
        } else {
            const double *p = static_cast<const double *>(v);
            for (size_t i = 0; i < nIn && !bad; ++i) bad = !(p[i] > 0);
        }
        if (bad) return fail(EIKX_ERR_INVALID, nodal ? "Non-positive velocities detected"
                                                     : "Non-positive slowness detected");
    }
    const size_t nCell = static_cast<size_t>(nx - 1) * (ny - 1) * (nz - 1);
    DevBuf &dst = dim == 3 ? c->slow3 : c->slow2;
    EIKX_CUDA(dst.ensure(nCell * sizeof(double)));
    if (dtype == EIKX_F32) {
        const float *d = nullptr;
        if (eikx_status r = toDevice<float>(c, static_cast<const float *>(v), nIn, where, &d); r) return r;
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
        if (nodal) {
            if (dim == 3) EIKX_CUDA(eikx::launchNodalToCell3<double>(dst.as<double>(), d, nx, ny, nz, ordering, c->stream));
            else EIKX_CUDA(eikx::launchNodalToCell2<double>(dst.as<double>(), d, nx, nz, ordering, c->stream));
        } else {
            if (dim == 3) EIKX_CUDA(eikx::launchCellsToNatural3<double>(dst.as<double>(), d, nx, ny, nz, ordering, c->stream));
            else EIKX_CUDA(eikx::launchCellsToNatural2<double>(dst.as<double>(), d, nx, nz, ordering, c->stream));
        }
    }
    return dim == 3 ? finishModel3(c) : finishModel2(c);
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
    if (dtype == EIKX_F64) {
        std::memcpy(out, c->hostSlow3.data(), c->hostSlow3.size() * sizeof(double));
    } else if (dtype == EIKX_F32) {
        float *o = static_cast<float *>(out);
        for (size_t i = 0; i < c->hostSlow3.size(); ++i) o[i] = static_cast<float>(c->hostSlow3[i]);
    } else {
        return fail(EIKX_ERR_INVALID, "dtype must be EIKX_F32 or EIKX_F64");
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
