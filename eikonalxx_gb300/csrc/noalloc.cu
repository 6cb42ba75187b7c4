// eikx_solve3d_noalloc: a 3D FP32 solve that allocates nothing.
//
// Who needs it: callers that must not allocate GPU memory while they run -- code that
// runs between the steps of a host framework which owns every device allocation (a
// memory pool that would be bypassed and fragmented by cudaMalloc), real-time or
// embedded pipelines that forbid allocation after start-up, and hosts that call the
// solver from a context where cudaMalloc/cudaFree would synchronise the device or
// fail outright.  The regular entry points (eikx_solve3d) keep per-context buffers
// that they grow with cudaMalloc; this one keeps every intermediate buffer of the
// solve in one fixed array compiled into the library.
//
// The scratch: a file-scope `static __device__` array of kScratchBytes (64 MiB).  It
// belongs to this translation unit's module.  Under CUDA's default lazy module loading
// the driver loads that module -- and reserves the array and loads the sweep kernels --
// on a device the first time this entry point runs there, so that first call is not
// free of allocation; with CUDA_MODULE_LOADING=EAGER it happens when the library is
// loaded.  From then on the device holds the array until the process exits.  A caller
// that cannot allocate at all makes one warm-up call per device at start-up, before
// its own pool takes the memory and before any stream capture; every later call makes
// no allocating call.  A grid needs about 15 bytes per node of the array (padded
// travel times 4 B, two edge-replicated slowness copies 8 B, block-face mailbox 3 B,
// plus a few kB); grids whose need exceeds it are rejected with EIKX_ERR_INVALID before
// anything runs -- about 4 million nodes (e.g. 160^3).
//
// Sharing: all calls on a device share the array and it keeps the previous call's
// contents.  Whatever a solve requires to start at zero (queue heads, residual slots,
// convergence flags, the abort flag, the model check) is cleared by the solve itself;
// mailbox words carry a tag that only the current solve uses.  Two calls whose work
// overlaps on the GPU (different streams, or different host threads) race on the array
// and corrupt each other's fields: serialise them.
//
// Set-up: the first call on a device, with that device current, looks up the device
// address of the array (cudaGetSymbolAddress; in host code the array's name is only a
// host-side stand-in) and clears the array once.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "eikx/eikx_c.h"
#include "sweep.h"

eikx_status eikxSetLastError(eikx_status code, const char *msg);

namespace {

constexpr size_t kScratchBytes = 64ull << 20;
// FP64 analytic-factor table of a near_fp64 solve: 2.6 MB of the array, factored radius 7
constexpr int kFactorEntries = 32768;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char gScratch[kScratchBytes];

std::mutex gSetupMutex;
void *gScratchAddr[kMaxDevices] = {};

eikx_status err(eikx_status code, const std::string &msg) { return eikxSetLastError(code, msg.c_str()); }

#define NOALLOC_CUDA(expr)                                                                        \
    do {                                                                                          \
        cudaError_t e_ = (expr);                                                                  \
        if (e_ != cudaSuccess) return err(EIKX_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Device address of the scratch array on the current device; the first call per device
// resolves it and clears the array.
eikx_status scratchAddress(int device, cudaStream_t stream, unsigned char **out) {
    std::lock_guard<std::mutex> lock(gSetupMutex);
    if (device < 0 || device >= kMaxDevices) return err(EIKX_ERR_UNSUPPORTED, "device index above 63");
    if (!gScratchAddr[device]) {
        void *p = nullptr;
        NOALLOC_CUDA(cudaGetSymbolAddress(&p, gScratch));
        NOALLOC_CUDA(cudaMemsetAsync(p, 0, kScratchBytes, stream));
        gScratchAddr[device] = p;
    }
    *out = static_cast<unsigned char *>(gScratchAddr[device]);
    return EIKX_OK;
}

// Bump allocator over the scratch array (256-byte aligned regions).
struct Carve {
    unsigned char *base;
    size_t used = 0;
    template <class X> X *take(size_t count) {
        used = (used + 255) & ~static_cast<size_t>(255);
        X *p = reinterpret_cast<X *>(base ? base + used : nullptr);
        used += count * sizeof(X);
        return p;
    }
};

// Work order of one field's warp blocks of ly x lz pencils, sorted by start step
// (by*ly + bz*lz, then by): each thread ranks its block by counting the blocks that come
// before it.
__global__ void orderKernel(int4 *order, int tilesY, int tilesZ, int ly, int lz) {
    const int n = tilesY * tilesZ;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int b = t % tilesY, c = t / tilesY;
        const int key = b * ly + c * lz;
        int rank = 0;
        for (int u = 0; u < n; ++u) {
            const int b2 = u % tilesY, c2 = u / tilesY;
            const int k2 = b2 * ly + c2 * lz;
            rank += (k2 < key || (k2 == key && b2 < b)) ? 1 : 0;
        }
        order[rank] = make_int4(0, b, c, 0);
    }
}

// Source table of the field: the source-cell slowness is read from the caller's model;
// src64 (the FP64 analytic factor, eikx_options.near_fp64) is copied when not null.
__global__ void sourceKernel(eikx::SourceT<float> *src, eikx::Corner3 *corner, eikx::SourceFp64 *src64,
                             eikx::SourceFp64 f64, const float *slowness, int ncx, int ncy, int cx, int cy, int cz,
                             double ox, double oy, double oz) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const float s = slowness[(static_cast<long long>(cz) * ncy + cy) * ncx + cx];
    src->isx = cx; src->isy = cy; src->isz = cz;
    src->xs = static_cast<float>(ox); src->ys = static_cast<float>(oy); src->zs = static_cast<float>(oz);
    src->sSrc = s;
    if (src64) *src64 = f64;
    corner->isx = cx; corner->isy = cy; corner->isz = cz;
    corner->xo = ox; corner->yo = oy; corner->zo = oz;
    corner->s = static_cast<double>(s);
}

bool locate(double x, double x0, double d, int n, int *cell, double *offset) {
    const double x1 = x0 + static_cast<double>(n - 1) * d;
    if (!(x >= x0 && x <= x1)) return false;
    *offset = x - x0;
    *cell = std::min(n - 2, static_cast<int>(*offset / d));
    return true;
}

}  // namespace

extern "C" eikx_status eikx_solve3d_noalloc(int nx, int ny, int nz, double dx, double dy, double dz, double x0,
                                            double y0, double z0, const float *slowness,
                                            const eikx_source3d *src, const eikx_options *opt, float *tOut,
                                            void *streamHandle) {
    if (nx < 3 || ny < 3 || nz < 3) return err(EIKX_ERR_INVALID, "grid needs at least 3 points per axis");
    if (!(dx > 0) || !(dy > 0) || !(dz > 0)) return err(EIKX_ERR_INVALID, "grid spacing must be positive");
    if (!slowness || !src || !tOut) return err(EIKX_ERR_INVALID, "slowness, source and output must not be NULL");
    eikx_options o;
    if (opt) o = *opt; else eikx_options_default(&o);
    // the option checks of eikx_solve3d
    if (o.n_sweeps < 0) return err(EIKX_ERR_INVALID, "n_sweeps must be non-negative");
    if (o.factored_radius < 0) o.factored_radius = 0;
    if (o.block_shape < 0 || o.block_shape > eikx::kNumShapes) return err(EIKX_ERR_INVALID, "block_shape must be 0..3");
    if (o.sweep_kernel < 0 || o.sweep_kernel > 2) return err(EIKX_ERR_INVALID, "sweep_kernel must be 0..2");
    if (o.blocks_per_sm < 0) return err(EIKX_ERR_INVALID, "blocks_per_sm must be >= 0");
    if (o.near_fp64 < 0 || o.near_fp64 > 1) return err(EIKX_ERR_INVALID, "near_fp64 must be 0 or 1");
    if (o.near_fp64) o.sweep_kernel = eikx::kChunkStep;   // the FP64 factored branch's kernel
    int cx, cy, cz;
    double ox, oy, oz;
    if (!locate(src->x, x0, dx, nx, &cx, &ox) || !locate(src->y, y0, dy, ny, &cy, &oy) ||
        !locate(src->z, z0, dz, nz, &cz, &oz))
        return err(EIKX_ERR_INVALID, "source position outside the grid");

    // the FP64 analytic factor's table box (near_fp64): the nodes within the radius
    int bo[3] = {0, 0, 0}, be[3] = {0, 0, 0};
    if (o.near_fp64 && (!eikx::factorBox(cx, cy, cz, o.factored_radius, nx, ny, nz, bo, be) ||
                        8ll * be[0] * be[1] * be[2] > kFactorEntries))
        return err(EIKX_ERR_UNSUPPORTED, "near_fp64: the factored region of radius " +
                                             std::to_string(o.factored_radius) + " needs more than " +
                                             std::to_string(kFactorEntries) + " table entries");

    // layout and scratch need (same shapes as eikx_solve3d): the chunk-step kernel takes
    // the requested warp-block shape, the node-step kernel is 8x4
    const bool chunk = o.sweep_kernel != eikx::kNodeStep;
    const int shape = chunk && o.block_shape > 0 ? o.block_shape - 1 : eikx::kShape8x4;
    const int ly = eikx::shapeLY(shape), lz = eikx::shapeLZ(shape);
    const int Px = (nx + 3) / 4 * 4;
    const int spPitch = Px + 8;
    const int tilesY = (ny + ly - 1) / ly, tilesZ = (nz + lz - 1) / lz;
    const int nTiles = tilesY * tilesZ;
    const int nSweeps = o.n_sweeps;
    const int nSweepLaunches = 8 * ((o.init_sweeps ? 1 : 0) + nSweeps);
    const int resStride = 8 * (1 + nSweeps);
    const size_t spElems = static_cast<size_t>(spPitch) * (ny + 1) * (nz + 1);
    Carve plan{nullptr};
    plan.take<float>(static_cast<size_t>(Px) * ny * nz);                       // travel times
    plan.take<float>(spElems);                                                  // slowness, +x sweeps
    plan.take<float>(spElems);                                                  // slowness, -x sweeps
    plan.take<unsigned long long>(static_cast<size_t>(nTiles) * (ly + lz) * Px);  // mailbox
    plan.take<unsigned long long>(static_cast<size_t>(resStride));             // residual slots
    plan.take<unsigned>(8);                                                     // queue heads, epoch, flags
    plan.take<int4>(static_cast<size_t>(nTiles));                               // work order
    plan.take<eikx::SourceT<float>>(1);
    plan.take<eikx::Corner3>(1);
    plan.take<eikx::SourceFp64>(1);
    if (o.near_fp64) plan.take<eikx::NearFactor>(kFactorEntries);               // FP64 factor table
    if (plan.used > kScratchBytes)
        return err(EIKX_ERR_INVALID, "grid " + std::to_string(nx) + "x" + std::to_string(ny) + "x" +
                                         std::to_string(nz) + " needs " + std::to_string(plan.used) +
                                         " bytes of scratch; the no-allocation solve has " +
                                         std::to_string(kScratchBytes) + " (64 MiB)");

    cudaStream_t stream = static_cast<cudaStream_t>(streamHandle);
    int device = 0;
    NOALLOC_CUDA(cudaGetDevice(&device));
    unsigned char *base = nullptr;
    if (eikx_status r = scratchAddress(device, stream, &base); r != EIKX_OK) return r;
    Carve cv{base};
    float *tt = cv.take<float>(static_cast<size_t>(Px) * ny * nz);
    float *spPos = cv.take<float>(spElems);
    float *spNeg = cv.take<float>(spElems);
    const size_t mboxWords = static_cast<size_t>(nTiles) * (ly + lz) * Px;
    unsigned long long *mbox = cv.take<unsigned long long>(mboxWords);
    unsigned long long *residual = cv.take<unsigned long long>(static_cast<size_t>(resStride));
    // [0..1] queue heads, [2] model check, [3] abort, [4] converged, [5] iterations,
    // [6..7] mailbox epoch
    unsigned *small = cv.take<unsigned>(8);
    int4 *order = cv.take<int4>(static_cast<size_t>(nTiles));
    eikx::SourceT<float> *srcDev = cv.take<eikx::SourceT<float>>(1);
    eikx::Corner3 *cornerDev = cv.take<eikx::Corner3>(1);
    eikx::SourceFp64 *src64Dev = cv.take<eikx::SourceFp64>(1);
    eikx::NearFactor *factorDev = o.near_fp64 ? cv.take<eikx::NearFactor>(kFactorEntries) : nullptr;

    int numSMs = 0;
    NOALLOC_CUDA(cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, device));
    const double eps = std::numeric_limits<float>::epsilon() * 100;
    const bool uniform = std::abs(dx - dy) < eps && std::abs(dx - dz) < eps;
    int perSM = chunk ? eikx::sweep3ChunkBlocksPerSM<float>(uniform, false, shape)
                      : eikx::sweep3BlocksPerSM<float>(uniform);
    if (o.blocks_per_sm > 0) perSM = std::min(perSM, o.blocks_per_sm);
    const int blocks = std::max(1, std::min(numSMs * perSM, (nTiles + eikx::kWarpsPerBlock - 1) / eikx::kWarpsPerBlock));

    eikx::SolveState st{};
    st.queue[0] = small;
    st.queue[1] = small + 1;
    st.epoch = small + 6;
    st.abortFlag = reinterpret_cast<int *>(small + 3);
    st.converged = reinterpret_cast<int *>(small + 4);
    st.sweepsRun = reinterpret_cast<int *>(small + 5);
    st.mbox = mbox;
    st.epochStride = nSweepLaunches + 1;
    st.residual = residual;
    st.residualStride = resStride;
    st.order = order;
    const int drop = std::min(std::max(o.test_drop_blocks, 0), nTiles);
    st.order = order + drop;
    st.totalItems = nTiles - drop;
    const int spinLog2 = o.spin_limit_log2 > 0 ? std::min(o.spin_limit_log2, 40) : 22;
    st.spinLimit = 1ull << spinLog2;

    // The scratch array is laid out afresh for each grid, so the mailbox and the control
    // words may hold another call's data: clear them (tag 0 is never a sweep's tag).
    NOALLOC_CUDA(cudaMemsetAsync(mbox, 0, mboxWords * sizeof(unsigned long long), stream));
    NOALLOC_CUDA(cudaMemsetAsync(small, 0, 8 * sizeof(unsigned), stream));
    // the model check of eikx_set_slowness3d: every slowness positive and finite
    int bad = 0;
    NOALLOC_CUDA(eikx::launchCheckPositive(slowness, static_cast<long long>(nx - 1) * (ny - 1) * (nz - 1),
                                           reinterpret_cast<int *>(small + 2), stream));
    NOALLOC_CUDA(cudaMemcpyAsync(&bad, small + 2, sizeof(int), cudaMemcpyDeviceToHost, stream));
    NOALLOC_CUDA(cudaStreamSynchronize(stream));
    if (bad) return err(EIKX_ERR_INVALID, "Non-positive velocities detected");
    orderKernel<<<(nTiles + 127) / 128, 128, 0, stream>>>(order, tilesY, tilesZ, ly, lz);
    NOALLOC_CUDA(cudaGetLastError());
    // FP64 analytic factor: offsets, spacing and the factor table carved from the scratch
    eikx::SourceFp64 f64{};
    f64.xs = ox; f64.ys = oy; f64.zs = oz; f64.dx = dx; f64.dy = dy; f64.dz = dz;
    f64.sp = spNeg; f64.spPitch = spPitch; f64.spPlane = static_cast<long long>(spPitch) * (ny + 1);
    f64.ncx = nx - 1; f64.ncy = ny - 1; f64.ncz = nz - 1;
    if (o.near_fp64) {
        f64.table = factorDev;
        f64.bx0 = bo[0]; f64.by0 = bo[1]; f64.bz0 = bo[2];
        f64.bnx = be[0]; f64.bny = be[1]; f64.bnz = be[2];
    }
    sourceKernel<<<1, 32, 0, stream>>>(srcDev, cornerDev, o.near_fp64 ? src64Dev : nullptr, f64, slowness, nx - 1,
                                       ny - 1, cx, cy, cz, ox, oy, oz);
    NOALLOC_CUDA(cudaGetLastError());
    // the table is filled after the padded slowness copies (below)
    NOALLOC_CUDA((eikx::launchPadSlowness3<float, float>(spPos, spPitch, 3, slowness, nx, ny, nz, stream)));
    NOALLOC_CUDA((eikx::launchPadSlowness3<float, float>(spNeg, spPitch, 0, slowness, nx, ny, nz, stream)));
    if (o.near_fp64 && f64.table) NOALLOC_CUDA(eikx::launchFactorTables(src64Dev, 1, stream));
    NOALLOC_CUDA(eikx::launchResetState(st, 1, 0, stream));
    NOALLOC_CUDA(eikx::launchInit3<float>(tt, 1, static_cast<long long>(Px) * ny * nz, Px, nx, ny, nz, dx, dy, dz,
                                          cornerDev, o.init_fp64 ? 1 : 0, stream));
    const float fdx = static_cast<float>(dx), fdy = static_cast<float>(dy), fdz = static_cast<float>(dz);
    eikx::Spacing3<float> g;
    g.dx = fdx; g.dy = fdy; g.dz = fdz;
    g.dxInv = 1 / fdx; g.dyInv = 1 / fdy; g.dzInv = 1 / fdz;
    g.dx2Inv = 1 / (fdx * fdx); g.dy2Inv = 1 / (fdy * fdy); g.dz2Inv = 1 / (fdz * fdz);
    g.dx_dz = fdx / fdz; g.dz_dx = fdz / fdx; g.dy_dz = fdy / fdz; g.dz_dy = fdz / fdy;
    g.dx_dy = fdx / fdy; g.dy_dx = fdy / fdx;
    g.dx2_p_dz2_inv = 1 / (fdx * fdx + fdz * fdz);
    g.dy2_p_dz2_inv = 1 / (fdy * fdy + fdz * fdz);
    g.dx2_p_dy2_inv = 1 / (fdx * fdx + fdy * fdy);
    int buf = 0, launched = 0;
    auto sweep = [&](int e, int init, int slot) -> eikx_status {
        eikx::Sweep3Args<float> a{};
        a.tt = tt; a.fieldStride = static_cast<long long>(Px) * ny * nz; a.pitch = Px;
        a.spPos = spPos; a.spNeg = spNeg; a.spPitch = spPitch; a.spPlane = static_cast<long long>(spPitch) * (ny + 1);
        a.nx = nx; a.ny = ny; a.nz = nz; a.tilesY = tilesY; a.tilesZ = tilesZ;
        a.srcs = srcDev; a.st = st; a.buf = buf; a.sweepIndex = launched; a.residualSlot = slot;
        a.sweep = e; a.init = init; a.radius = o.factored_radius; a.h = fdx; a.sp3 = g;
        a.srcs64 = o.near_fp64 ? src64Dev : nullptr;
        if (chunk) NOALLOC_CUDA(eikx::launchSweep3Chunk<float>(a, uniform, shape, blocks, stream));
        else NOALLOC_CUDA(eikx::launchSweep3<float>(a, uniform, blocks, stream));
        buf ^= 1;
        ++launched;
        return EIKX_OK;
    };
    if (o.init_sweeps)
        for (int e = 0; e < 8; ++e)
            if (eikx_status r = sweep(e, 1, e); r != EIKX_OK) return r;
    for (int k = 0; k < nSweeps; ++k) {
        for (int e = 0; e < 8; ++e) {
            if (eikx_status r = sweep(e, 0, 8 * (1 + k) + e); r != EIKX_OK) return r;
            // the window: the last 8 refinement sweeps (fewer in the first iteration: no test)
            const int j = 8 * k + e, lo = std::max(0, j - 7);
            NOALLOC_CUDA(eikx::launchCheckConvergence(st, 1, 8 + lo, j - lo + 1, j + 1, j >= 7 ? o.tolerance : -1.0,
                                                      stream));
        }
    }
    NOALLOC_CUDA(eikx::copyRows(tOut, static_cast<size_t>(nx) * sizeof(float), tt, static_cast<size_t>(Px) * sizeof(float),
                                   static_cast<size_t>(nx) * sizeof(float), static_cast<size_t>(ny) * nz,
                                   cudaMemcpyDeviceToDevice, stream));
    int aborted = 0;
    NOALLOC_CUDA(cudaMemcpyAsync(&aborted, st.abortFlag, sizeof(int), cudaMemcpyDeviceToHost, stream));
    NOALLOC_CUDA(cudaStreamSynchronize(stream));
    if (aborted) return err(EIKX_ERR_TIMEOUT, "a bounded inter-tile wait ran out; the field is not valid");
    return EIKX_OK;
}
