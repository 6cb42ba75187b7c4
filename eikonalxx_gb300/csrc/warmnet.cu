// Host side of the learned warm start: the travel-time predictor behind
// eikx_warmnet_* (include/eikx/eikx_c.h).  No counterpart in the reference.
//
// A network object owns its stream, its parameters (FP32 master vector, BF16 copy,
// flipped-and-transposed BF16 copies for the input-gradient convolutions, Adam moments)
// and every activation and gradient buffer for `batch` samples, allocated once at
// creation.  A training step is: features -> 14 convolutions (pooling and up-and-concat
// kernels between levels) -> head and loss -> the backward pass in reverse (per
// convolution: weight gradient, bias gradient, input gradient with the ReLU gate of its
// input fused where that input has no other consumer) -> Adam.  All of it runs on the
// network's stream; the call returns after reading the loss.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "eikx/eikx_c.h"
#include "warmnet.h"

eikx_status eikxSetLastError(eikx_status code, const char *msg);

using eikx::net::bf16;

namespace {

eikx_status err(eikx_status code, const std::string &m) { return eikxSetLastError(code, m.c_str()); }

#define NET_CUDA(expr)                                                                               \
    do {                                                                                             \
        cudaError_t e_ = (expr);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            return err(e_ == cudaErrorMemoryAllocation ? EIKX_ERR_ALLOC : EIKX_ERR_CUDA,             \
                       std::string(#expr) + ": " + cudaGetErrorString(e_));                          \
    } while (0)

enum Layer { E0a, E0b, E1a, E1b, E2a, E2b, Ba, Bb, D2a, D2b, D1a, D1b, D0a, D0b, kLayers };
// input channels, output channels, level (resolution 2^-level)
constexpr int kSpec[kLayers][3] = {{16, 16, 0}, {16, 16, 0},   {16, 32, 1},  {32, 32, 1},   {32, 64, 2},
                                   {64, 64, 2}, {64, 128, 3},  {128, 128, 3}, {192, 64, 2}, {64, 64, 2},
                                   {96, 32, 1}, {32, 32, 1},   {48, 16, 0},  {16, 16, 0}};
constexpr int kHeadIn = 16;
constexpr int kFeatures = 16;

enum Category { kFwd, kDgrad, kWgrad, kOther, kCategories };

}  // namespace

struct eikx_warmnet {
    int device = 0, numSMs = 0, batch = 0;
    cudaStream_t stream = nullptr;
    eikx::net::Geometry g{};
    int dim[4][3] = {};        // level -> D, H, W
    long long V[4] = {};       // nodes per sample per level
    long long wOff[kLayers] = {}, bOff[kLayers] = {}, wtOff[kLayers] = {};
    long long headOff = 0, nParams = 0, nWt = 0;
    float *P = nullptr, *G = nullptr, *M = nullptr, *Vm = nullptr;
    bf16 *Pb = nullptr, *Wt = nullptr;
    bf16 *feat = nullptr;
    bf16 *act[kLayers] = {}, *gpre[kLayers] = {};
    bf16 *pool[3] = {}, *cat[3] = {}, *gcat[3] = {}, *gpool[3] = {};
    float *tOut = nullptr;
    float *slow = nullptr;          // [batch][V] nodal slowness of the current samples
    eikx::net::Sample *dSamples = nullptr, *hSamples = nullptr;
    double *dLoss = nullptr, *hLoss = nullptr;
    int *dStatus = nullptr, *hStatus = nullptr;   // raised by a bounded wait that ran out
    long long spin = 0;             // tcgen05 waits: polls before giving up (0: the kernel's default)
    int testLate = 0;               // test hook of the tcgen05 waits (eikx_warmnet_set_test_hooks)
    long long step = 0;
    std::vector<void *> allocs;
    // profiling: an event pair per launch and its category
    bool prof = false;
    std::vector<cudaEvent_t> events;
    std::vector<int> evCat;
    size_t evUsed = 0;
};

namespace {

template <class T>
cudaError_t alloc(eikx_warmnet *n, T **p, long long count) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, static_cast<size_t>(std::max<long long>(count, 1)) * sizeof(T));
    if (e != cudaSuccess) return e;
    n->allocs.push_back(q);
    *p = static_cast<T *>(q);
    return cudaSuccess;
}

void freeAll(eikx_warmnet *n) {
    for (void *p : n->allocs) cudaFree(p);
    n->allocs.clear();
    if (n->hSamples) cudaFreeHost(n->hSamples);
    if (n->hLoss) cudaFreeHost(n->hLoss);
    if (n->hStatus) cudaFreeHost(n->hStatus);
    for (cudaEvent_t e : n->events) cudaEventDestroy(e);
    if (n->stream) cudaStreamDestroy(n->stream);
}

// splitmix64 + Box-Muller: a seeded normal stream that is the same on every platform.
struct Rng {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (static_cast<double>(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
    double normal() {
        const double u1 = uniform(), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

// Runs `launch` (returning cudaError_t) and, when profiling, brackets it with events.
template <class F>
cudaError_t timed(eikx_warmnet *n, int category, F &&launch) {
    if (!n->prof) return launch();
    if (n->evUsed + 2 > n->events.size()) {
        for (int k = 0; k < 2; ++k) {
            cudaEvent_t e;
            cudaError_t r = cudaEventCreate(&e);
            if (r != cudaSuccess) return r;
            n->events.push_back(e);
        }
    }
    cudaEventRecord(n->events[n->evUsed], n->stream);
    cudaError_t r = launch();
    cudaEventRecord(n->events[n->evUsed + 1], n->stream);
    n->evCat.push_back(category);
    n->evUsed += 2;
    return r;
}

const bf16 *inputOf(const eikx_warmnet *n, int L) {
    switch (L) {
        case E0a: return n->feat;
        case E1a: return n->pool[0];
        case E2a: return n->pool[1];
        case Ba: return n->pool[2];
        case D2a: return n->cat[2];
        case D1a: return n->cat[1];
        case D0a: return n->cat[0];
        default: return n->act[L - 1];
    }
}

double convFlops(const eikx_warmnet *n, int L, int B) {
    return 2.0 * B * n->V[kSpec[L][2]] * 27.0 * kSpec[L][0] * kSpec[L][1];
}

cudaError_t conv(eikx_warmnet *n, int L, int B) {
    const int lv = kSpec[L][2];
    eikx::net::ConvArgs a{};
    a.x = inputOf(n, L);
    a.cin = kSpec[L][0];
    a.w = n->Pb + n->wOff[L];
    a.bias = n->P + n->bOff[L];
    a.y = n->act[L];
    a.cout = kSpec[L][1];
    a.relu = 1;
    a.D = n->dim[lv][0];
    a.H = n->dim[lv][1];
    a.W = n->dim[lv][2];
    a.B = B;
    a.status = n->dStatus;
    a.spin = n->spin;
    a.testLate = n->testLate;
    return timed(n, kFwd, [&] { return eikx::net::launchConv(a, n->stream); });
}

// Weight and bias gradients of layer L, then (when dx) its input gradient, gated by
// mask (the ReLU output feeding L) when given.
cudaError_t convBack(eikx_warmnet *n, int L, int B, bf16 *dx, const bf16 *mask) {
    const int lv = kSpec[L][2];
    const int D = n->dim[lv][0], H = n->dim[lv][1], W = n->dim[lv][2];
    eikx::net::WGradArgs w{};
    w.x = inputOf(n, L);
    w.cin = kSpec[L][0];
    w.dy = n->gpre[L];
    w.cout = kSpec[L][1];
    w.dw = n->G + n->wOff[L];
    w.D = D;
    w.H = H;
    w.W = W;
    w.B = B;
    cudaError_t e = timed(n, kWgrad, [&] { return eikx::net::launchWGrad(w, n->numSMs, n->stream); });
    if (e != cudaSuccess) return e;
    e = timed(n, kOther, [&] {
        return eikx::net::launchBiasGrad(n->gpre[L], kSpec[L][1], B * n->V[lv], n->G + n->bOff[L], n->numSMs,
                                         n->stream);
    });
    if (e != cudaSuccess || !dx) return e;
    eikx::net::ConvArgs a{};
    a.x = n->gpre[L];
    a.cin = kSpec[L][1];
    a.w = n->Wt + n->wtOff[L];
    a.bias = nullptr;
    a.y = dx;
    a.cout = kSpec[L][0];
    a.mask = mask;
    a.relu = 0;
    a.D = D;
    a.H = H;
    a.W = W;
    a.B = B;
    a.status = n->dStatus;
    a.spin = n->spin;
    a.testLate = n->testLate;
    return timed(n, kDgrad, [&] { return eikx::net::launchConv(a, n->stream); });
}

#define NET_STEP(expr)                           \
    do {                                         \
        cudaError_t e_ = (expr);                 \
        if (e_ != cudaSuccess) return e_;        \
    } while (0)

cudaError_t forward(eikx_warmnet *n, int B) {
    auto lvl = [&](int l, int k) { return n->dim[l][k]; };
    NET_STEP(timed(n, kOther, [&] { return eikx::net::launchSlowness(n->dSamples, n->g, B, n->slow, n->stream); }));
    NET_STEP(timed(n, kOther,
                   [&] { return eikx::net::launchFeatures(n->dSamples, n->slow, n->g, B, n->feat, n->stream); }));
    NET_STEP(conv(n, E0a, B));
    NET_STEP(conv(n, E0b, B));
    NET_STEP(timed(n, kOther, [&] {
        return eikx::net::launchPool(n->act[E0b], 16, lvl(0, 0), lvl(0, 1), lvl(0, 2), B, n->pool[0], n->stream);
    }));
    NET_STEP(conv(n, E1a, B));
    NET_STEP(conv(n, E1b, B));
    NET_STEP(timed(n, kOther, [&] {
        return eikx::net::launchPool(n->act[E1b], 32, lvl(1, 0), lvl(1, 1), lvl(1, 2), B, n->pool[1], n->stream);
    }));
    NET_STEP(conv(n, E2a, B));
    NET_STEP(conv(n, E2b, B));
    NET_STEP(timed(n, kOther, [&] {
        return eikx::net::launchPool(n->act[E2b], 64, lvl(2, 0), lvl(2, 1), lvl(2, 2), B, n->pool[2], n->stream);
    }));
    NET_STEP(conv(n, Ba, B));
    NET_STEP(conv(n, Bb, B));
    NET_STEP(timed(n, kOther, [&] {
        return eikx::net::launchUpcat(n->act[Bb], 128, n->act[E2b], 64, lvl(2, 0), lvl(2, 1), lvl(2, 2), B,
                                      n->cat[2], n->stream);
    }));
    NET_STEP(conv(n, D2a, B));
    NET_STEP(conv(n, D2b, B));
    NET_STEP(timed(n, kOther, [&] {
        return eikx::net::launchUpcat(n->act[D2b], 64, n->act[E1b], 32, lvl(1, 0), lvl(1, 1), lvl(1, 2), B,
                                      n->cat[1], n->stream);
    }));
    NET_STEP(conv(n, D1a, B));
    NET_STEP(conv(n, D1b, B));
    NET_STEP(timed(n, kOther, [&] {
        return eikx::net::launchUpcat(n->act[D1b], 32, n->act[E0b], 16, lvl(0, 0), lvl(0, 1), lvl(0, 2), B,
                                      n->cat[0], n->stream);
    }));
    NET_STEP(conv(n, D0a, B));
    NET_STEP(conv(n, D0b, B));
    return cudaSuccess;
}

cudaError_t backward(eikx_warmnet *n, int B, double invN) {
    auto lvl = [&](int l, int k) { return n->dim[l][k]; };
    NET_STEP(cudaMemsetAsync(n->G, 0, sizeof(float) * n->nParams, n->stream));
    NET_STEP(timed(n, kOther, [&] {
        return eikx::net::launchHeadLoss(n->act[D0b], n->P + n->headOff, n->dSamples, n->slow, n->g, B, invN,
                                         n->G + n->headOff, n->gpre[D0b], n->dLoss, n->stream);
    }));
    NET_STEP(convBack(n, D0b, B, n->gpre[D0a], n->act[D0a]));
    NET_STEP(convBack(n, D0a, B, n->gcat[0], nullptr));
    NET_STEP(timed(n, kOther, [&] {
        return eikx::net::launchUpSumMask(n->gcat[0], 48, n->act[D1b], 32, lvl(1, 0), lvl(1, 1), lvl(1, 2), B,
                                          n->gpre[D1b], n->stream);
    }));
    NET_STEP(convBack(n, D1b, B, n->gpre[D1a], n->act[D1a]));
    NET_STEP(convBack(n, D1a, B, n->gcat[1], nullptr));
    NET_STEP(timed(n, kOther, [&] {
        return eikx::net::launchUpSumMask(n->gcat[1], 96, n->act[D2b], 64, lvl(2, 0), lvl(2, 1), lvl(2, 2), B,
                                          n->gpre[D2b], n->stream);
    }));
    NET_STEP(convBack(n, D2b, B, n->gpre[D2a], n->act[D2a]));
    NET_STEP(convBack(n, D2a, B, n->gcat[2], nullptr));
    NET_STEP(timed(n, kOther, [&] {
        return eikx::net::launchUpSumMask(n->gcat[2], 192, n->act[Bb], 128, lvl(3, 0), lvl(3, 1), lvl(3, 2), B,
                                          n->gpre[Bb], n->stream);
    }));
    NET_STEP(convBack(n, Bb, B, n->gpre[Ba], n->act[Ba]));
    NET_STEP(convBack(n, Ba, B, n->gpool[2], nullptr));
    NET_STEP(timed(n, kOther, [&] {
        return eikx::net::launchCombineSkip(n->gcat[2], 192, 128, n->gpool[2], n->act[E2b], 64, lvl(2, 0),
                                            lvl(2, 1), lvl(2, 2), B, n->gpre[E2b], n->stream);
    }));
    NET_STEP(convBack(n, E2b, B, n->gpre[E2a], n->act[E2a]));
    NET_STEP(convBack(n, E2a, B, n->gpool[1], nullptr));
    NET_STEP(timed(n, kOther, [&] {
        return eikx::net::launchCombineSkip(n->gcat[1], 96, 64, n->gpool[1], n->act[E1b], 32, lvl(1, 0), lvl(1, 1),
                                            lvl(1, 2), B, n->gpre[E1b], n->stream);
    }));
    NET_STEP(convBack(n, E1b, B, n->gpre[E1a], n->act[E1a]));
    NET_STEP(convBack(n, E1a, B, n->gpool[0], nullptr));
    NET_STEP(timed(n, kOther, [&] {
        return eikx::net::launchCombineSkip(n->gcat[0], 48, 32, n->gpool[0], n->act[E0b], 16, lvl(0, 0), lvl(0, 1),
                                            lvl(0, 2), B, n->gpre[E0b], n->stream);
    }));
    NET_STEP(convBack(n, E0b, B, n->gpre[E0a], n->act[E0a]));
    NET_STEP(convBack(n, E0a, B, nullptr, nullptr));
    return cudaSuccess;
}

// BF16 copies of the parameters after they change.
cudaError_t refreshCopies(eikx_warmnet *n) {
    for (int L = 0; L < kLayers; ++L)
        NET_STEP(eikx::net::launchFlipTranspose(n->Pb + n->wOff[L], kSpec[L][1], kSpec[L][0], n->Wt + n->wtOff[L],
                                                n->stream));
    return cudaSuccess;
}

eikx_status checkNet(const eikx_warmnet *n) {
    if (!n) return err(EIKX_ERR_INVALID, "net is NULL");
    return EIKX_OK;
}

// Copies the samples to the device; returns the number of nodes with T0 > 0.
eikx_status stageSamples(eikx_warmnet *n, const eikx_warmnet_sample *s, int count, bool needTarget,
                         long long *nodes) {
    if (!s) return err(EIKX_ERR_INVALID, "samples is NULL");
    if (count < 1 || count > n->batch)
        return err(EIKX_ERR_INVALID, "number of samples = " + std::to_string(count) + " must be in [1, " +
                                         std::to_string(n->batch) + "]");
    long long zero = 0;
    const eikx::net::Geometry &g = n->g;
    for (int i = 0; i < count; ++i) {
        if (!s[i].velocity) return err(EIKX_ERR_INVALID, "sample " + std::to_string(i) + ": velocity is NULL");
        if (needTarget && !s[i].travel_time)
            return err(EIKX_ERR_INVALID, "sample " + std::to_string(i) + ": travel_time is NULL");
        if (!std::isfinite(s[i].x) || !std::isfinite(s[i].y) || !std::isfinite(s[i].z))
            return err(EIKX_ERR_INVALID, "sample " + std::to_string(i) + ": source position is not finite");
        n->hSamples[i] = eikx::net::Sample{s[i].velocity, s[i].travel_time, s[i].x, s[i].y, s[i].z};
        // the node nearest the source, as the kernels find it; T0 = 0 only there
        auto near = [](double p, double o, double d, int nn) {
            const double r = std::nearbyint((p - o) / d);
            return static_cast<int>(std::min<double>(nn - 1, std::max<double>(0.0, r)));
        };
        const int ix = near(s[i].x, g.x0, g.dx, g.nx), iy = near(s[i].y, g.y0, g.dy, g.ny),
                  iz = near(s[i].z, g.z0, g.dz, g.nz);
        if (g.x0 + ix * g.dx == s[i].x && g.y0 + iy * g.dy == s[i].y && g.z0 + iz * g.dz == s[i].z) ++zero;
    }
    NET_CUDA(cudaMemcpyAsync(n->dSamples, n->hSamples, sizeof(eikx::net::Sample) * count, cudaMemcpyHostToDevice,
                             n->stream));
    *nodes = count * n->V[0] - zero;
    return EIKX_OK;
}

eikx_status finishLoss(eikx_warmnet *n, long long nodes, double *loss) {
    NET_CUDA(cudaMemcpyAsync(n->hLoss, n->dLoss, sizeof(double), cudaMemcpyDeviceToHost, n->stream));
    NET_CUDA(cudaMemcpyAsync(n->hStatus, n->dStatus, sizeof(int), cudaMemcpyDeviceToHost, n->stream));
    NET_CUDA(cudaStreamSynchronize(n->stream));
    if (*n->hStatus) {
        NET_CUDA(cudaMemsetAsync(n->dStatus, 0, sizeof(int), n->stream));
        NET_CUDA(cudaStreamSynchronize(n->stream));
        return err(EIKX_ERR_TIMEOUT, "a bounded wait of a tensor-core convolution ran out; the results are not valid");
    }
    if (loss) *loss = nodes > 0 ? *n->hLoss / static_cast<double>(nodes) : 0.0;
    return EIKX_OK;
}

eikx_status trainStep(eikx_warmnet *n, const eikx_warmnet_sample *s, int count, float lr, double *loss) {
    if (!(lr >= 0.f) || !std::isfinite(lr)) return err(EIKX_ERR_INVALID, "learning rate must be finite and >= 0");
    long long nodes = 0;
    if (eikx_status r = stageSamples(n, s, count, true, &nodes); r != EIKX_OK) return r;
    NET_CUDA(cudaMemsetAsync(n->dLoss, 0, sizeof(double), n->stream));
    NET_CUDA(forward(n, count));
    NET_CUDA(backward(n, count, nodes > 0 ? 1.0 / static_cast<double>(nodes) : 0.0));
    ++n->step;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = static_cast<float>(1.0 - std::pow(0.9, static_cast<double>(n->step)));
    const float bc2 = static_cast<float>(1.0 - std::pow(0.999, static_cast<double>(n->step)));
    NET_CUDA(timed(n, kOther, [&] {
        return eikx::net::launchAdam(n->P, n->G, n->M, n->Vm, n->Pb, n->nParams, lr, b1, b2, 1e-8f, bc1, bc2,
                                     n->stream);
    }));
    NET_CUDA(timed(n, kOther, [&] { return refreshCopies(n); }));
    return finishLoss(n, nodes, loss);
}

}  // namespace

extern "C" {

eikx_status eikx_warmnet_create(int device, const eikx_warmnet_config *cfg, eikx_warmnet **out) {
    if (!out) return err(EIKX_ERR_INVALID, "net is NULL");
    *out = nullptr;
    if (!cfg) return err(EIKX_ERR_INVALID, "config is NULL");
    const int ext[3] = {cfg->nx, cfg->ny, cfg->nz};
    const char *axis = "xyz";
    for (int k = 0; k < 3; ++k)
        if (ext[k] < 8 || ext[k] % 8)
            return err(EIKX_ERR_INVALID, std::string("Number of grid points in ") + axis[k] + " = " +
                                             std::to_string(ext[k]) + " must be a positive multiple of 8");
    if (!(cfg->dx > 0) || !(cfg->dy > 0) || !(cfg->dz > 0) || !std::isfinite(cfg->dx) || !std::isfinite(cfg->dy) ||
        !std::isfinite(cfg->dz))
        return err(EIKX_ERR_INVALID, "grid spacing must be positive and finite");
    if (!std::isfinite(cfg->x0) || !std::isfinite(cfg->y0) || !std::isfinite(cfg->z0))
        return err(EIKX_ERR_INVALID, "grid origin must be finite");
    if (cfg->batch < 1) return err(EIKX_ERR_INVALID, "batch must be at least 1");
    int nDev = 0;
    if (cudaGetDeviceCount(&nDev) != cudaSuccess || nDev == 0) return err(EIKX_ERR_CUDA, "no CUDA device");
    if (device < 0 || device >= nDev) return err(EIKX_ERR_INVALID, "device " + std::to_string(device) + " not present");
    NET_CUDA(cudaSetDevice(device));

    auto *n = new eikx_warmnet;
    n->device = device;
    n->batch = cfg->batch;
    cudaDeviceGetAttribute(&n->numSMs, cudaDevAttrMultiProcessorCount, device);
    eikx::net::Geometry &g = n->g;
    g.nx = cfg->nx;
    g.ny = cfg->ny;
    g.nz = cfg->nz;
    g.dx = cfg->dx;
    g.dy = cfg->dy;
    g.dz = cfg->dz;
    g.x0 = cfg->x0;
    g.y0 = cfg->y0;
    g.z0 = cfg->z0;
    const double lx = (g.nx - 1) * g.dx, ly = (g.ny - 1) * g.dy, lz = (g.nz - 1) * g.dz;
    g.invL = 1.0 / std::sqrt(lx * lx + ly * ly + lz * lz);
    for (int l = 0; l < 4; ++l) {
        n->dim[l][0] = g.nz >> l;
        n->dim[l][1] = g.ny >> l;
        n->dim[l][2] = g.nx >> l;
        n->V[l] = static_cast<long long>(n->dim[l][0]) * n->dim[l][1] * n->dim[l][2];
    }
    long long off = 0, woff = 0;
    for (int L = 0; L < kLayers; ++L) {
        n->wOff[L] = off;
        off += 27LL * kSpec[L][0] * kSpec[L][1];
        n->bOff[L] = off;
        off += kSpec[L][1];
        n->wtOff[L] = woff;
        woff += 27LL * kSpec[L][0] * kSpec[L][1];
    }
    n->headOff = off;
    n->nParams = off + kHeadIn + 1;
    n->nWt = woff;

    auto fail = [&](cudaError_t e, const char *what) {
        freeAll(n);
        delete n;
        return err(e == cudaErrorMemoryAllocation ? EIKX_ERR_ALLOC : EIKX_ERR_CUDA,
                   std::string(what) + ": " + cudaGetErrorString(e));
    };
    cudaError_t e = cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail(e, "cudaStreamCreate");
    const long long B = cfg->batch;
    bool ok = alloc(n, &n->P, n->nParams) == cudaSuccess && alloc(n, &n->G, n->nParams) == cudaSuccess &&
              alloc(n, &n->M, n->nParams) == cudaSuccess && alloc(n, &n->Vm, n->nParams) == cudaSuccess &&
              alloc(n, &n->Pb, n->nParams) == cudaSuccess && alloc(n, &n->Wt, n->nWt) == cudaSuccess &&
              alloc(n, &n->feat, B * n->V[0] * kFeatures) == cudaSuccess &&
              alloc(n, &n->tOut, B * n->V[0]) == cudaSuccess && alloc(n, &n->slow, B * n->V[0]) == cudaSuccess &&
              alloc(n, &n->dSamples, B) == cudaSuccess &&
              alloc(n, &n->dLoss, 1) == cudaSuccess && alloc(n, &n->dStatus, 1) == cudaSuccess;
    for (int L = 0; ok && L < kLayers; ++L) {
        const long long c = B * n->V[kSpec[L][2]] * kSpec[L][1];
        ok = alloc(n, &n->act[L], c) == cudaSuccess && alloc(n, &n->gpre[L], c) == cudaSuccess;
    }
    const int catC[3] = {48, 96, 192}, poolC[3] = {16, 32, 64};
    for (int l = 0; ok && l < 3; ++l)
        ok = alloc(n, &n->cat[l], B * n->V[l] * catC[l]) == cudaSuccess &&
             alloc(n, &n->gcat[l], B * n->V[l] * catC[l]) == cudaSuccess &&
             alloc(n, &n->pool[l], B * n->V[l + 1] * poolC[l]) == cudaSuccess &&
             alloc(n, &n->gpool[l], B * n->V[l + 1] * poolC[l]) == cudaSuccess;
    if (!ok) return fail(cudaErrorMemoryAllocation, "allocating the network's buffers");
    if ((e = cudaMallocHost(&n->hSamples, sizeof(eikx::net::Sample) * B)) != cudaSuccess) return fail(e, "cudaMallocHost");
    if ((e = cudaMallocHost(&n->hLoss, sizeof(double))) != cudaSuccess) return fail(e, "cudaMallocHost");
    if ((e = cudaMallocHost(&n->hStatus, sizeof(int))) != cudaSuccess) return fail(e, "cudaMallocHost");
    if ((e = cudaMemsetAsync(n->dStatus, 0, sizeof(int), n->stream)) != cudaSuccess) return fail(e, "cudaMemset");

    // He-normal convolution weights (fan-in: 27 x the input channels carrying data), zero
    // biases and head: the untrained network predicts tau = 1, i.e. T = T0.
    std::vector<float> p(n->nParams, 0.f);
    Rng rng{cfg->seed};
    for (int L = 0; L < kLayers; ++L) {
        const int fanIn = 27 * (L == E0a ? 6 : kSpec[L][0]);
        const double sd = std::sqrt(2.0 / fanIn);
        for (long long i = 0; i < 27LL * kSpec[L][0] * kSpec[L][1]; ++i)
            p[n->wOff[L] + i] = static_cast<float>(sd * rng.normal());
    }
    eikx_status r = eikx_warmnet_set_params(n, p.data());
    if (r != EIKX_OK) {
        freeAll(n);
        delete n;
        return r;
    }
    *out = n;
    return EIKX_OK;
}

eikx_status eikx_warmnet_set_test_hooks(eikx_warmnet *n, int spin_limit_log2, int late) {
    if (eikx_status r = checkNet(n); r != EIKX_OK) return r;
    if (spin_limit_log2 < 0 || spin_limit_log2 > 40) return err(EIKX_ERR_INVALID, "spin_limit_log2 must be 0..40");
    if (late < 0 || late > 2) return err(EIKX_ERR_INVALID, "late must be 0, 1 or 2");
    n->spin = spin_limit_log2 > 0 ? (1ll << spin_limit_log2) : 0;
    n->testLate = late;
    return EIKX_OK;
}

eikx_status eikx_warmnet_destroy(eikx_warmnet *n) {
    if (!n) return EIKX_OK;
    cudaSetDevice(n->device);
    if (n->stream) cudaStreamSynchronize(n->stream);
    freeAll(n);
    delete n;
    return EIKX_OK;
}

eikx_status eikx_warmnet_num_params(const eikx_warmnet *n, long long *count) {
    if (eikx_status r = checkNet(n); r != EIKX_OK) return r;
    if (!count) return err(EIKX_ERR_INVALID, "count is NULL");
    *count = n->nParams;
    return EIKX_OK;
}

eikx_status eikx_warmnet_get_params(eikx_warmnet *n, float *params) {
    if (eikx_status r = checkNet(n); r != EIKX_OK) return r;
    if (!params) return err(EIKX_ERR_INVALID, "params is NULL");
    NET_CUDA(cudaSetDevice(n->device));
    NET_CUDA(cudaMemcpyAsync(params, n->P, sizeof(float) * n->nParams, cudaMemcpyDeviceToHost, n->stream));
    NET_CUDA(cudaStreamSynchronize(n->stream));
    return EIKX_OK;
}

eikx_status eikx_warmnet_set_params(eikx_warmnet *n, const float *params) {
    if (eikx_status r = checkNet(n); r != EIKX_OK) return r;
    if (!params) return err(EIKX_ERR_INVALID, "params is NULL");
    for (long long i = 0; i < n->nParams; ++i)
        if (!std::isfinite(params[i])) return err(EIKX_ERR_INVALID, "parameter " + std::to_string(i) + " is not finite");
    NET_CUDA(cudaSetDevice(n->device));
    NET_CUDA(cudaMemcpyAsync(n->P, params, sizeof(float) * n->nParams, cudaMemcpyHostToDevice, n->stream));
    NET_CUDA(cudaMemsetAsync(n->M, 0, sizeof(float) * n->nParams, n->stream));
    NET_CUDA(cudaMemsetAsync(n->Vm, 0, sizeof(float) * n->nParams, n->stream));
    NET_CUDA(eikx::net::launchToBF16(n->P, n->Pb, n->nParams, n->stream));
    NET_CUDA(refreshCopies(n));
    NET_CUDA(cudaStreamSynchronize(n->stream));
    n->step = 0;
    return EIKX_OK;
}

eikx_status eikx_warmnet_train_step(eikx_warmnet *n, const eikx_warmnet_sample *s, int count, float lr,
                                    double *loss) {
    if (eikx_status r = checkNet(n); r != EIKX_OK) return r;
    NET_CUDA(cudaSetDevice(n->device));
    return trainStep(n, s, count, lr, loss);
}

eikx_status eikx_warmnet_gradients(eikx_warmnet *n, const eikx_warmnet_sample *s, int count, float *grads,
                                   double *loss) {
    if (eikx_status r = checkNet(n); r != EIKX_OK) return r;
    if (!grads) return err(EIKX_ERR_INVALID, "grads is NULL");
    NET_CUDA(cudaSetDevice(n->device));
    long long nodes = 0;
    if (eikx_status r = stageSamples(n, s, count, true, &nodes); r != EIKX_OK) return r;
    NET_CUDA(cudaMemsetAsync(n->dLoss, 0, sizeof(double), n->stream));
    NET_CUDA(forward(n, count));
    NET_CUDA(backward(n, count, nodes > 0 ? 1.0 / static_cast<double>(nodes) : 0.0));
    NET_CUDA(cudaMemcpyAsync(grads, n->G, sizeof(float) * n->nParams, cudaMemcpyDeviceToHost, n->stream));
    return finishLoss(n, nodes, loss);
}

eikx_status eikx_warmnet_predict(eikx_warmnet *n, const eikx_warmnet_sample *s, int count, double inflate,
                                 float *t_out, int where, double *loss) {
    if (eikx_status r = checkNet(n); r != EIKX_OK) return r;
    if (!t_out) return err(EIKX_ERR_INVALID, "t_out is NULL");
    if (where != EIKX_HOST && where != EIKX_DEVICE) return err(EIKX_ERR_INVALID, "where must be EIKX_HOST or EIKX_DEVICE");
    if (!(inflate > 0) || !std::isfinite(inflate)) return err(EIKX_ERR_INVALID, "inflate must be positive and finite");
    NET_CUDA(cudaSetDevice(n->device));
    bool haveTargets = s != nullptr;
    for (int i = 0; haveTargets && i < count; ++i) haveTargets = s[i].travel_time != nullptr;
    long long nodes = 0;
    if (eikx_status r = stageSamples(n, s, count, false, &nodes); r != EIKX_OK) return r;
    NET_CUDA(cudaMemsetAsync(n->dLoss, 0, sizeof(double), n->stream));
    NET_CUDA(forward(n, count));
    float *dst = where == EIKX_DEVICE ? t_out : n->tOut;
    NET_CUDA(eikx::net::launchPredict(n->act[D0b], n->P + n->headOff, n->dSamples, n->slow, n->g, count, inflate, dst,
                                      haveTargets && loss ? n->dLoss : nullptr, n->stream));
    if (where == EIKX_HOST)
        NET_CUDA(cudaMemcpyAsync(t_out, n->tOut, sizeof(float) * count * n->V[0], cudaMemcpyDeviceToHost, n->stream));
    if (eikx_status r = finishLoss(n, nodes, haveTargets ? loss : nullptr); r != EIKX_OK) return r;
    if (loss && !haveTargets) *loss = -1.0;
    return EIKX_OK;
}

eikx_status eikx_warmnet_profile_step(eikx_warmnet *n, const eikx_warmnet_sample *s, int count, float lr, double *ms,
                                      double *flops) {
    if (eikx_status r = checkNet(n); r != EIKX_OK) return r;
    if (!ms || !flops) return err(EIKX_ERR_INVALID, "ms and flops must not be NULL");
    NET_CUDA(cudaSetDevice(n->device));
    n->prof = true;
    n->evUsed = 0;
    n->evCat.clear();
    double loss = 0;
    eikx_status r = trainStep(n, s, count, lr, &loss);
    n->prof = false;
    if (r != EIKX_OK) return r;
    for (int k = 0; k < kCategories; ++k) ms[k] = 0;
    for (size_t i = 0; i < n->evCat.size(); ++i) {
        float t = 0;
        NET_CUDA(cudaEventElapsedTime(&t, n->events[2 * i], n->events[2 * i + 1]));
        ms[n->evCat[i]] += t;
    }
    flops[0] = flops[1] = flops[2] = 0;
    for (int L = 0; L < kLayers; ++L) {
        const double f = convFlops(n, L, count);
        flops[kFwd] += f;
        flops[kWgrad] += f;
        if (L != E0a) flops[kDgrad] += f;
    }
    return EIKX_OK;
}

}  // extern "C"
