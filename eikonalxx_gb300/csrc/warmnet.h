// Device kernels of the learned warm start (the travel-time predictor of
// eikx_warmnet_*): a 3D U-Net over channels-last BF16 activations
// [sample][z][y][x][channel].  The reference has no counterpart; the network is
// described with its C entry points in include/eikx/eikx_c.h.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace eikx {
namespace net {

using bf16 = __nv_bfloat16;

// Output tile of the convolution kernels: 2 (z) x 8 (y) x 16 (x) nodes, one 16-node
// x-row per MMA row block; 8 warps, two x-rows each.
constexpr int kTileZ = 2, kTileY = 8, kTileX = 16;
constexpr int kHaloZ = kTileZ + 2, kHaloY = kTileY + 2, kHaloX = kTileX + 2;
constexpr int kHaloNodes = kHaloZ * kHaloY * kHaloX;   // 720
constexpr int kRowHalfs = 24;                          // 16 channels + 8 pad (48 B, conflict-free ldmatrix)
constexpr int kThreads = 256;

// One sample of a step, as the kernels read it.
struct Sample {
    const float *velocity;     // [nz][ny][nx] nodal velocity (m/s)
    const float *travelTime;   // [nz][ny][nx] target travel times, or null
    double xs, ys, zs;         // source (m)
};

struct Geometry {
    int nx, ny, nz;
    double dx, dy, dz, x0, y0, z0;
    double invL;               // 1 / length of the grid's diagonal
};

// y[b][v][co] = act(bias[co] + sum_tap sum_ci x[b][v + off(tap)][ci] * w[tap][co][ci]),
// zero outside the grid; act = ReLU when relu, and y = 0 where mask[b][v][co] <= 0 when
// mask is given.  cin and cout multiples of 16.
struct ConvArgs {
    const bf16 *x;
    int cin;
    const bf16 *w;
    const float *bias;
    bf16 *y;
    int cout;
    const bf16 *mask;
    int relu;
    int D, H, W, B;
    int *status;        // raised (device) when a bounded wait of the tcgen05 path ran out; may be null
    long long spin;     // tcgen05 path: polls of an mbarrier before a wait gives up (<= 0: 2^24)
    int testLate;       // test hook, 0 in production (tcgen05 path, first input chunk): 1 = the
                        // operand barrier expects 16 bytes more than the copies bring, and those
                        // bytes are declared complete only after the wait ran out; 2 = the MMAs'
                        // completion is committed only after the wait ran out.  Either way the
                        // wait runs out while nothing is lost, and the recovery path runs.
};
// Grids with 128 nodes along x (and H % 4 == 0, D % 2 == 0) run on the tcgen05 tensor cores
// with TMEM accumulators; other shapes on mma.sync.
cudaError_t launchConv(const ConvArgs &a, cudaStream_t s);

// dw[tap][co][ci] += sum_b sum_v dy[b][v][co] * x[b][v + off(tap)][ci]  (FP32 atomics).
struct WGradArgs {
    const bf16 *x;
    int cin;
    const bf16 *dy;
    int cout;
    float *dw;
    int D, H, W, B;
};
cudaError_t launchWGrad(const WGradArgs &a, int numSMs, cudaStream_t s);

// db[c] += sum over nodes of dy[.][c].
cudaError_t launchBiasGrad(const bf16 *dy, int c, long long nodes, float *db, int numSMs, cudaStream_t s);

// 2x2x2 average pooling: x [B][D][H][W][C] -> y [B][D/2][H/2][W/2][C].
cudaError_t launchPool(const bf16 *x, int C, int D, int H, int W, int B, bf16 *y, cudaStream_t s);

// out[b][v] = concat(low[b][v/2][0:c1] (nearest upsampling), skip[b][v][0:c2]); D, H, W fine.
cudaError_t launchUpcat(const bf16 *low, int c1, const bf16 *skip, int c2, int D, int H, int W, int B,
                        bf16 *out, cudaStream_t s);

// Gradient of the upsampled part of a concatenation, gated by the low-resolution ReLU
// output: dpre[b][u][c] = (sum over the 8 children v of u of dcat[b][v][c]) if act > 0
// else 0, c < c1.  Dl, Hl, Wl: low-resolution extents.
cudaError_t launchUpSumMask(const bf16 *dcat, int ccat, const bf16 *act, int c1, int Dl, int Hl, int Wl, int B,
                            bf16 *dpre, cudaStream_t s);

// Gradient of an encoder output that feeds both a concatenation (channels c1..c1+c2 of
// dcat) and the next level's pooling (gradient dpool at the parent node):
// dpre = (dcat[v][c1 + c] + dpool[parent(v)][c] / 8) if skip[v][c] > 0 else 0.
cudaError_t launchCombineSkip(const bf16 *dcat, int ccat, int c1, const bf16 *dpool, const bf16 *skip, int c2,
                              int D, int H, int W, int B, bf16 *dpre, cudaStream_t s);

// Nodal slowness 1/v (FP32) of each sample: slow[b][v].  The per-node kernels below read it
// (and s_src = slow at the node nearest the source) instead of dividing again.
cudaError_t launchSlowness(const Sample *samples, Geometry g, int B, float *slow, cudaStream_t s);

// Input features [B][V][16] of the samples.
cudaError_t launchFeatures(const Sample *samples, const float *slow, Geometry g, int B, bf16 *feat, cudaStream_t s);

// Head (1x1x1 convolution of 16 channels) and loss: out = hb + hw . h; target
// tau - 1 = T / T0 - 1 from the sample's travel times, T0 = s_src |x - x_s| (FP32: the
// offsets from the source are FP64 differences rounded to FP32); accumulates the loss sum (double), the head's
// gradients (dhw: 16 weights then the bias) and writes dpre = dout * hw gated by h > 0.
// invN: 1 / the number of nodes with T0 > 0 over the samples.
cudaError_t launchHeadLoss(const bf16 *h, const float *hw, const Sample *samples, const float *slow, Geometry g,
                           int B, double invN, float *dhw, bf16 *dpre, double *lossSum, cudaStream_t s);

// Predicted travel times out[b][v] = T0 (1 + hb + hw . h) * inflate; also the loss sum
// when the samples carry travel times.
cudaError_t launchPredict(const bf16 *h, const float *hw, const Sample *samples, const float *slow, Geometry g, int B,
                          double inflate, float *out, double *lossSum, cudaStream_t s);

// Adam on n parameters; writes the BF16 copy pb.
cudaError_t launchAdam(float *p, const float *g, float *m, float *v, bf16 *pb, long long n, float lr, float b1,
                       float b2, float eps, float bc1, float bc2, cudaStream_t s);

// FP32 -> BF16 copy.
cudaError_t launchToBF16(const float *p, bf16 *pb, long long n, cudaStream_t s);

// Input-gradient weights: wt[tap][ci][co] = w[26 - tap][co][ci].
cudaError_t launchFlipTranspose(const bf16 *w, int cout, int cin, bf16 *wt, cudaStream_t s);

}  // namespace net
}  // namespace eikx
