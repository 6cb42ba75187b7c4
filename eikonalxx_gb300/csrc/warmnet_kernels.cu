// Kernels of the learned warm start's 3D U-Net (declared in warmnet.h).
//
// The 3x3x3 convolutions are implicit GEMMs on the BF16 tensor cores with FP32
// accumulation.  Levels whose x-rows hold 128 nodes run on tcgen05 (TMA staging, TMEM
// accumulators; convTcKernel below); the others on mma.sync m16n8k16:
//   * forward and input-gradient: M = output nodes (one 16-node x-row per MMA row block),
//     N = output channels, K = 27 taps x input channels.  A block stages a haloed
//     4 x 10 x 18-node tile of 16 input channels and the 27-tap weight slice of its
//     output channels in shared memory (cp.async, zero fill outside the grid); every
//     tap's A operand is an ldmatrix from the shifted halo, so each input value is read
//     from global memory once per block;
//   * weight gradient: M = output channels, N = 16 input channels, K = nodes; the A
//     operand (dy transposed) and the B operand (shifted input) come from the same two
//     tiles through ldmatrix.trans; each block loops over node tiles and adds its partial
//     sums to the FP32 gradient with one atomic per element at the end.
// Shared-memory rows are 48 bytes (an odd number of 16-byte segments), so the eight row
// addresses of every ldmatrix phase fall in distinct banks.
#include <cuda.h>
#include <cuda_bf16.h>

#include "warmnet.h"

namespace eikx {
namespace net {
namespace {

__device__ __forceinline__ unsigned smemAddr(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// 16-byte global -> shared copy; zero fill when !valid (src is then not read).
__device__ __forceinline__ void cpAsync16(void *dst, const void *src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smemAddr(dst)), "l"(src),
                 "r"(valid ? 16 : 0));
}
__device__ __forceinline__ void cpAsyncCommitWaitAll() {
    asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}


__device__ __forceinline__ void ldsm4(unsigned (&r)[4], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smemAddr(p)));
}
__device__ __forceinline__ void ldsm4t(unsigned (&r)[4], const void *p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smemAddr(p)));
}

__device__ __forceinline__ void mma16816(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

struct TileCoord {
    int gx0, gy0, gz0;
};
__device__ __forceinline__ TileCoord tileOf(int t, int D, int H, int W) {
    (void)D;
    const int tx = (W + kTileX - 1) / kTileX, ty = (H + kTileY - 1) / kTileY;
    TileCoord c;
    c.gx0 = (t % tx) * kTileX;
    t /= tx;
    c.gy0 = (t % ty) * kTileY;
    c.gz0 = (t / ty) * kTileZ;
    return c;
}
__host__ __device__ inline int tilesPerSample(int D, int H, int W) {
    return ((D + kTileZ - 1) / kTileZ) * ((H + kTileY - 1) / kTileY) * ((W + kTileX - 1) / kTileX);
}

// Stage 16 channels (ci0..ci0+15) of the haloed input tile: node (hz, hy, hx) of the
// halo at row (hz*kHaloY + hy)*kHaloX + hx, zero outside the grid.
__device__ __forceinline__ void stageHalo(bf16 *xs, const bf16 *xb, int cin, int ci0, TileCoord c, int D, int H,
                                          int W, const bf16 *anyValid) {
    for (int p = threadIdx.x; p < kHaloNodes * 2; p += kThreads) {
        const int hv = p >> 1, half = p & 1;
        const int hx = hv % kHaloX, hy = (hv / kHaloX) % kHaloY, hz = hv / (kHaloX * kHaloY);
        const int gx = c.gx0 - 1 + hx, gy = c.gy0 - 1 + hy, gz = c.gz0 - 1 + hz;
        const bool in = gx >= 0 && gx < W && gy >= 0 && gy < H && gz >= 0 && gz < D;
        const bf16 *src = in ? xb + ((static_cast<long long>(gz) * H + gy) * W + gx) * cin + ci0 + 8 * half : anyValid;
        cpAsync16(xs + hv * kRowHalfs + 8 * half, src, in);
    }
}

template <int NB>
__global__ void __launch_bounds__(kThreads) convKernel(ConvArgs a) {
    extern __shared__ __align__(16) unsigned char smemRaw[];
    bf16 *xs = reinterpret_cast<bf16 *>(smemRaw);
    bf16 *wsm = xs + kHaloNodes * kRowHalfs;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const TileCoord c = tileOf(blockIdx.x, a.D, a.H, a.W);
    const int b = blockIdx.z, co0 = blockIdx.y * NB;
    const long long V = static_cast<long long>(a.D) * a.H * a.W;
    const bf16 *xb = a.x + b * V * a.cin;

    float acc[2][NB / 8][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < NB / 8; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;

    const int li = lane >> 3, lj = lane & 7;
    for (int ci0 = 0; ci0 < a.cin; ci0 += 16) {
        stageHalo(xs, xb, a.cin, ci0, c, a.D, a.H, a.W, a.x);
        for (int p = threadIdx.x; p < 27 * NB * 2; p += kThreads) {
            const int row = p >> 1, half = p & 1;   // row = tap * NB + co
            const int tap = row / NB, co = row % NB;
            cpAsync16(wsm + row * kRowHalfs + 8 * half,
                      a.w + (static_cast<long long>(tap) * a.cout + co0 + co) * a.cin + ci0 + 8 * half, true);
        }
        cpAsyncCommitWaitAll();
        __syncthreads();
#pragma unroll 1
        for (int tap = 0; tap < 27; ++tap) {
            const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
            // B fragments: matrix li of ldmatrix.x4 = (channels 16p + 8*(li>>1) .. +7, k half li&1)
            unsigned bfr[NB / 16][4];
#pragma unroll
            for (int p = 0; p < NB / 16; ++p)
                ldsm4(bfr[p], wsm + (tap * NB + 16 * p + lj + 8 * (li >> 1)) * kRowHalfs + 8 * (li & 1));
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const int r = warp * 2 + mt, tz = r >> 3, ty = r & 7;
                // A fragment: matrix li = (nodes 8*(li&1) .. +7 of the x-row, k half li>>1)
                unsigned afr[4];
                ldsm4(afr, xs + (((tz + dz) * kHaloY + ty + dy) * kHaloX + lj + 8 * (li & 1) + dx) * kRowHalfs +
                               8 * (li >> 1));
#pragma unroll
                for (int nt = 0; nt < NB / 8; ++nt)
                    mma16816(acc[mt][nt], afr, bfr[nt >> 1][(nt & 1) * 2], bfr[nt >> 1][(nt & 1) * 2 + 1]);
            }
        }
        __syncthreads();
    }

    // Epilogue: accumulator (row lane/4 [+8], columns 2*(lane%4), +1) of each 16x8 block.
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        const int r = warp * 2 + mt;
        const int gz = c.gz0 + (r >> 3), gy = c.gy0 + (r & 7);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int gx = c.gx0 + (lane >> 2) + 8 * h;
            if (gz >= a.D || gy >= a.H || gx >= a.W) continue;
            const long long node = b * V + (static_cast<long long>(gz) * a.H + gy) * a.W + gx;
#pragma unroll
            for (int nt = 0; nt < NB / 8; ++nt) {
                const int co = co0 + 8 * nt + 2 * (lane & 3);
                float y0 = acc[mt][nt][2 * h], y1 = acc[mt][nt][2 * h + 1];
                if (a.bias) {
                    y0 += a.bias[co];
                    y1 += a.bias[co + 1];
                }
                if (a.relu) {
                    y0 = fmaxf(y0, 0.f);
                    y1 = fmaxf(y1, 0.f);
                }
                if (a.mask) {
                    const __nv_bfloat162 m = *reinterpret_cast<const __nv_bfloat162 *>(a.mask + node * a.cout + co);
                    if (!(__bfloat162float(m.x) > 0.f)) y0 = 0.f;
                    if (!(__bfloat162float(m.y) > 0.f)) y1 = 0.f;
                }
                *reinterpret_cast<__nv_bfloat162 *>(a.y + node * a.cout + co) = __floats2bfloat162_rn(y0, y1);
            }
        }
    }
}

// Weight gradient.  A warp owns one 16-channel block cb of dy and 4 consecutive taps:
// its 4 accumulators are 16 (co) x 16 (ci) blocks of dw that share the dy^T operand, so
// each 16-node row loads it once for 4 taps.  Warp w of block y is warp group
// g = y * 8 + w: cb = g / kTapGroups, taps 4 * (g % kTapGroups) + 0..3 (< 27).  grid.z
// walks the 16-channel input chunks, grid.x strides over the node tiles of all samples.
constexpr int kUnitsPerWarp = 4;
constexpr int kTapGroups = (27 + kUnitsPerWarp - 1) / kUnitsPerWarp;   // 7
__global__ void __launch_bounds__(kThreads) wgradKernel(WGradArgs a) {
    extern __shared__ __align__(16) unsigned char smemRaw[];
    bf16 *xs = reinterpret_cast<bf16 *>(smemRaw);
    bf16 *dys = xs + kHaloNodes * kRowHalfs;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int li = lane >> 3, lj = lane & 7;
    const int ci0 = blockIdx.z * 16;
    const int group = blockIdx.y * (kThreads / 32) + warp;
    const int cb = group / kTapGroups, tap0 = kUnitsPerWarp * (group % kTapGroups);
    const bool warpActive = cb < a.cout / 16;
    const int dyRow = a.cout + 8;   // halfs; an odd number of 16-byte segments
    const long long V = static_cast<long long>(a.D) * a.H * a.W;
    const int tps = tilesPerSample(a.D, a.H, a.W);
    const int nTiles = tps * a.B;

    float acc[kUnitsPerWarp][2][4];
#pragma unroll
    for (int i = 0; i < kUnitsPerWarp; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;

    for (int t = blockIdx.x; t < nTiles; t += gridDim.x) {
        const int b = t / tps;
        const TileCoord c = tileOf(t % tps, a.D, a.H, a.W);
        stageHalo(xs, a.x + b * V * a.cin, a.cin, ci0, c, a.D, a.H, a.W, a.x);
        const int pieces = a.cout / 8;
        for (int p = threadIdx.x; p < 256 * pieces; p += kThreads) {
            const int node = p / pieces, piece = p % pieces;
            const int r = node >> 4, xx = node & 15;
            const int gz = c.gz0 + (r >> 3), gy = c.gy0 + (r & 7), gx = c.gx0 + xx;
            const bool in = gz < a.D && gy < a.H && gx < a.W;
            const bf16 *src =
                in ? a.dy + (b * V + (static_cast<long long>(gz) * a.H + gy) * a.W + gx) * a.cout + 8 * piece : a.dy;
            cpAsync16(dys + node * dyRow + 8 * piece, src, in);
        }
        cpAsyncCommitWaitAll();
        __syncthreads();
        if (warpActive) {
#pragma unroll 2
            for (int r = 0; r < 16; ++r) {
                const int tz = r >> 3, ty = r & 7;
                // A = dy^T: matrix li = (co 16cb + 8*(li&1) .., nodes 16r + 8*(li>>1) ..)
                unsigned afr[4];
                ldsm4t(afr, dys + (16 * r + lj + 8 * (li >> 1)) * dyRow + 16 * cb + 8 * (li & 1));
#pragma unroll
                for (int kk = 0; kk < kUnitsPerWarp; ++kk) {
                    const int tap = tap0 + kk;
                    if (tap >= 27) continue;
                    const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
                    // B = shifted input: matrix li = (nodes 8*(li&1) .., channels 8*(li>>1) ..)
                    unsigned bfr[4];
                    ldsm4t(bfr, xs + (((tz + dz) * kHaloY + ty + dy) * kHaloX + lj + 8 * (li & 1) + dx) * kRowHalfs +
                                    8 * (li >> 1));
                    mma16816(acc[kk][0], afr, bfr[0], bfr[1]);
                    mma16816(acc[kk][1], afr, bfr[2], bfr[3]);
                }
            }
        }
        __syncthreads();
    }
    if (!warpActive) return;
#pragma unroll
    for (int kk = 0; kk < kUnitsPerWarp; ++kk) {
        const int tap = tap0 + kk;
        if (tap >= 27) continue;
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
            const int ci = ci0 + 8 * nt + 2 * (lane & 3);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int co = 16 * cb + (lane >> 2) + 8 * h;
                float *d = a.dw + (static_cast<long long>(tap) * a.cout + co) * a.cin + ci;
                atomicAdd(d, acc[kk][nt][2 * h]);
                atomicAdd(d + 1, acc[kk][nt][2 * h + 1]);
            }
        }
    }
}

__global__ void biasGradKernel(const bf16 *dy, int C, long long nodes, float *db) {
    __shared__ float part[kThreads];
    const int c = threadIdx.x % C, slot = threadIdx.x / C, slots = kThreads / C;
    float s = 0.f;
    for (long long v = static_cast<long long>(blockIdx.x) * slots + slot; v < nodes;
         v += static_cast<long long>(gridDim.x) * slots)
        s += __bfloat162float(dy[v * C + c]);
    part[threadIdx.x] = s;
    __syncthreads();
    if (slot == 0) {
        for (int k = 1; k < slots; ++k) s += part[k * C + c];
        atomicAdd(db + c, s);
    }
}

struct alignas(16) Vec8 {
    __nv_bfloat162 h[4];
};
__device__ __forceinline__ void load8(float (&f)[8], const bf16 *p) {
    const Vec8 v = *reinterpret_cast<const Vec8 *>(p);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        f[2 * i] = __bfloat162float(v.h[i].x);
        f[2 * i + 1] = __bfloat162float(v.h[i].y);
    }
}
__device__ __forceinline__ void store8(bf16 *p, const float (&f)[8]) {
    Vec8 v;
#pragma unroll
    for (int i = 0; i < 4; ++i) v.h[i] = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
    *reinterpret_cast<Vec8 *>(p) = v;
}

__global__ void poolKernel(const bf16 *x, int C, int D, int H, int W, int B, bf16 *y) {
    const int Dl = D / 2, Hl = H / 2, Wl = W / 2, groups = C / 8;
    const long long total = static_cast<long long>(B) * Dl * Hl * Wl * groups;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int g = i % groups;
        long long u = i / groups;
        const int ux = u % Wl, uy = (u / Wl) % Hl, uz = (u / (static_cast<long long>(Wl) * Hl)) % Dl;
        const long long b = u / (static_cast<long long>(Wl) * Hl * Dl);
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int k = 0; k < 8; ++k) {
            const int z = 2 * uz + (k >> 2), yy = 2 * uy + ((k >> 1) & 1), xx = 2 * ux + (k & 1);
            float f[8];
            load8(f, x + ((b * D + z) * H * static_cast<long long>(W) + static_cast<long long>(yy) * W + xx) * C + 8 * g);
#pragma unroll
            for (int j = 0; j < 8; ++j) s[j] += f[j];
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) s[j] *= 0.125f;
        store8(y + u * C + 8 * g, s);
    }
}

__global__ void upcatKernel(const bf16 *low, int c1, const bf16 *skip, int c2, int D, int H, int W, int B,
                            bf16 *out) {
    const int C = c1 + c2, groups = C / 8;
    const long long total = static_cast<long long>(B) * D * H * W * groups;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int g = i % groups;
        const long long v = i / groups;
        const int x = v % W, y = (v / W) % H, z = (v / (static_cast<long long>(W) * H)) % D;
        const long long b = v / (static_cast<long long>(W) * H * D);
        const bf16 *src;
        if (8 * g < c1) {
            const long long u = ((b * (D / 2) + z / 2) * (H / 2) + y / 2) * (W / 2) + x / 2;
            src = low + u * c1 + 8 * g;
        } else {
            src = skip + v * c2 + 8 * g - c1;
        }
        *reinterpret_cast<Vec8 *>(out + v * C + 8 * g) = *reinterpret_cast<const Vec8 *>(src);
    }
}

__global__ void upSumMaskKernel(const bf16 *dcat, int ccat, const bf16 *act, int c1, int Dl, int Hl, int Wl, int B,
                                bf16 *dpre) {
    const int groups = c1 / 8, D = 2 * Dl, H = 2 * Hl, W = 2 * Wl;
    const long long total = static_cast<long long>(B) * Dl * Hl * Wl * groups;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int g = i % groups;
        const long long u = i / groups;
        const int ux = u % Wl, uy = (u / Wl) % Hl, uz = (u / (static_cast<long long>(Wl) * Hl)) % Dl;
        const long long b = u / (static_cast<long long>(Wl) * Hl * Dl);
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int k = 0; k < 8; ++k) {
            const int z = 2 * uz + (k >> 2), yy = 2 * uy + ((k >> 1) & 1), xx = 2 * ux + (k & 1);
            float f[8];
            load8(f, dcat + ((b * D + z) * H * static_cast<long long>(W) + static_cast<long long>(yy) * W + xx) * ccat +
                         8 * g);
#pragma unroll
            for (int j = 0; j < 8; ++j) s[j] += f[j];
        }
        float m[8];
        load8(m, act + u * c1 + 8 * g);
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (!(m[j] > 0.f)) s[j] = 0.f;
        store8(dpre + u * c1 + 8 * g, s);
    }
}

__global__ void combineSkipKernel(const bf16 *dcat, int ccat, int c1, const bf16 *dpool, const bf16 *skip, int c2,
                                  int D, int H, int W, int B, bf16 *dpre) {
    const int groups = c2 / 8;
    const long long total = static_cast<long long>(B) * D * H * W * groups;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int g = i % groups;
        const long long v = i / groups;
        const int x = v % W, y = (v / W) % H, z = (v / (static_cast<long long>(W) * H)) % D;
        const long long b = v / (static_cast<long long>(W) * H * D);
        const long long u = ((b * (D / 2) + z / 2) * (H / 2) + y / 2) * (W / 2) + x / 2;
        float a[8], p[8], m[8];
        load8(a, dcat + v * ccat + c1 + 8 * g);
        load8(p, dpool + u * c2 + 8 * g);
        load8(m, skip + v * c2 + 8 * g);
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = (m[j] > 0.f) ? a[j] + 0.125f * p[j] : 0.f;
        store8(dpre + v * c2 + 8 * g, a);
    }
}

// Per-node geometry, FP32: the offsets from the source are FP64 differences rounded to
// FP32, the distance an FP32 square root; s_src is the slowness at the node nearest the
// source.
__device__ __forceinline__ long long nearestNode(const Sample &s, const Geometry &g) {
    const int ix = min(g.nx - 1, max(0, __double2int_rn((s.xs - g.x0) / g.dx)));
    const int iy = min(g.ny - 1, max(0, __double2int_rn((s.ys - g.y0) / g.dy)));
    const int iz = min(g.nz - 1, max(0, __double2int_rn((s.zs - g.z0) / g.dz)));
    return (static_cast<long long>(iz) * g.ny + iy) * g.nx + ix;
}
struct NodeGeom {
    float ddx, ddy, ddz, dist;
};
__device__ __forceinline__ NodeGeom nodeGeom(long long v, const Sample &s, const Geometry &g) {
    const int x = v % g.nx, y = (v / g.nx) % g.ny, z = v / (static_cast<long long>(g.nx) * g.ny);
    NodeGeom n;
    n.ddx = static_cast<float>((g.x0 + x * g.dx) - s.xs);
    n.ddy = static_cast<float>((g.y0 + y * g.dy) - s.ys);
    n.ddz = static_cast<float>((g.z0 + z * g.dz) - s.zs);
    n.dist = sqrtf(n.ddx * n.ddx + n.ddy * n.ddy + n.ddz * n.ddz);
    return n;
}

__global__ void slownessKernel(const Sample *samples, Geometry g, int B, float *slow) {
    const long long V = static_cast<long long>(g.nx) * g.ny * g.nz;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < B * V;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        slow[i] = 1.f / samples[i / V].velocity[i % V];
}

// Straight-ray estimate of tau - 1 at node (x, y, z): the mean of s/s_src - 1 over
// kRaySamples midpoints of the segment from the source to the node, the slowness
// trilinear in the nodal 1/v.  FP32, in an operation order the oracle repeats.
constexpr int kRaySamples = 32;
__device__ float straightRayContrast(const Sample &s, const float *sl, const Geometry &g, float sSrc, int x, int y,
                                     int z) {
    auto at = [&](int ix, int iy, int iz) { return sl[(static_cast<long long>(iz) * g.ny + iy) * g.nx + ix]; };
    const float sx = static_cast<float>((s.xs - g.x0) / g.dx), sy = static_cast<float>((s.ys - g.y0) / g.dy),
                sz = static_cast<float>((s.zs - g.z0) / g.dz);
    const float ex = static_cast<float>(x) - sx, ey = static_cast<float>(y) - sy, ez = static_cast<float>(z) - sz;
    float acc = 0.f;
    for (int k = 0; k < kRaySamples; ++k) {
        const float t = (static_cast<float>(k) + 0.5f) / static_cast<float>(kRaySamples);
        const float px = fminf(fmaxf(sx + t * ex, 0.f), static_cast<float>(g.nx - 1));
        const float py = fminf(fmaxf(sy + t * ey, 0.f), static_cast<float>(g.ny - 1));
        const float pz = fminf(fmaxf(sz + t * ez, 0.f), static_cast<float>(g.nz - 1));
        const int ix = min(static_cast<int>(floorf(px)), g.nx - 2), iy = min(static_cast<int>(floorf(py)), g.ny - 2),
                  iz = min(static_cast<int>(floorf(pz)), g.nz - 2);
        const float fx = px - static_cast<float>(ix), fy = py - static_cast<float>(iy), fz = pz - static_cast<float>(iz);
        const float s000 = at(ix, iy, iz), s100 = at(ix + 1, iy, iz);
        const float s010 = at(ix, iy + 1, iz), s110 = at(ix + 1, iy + 1, iz);
        const float s001 = at(ix, iy, iz + 1), s101 = at(ix + 1, iy, iz + 1);
        const float s011 = at(ix, iy + 1, iz + 1), s111 = at(ix + 1, iy + 1, iz + 1);
        const float c00 = s000 + fx * (s100 - s000), c10 = s010 + fx * (s110 - s010);
        const float c01 = s001 + fx * (s101 - s001), c11 = s011 + fx * (s111 - s011);
        const float c0 = c00 + fy * (c10 - c00), c1 = c01 + fy * (c11 - c01);
        const float c = c0 + fz * (c1 - c0);
        acc += c / sSrc - 1.f;
    }
    return acc / static_cast<float>(kRaySamples);
}

__global__ void featuresKernel(const Sample *samples, const float *slow, Geometry g, int B, bf16 *feat) {
    const long long V = static_cast<long long>(g.nx) * g.ny * g.nz;
    const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (i >= B * V) return;
    const int b = i / V;
    const long long v = i % V;
    const Sample s = samples[b];
    const float *sl = slow + b * V;
    const float sSrc = sl[nearestNode(s, g)];
    const NodeGeom n = nodeGeom(v, s, g);
    const float invL = static_cast<float>(g.invL);
    float f[8] = {sl[v] / sSrc - 1.f,
                  n.dist * invL,
                  n.ddx * invL,
                  n.ddy * invL,
                  n.ddz * invL,
                  straightRayContrast(s, sl, g, sSrc, static_cast<int>(v % g.nx), static_cast<int>((v / g.nx) % g.ny),
                                      static_cast<int>(v / (static_cast<long long>(g.nx) * g.ny))),
                  0.f,
                  0.f};
    store8(feat + i * 16, f);
    const float z[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    store8(feat + i * 16 + 8, z);
}

__device__ __forceinline__ float warpSum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warpSumD(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float headOut(const float (&h)[16], const float *hw) {
    float o = hw[16];
    for (int c = 0; c < 16; ++c) o += hw[c] * h[c];
    return o;
}

__global__ void __launch_bounds__(kThreads) headLossKernel(const bf16 *h, const float *hw, const Sample *samples,
                                                           const float *slow, Geometry g, int B, double invN,
                                                           float *dhw, bf16 *dpre, double *lossSum) {
    __shared__ float red[kThreads / 32][17];
    __shared__ double redL[kThreads / 32];
    const long long V = static_cast<long long>(g.nx) * g.ny * g.nz;
    const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    float hv[16];
    float dout = 0.f;
    double l = 0.0;
    if (i < B * V) {
        const int b = i / V;
        const long long v = i % V;
        const Sample s = samples[b];
        float a[8], c[8];
        load8(a, h + i * 16);
        load8(c, h + i * 16 + 8);
        for (int k = 0; k < 8; ++k) {
            hv[k] = a[k];
            hv[8 + k] = c[k];
        }
        const float o = headOut(hv, hw);
        const float T0 = slow[b * V + nearestNode(s, g)] * nodeGeom(v, s, g).dist;
        if (T0 > 0.f) {
            const float tgt = s.travelTime[v] / T0 - 1.f;
            const float diff = o - tgt;
            l = static_cast<double>(diff) * diff;
            dout = static_cast<float>(2.0 * diff * invN);
        }
        float d[8], e[8];
        for (int k = 0; k < 8; ++k) {
            d[k] = hv[k] > 0.f ? dout * hw[k] : 0.f;
            e[k] = hv[8 + k] > 0.f ? dout * hw[8 + k] : 0.f;
        }
        store8(dpre + i * 16, d);
        store8(dpre + i * 16 + 8, e);
    } else {
        for (int k = 0; k < 16; ++k) hv[k] = 0.f;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = 0; k < 16; ++k) {
        const float t = warpSum(dout * hv[k]);
        if (lane == 0) red[warp][k] = t;
    }
    const float tb = warpSum(dout);
    const double tl = warpSumD(l);
    if (lane == 0) {
        red[warp][16] = tb;
        redL[warp] = tl;
    }
    __syncthreads();
    if (threadIdx.x < 17) {
        float s = 0.f;
        for (int w = 0; w < kThreads / 32; ++w) s += red[w][threadIdx.x];
        atomicAdd(dhw + threadIdx.x, s);
    } else if (threadIdx.x == 32) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += redL[w];
        atomicAdd(lossSum, s);
    }
}

__global__ void __launch_bounds__(kThreads) predictKernel(const bf16 *h, const float *hw, const Sample *samples,
                                                          const float *slow, Geometry g, int B, float inflate,
                                                          float *out, double *lossSum) {
    __shared__ double redL[kThreads / 32];
    const long long V = static_cast<long long>(g.nx) * g.ny * g.nz;
    const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    double l = 0.0;
    if (i < B * V) {
        const int b = i / V;
        const long long v = i % V;
        const Sample s = samples[b];
        float a[8], c[8], hv[16];
        load8(a, h + i * 16);
        load8(c, h + i * 16 + 8);
        for (int k = 0; k < 8; ++k) {
            hv[k] = a[k];
            hv[8 + k] = c[k];
        }
        const float o = headOut(hv, hw);
        const float T0 = slow[b * V + nearestNode(s, g)] * nodeGeom(v, s, g).dist;
        out[i] = T0 * (1.f + o) * inflate;
        if (lossSum && s.travelTime && T0 > 0.f) {
            const float diff = o - (s.travelTime[v] / T0 - 1.f);
            l = static_cast<double>(diff) * diff;
        }
    }
    if (!lossSum) return;
    const double t = warpSumD(l);
    if ((threadIdx.x & 31) == 0) redL[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) s += redL[w];
        atomicAdd(lossSum, s);
    }
}

__global__ void adamKernel(float *p, const float *g, float *m, float *v, bf16 *pb, long long n, float lr, float b1,
                           float b2, float eps, float bc1, float bc2) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float pi = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        p[i] = pi;
        pb[i] = __float2bfloat16_rn(pi);
    }
}

__global__ void toBF16Kernel(const float *p, bf16 *pb, long long n) {
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        pb[i] = __float2bfloat16_rn(p[i]);
}

__global__ void flipTransposeKernel(const bf16 *w, int cout, int cin, bf16 *wt) {
    const long long n = 27LL * cout * cin;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int co = i % cout;
        const int ci = (i / cout) % cin;
        const int tap = i / (static_cast<long long>(cout) * cin);
        wt[i] = w[(static_cast<long long>(26 - tap) * cout + co) * cin + ci];
    }
}

// ---- tcgen05 convolution for x-rows of 128 nodes ------------------------------------------
// A block computes 8 output x-rows (4 along y, 2 along z), each a full row of 128 nodes, for
// N output channels.  Each row accumulates in its own TMEM region (128 lanes = the row's
// nodes, N FP32 columns).  Per 16-channel input chunk, one thread stages with TMA
// (cp.async.bulk.tensor, zero fill outside the grid):
//   * the 6 x 4 haloed input rows of 130 nodes, one box per 8-channel group: in shared memory
//     [group][row][node][8 channels], so a node's 8 channels are one 16-byte row of a core
//     matrix and node r + dx starts 16 * dx bytes later;
//   * the 27-tap weight slice, one box per group: [group][tap][channel out][8 channels in].
// Both are the no-swizzle K-major canonical layout (K-direction core matrices one group
// apart, 8-row core matrices 128 bytes apart).  The same thread then issues 8 rows x 27 taps
// MMAs (M = 128 nodes, N channels, K = 16): every tap's A operand is the staged row, shifted.
// mbarriers (bounded waits) signal the TMA bytes' arrival and the MMAs' completion; the
// epilogue reads TMEM with tcgen05.ld (warp w: lanes 32w..32w+31).
namespace tc {
constexpr int kRY = 4, kRZ = 2, kRows = kRY * kRZ;
constexpr int kHY = kRY + 2, kHZ = kRZ + 2, kHaloRows = kHY * kHZ;
constexpr int kXN = 130;                          // a 128-node row with its two halo nodes
constexpr int kRowB = kXN * 16;                   // one staged row of one 8-channel group (bytes)
constexpr int kGroupB = kHaloRows * kRowB;        // one group of the halo: 49,920
constexpr int kHaloB = 2 * kGroupB;               // 99,840
constexpr long long kSpin = 1ll << 24;

__device__ __forceinline__ unsigned long long sdesc(unsigned addr, unsigned lbo, unsigned sbo) {
    // start address, leading (K-direction core-matrix) and stride (8-row) byte offsets, all
    // in 16-byte units; bit 46: descriptor version of tcgen05; no swizzle
    return static_cast<unsigned long long>((addr >> 4) & 0x3FFF) |
           (static_cast<unsigned long long>((lbo >> 4) & 0x3FFF) << 16) |
           (static_cast<unsigned long long>((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}
__device__ __forceinline__ void mma(unsigned d, unsigned long long ad, unsigned long long bd, unsigned idesc,
                                    unsigned accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ bool waitParity(unsigned mbar, unsigned parity, long long spin) {
    unsigned done = 0;
    for (long long it = 0; it < spin && !done; ++it)
        asm volatile(
            "{\n .reg .pred q;\n mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n selp.u32 %0, 1, 0, q;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
    return done != 0;
}
__device__ __forceinline__ void fenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tma5(unsigned dst, const CUtensorMap *map, int c0, int c1, int c2, int c3, int c4,
                                     unsigned mbar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
        "%6}], [%7];" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(mbar)
        : "memory");
}
__device__ __forceinline__ void tma3(unsigned dst, const CUtensorMap *map, int c0, int c1, int c2, unsigned mbar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(mbar)
        : "memory");
}

template <int N> __host__ __device__ constexpr int colStride() { return N <= 32 ? 32 : 64; }
template <int N> __host__ __device__ constexpr int weightGroupB() { return 27 * N * 16; }
template <int N> __host__ __device__ constexpr int smemBytes() { return kHaloB + 2 * weightGroupB<N>() + 32; }

template <int N>
__global__ void __launch_bounds__(128) convTcKernel(ConvArgs a, const __grid_constant__ CUtensorMap mapX,
                                                    const __grid_constant__ CUtensorMap mapW) {
    constexpr int CS = colStride<N>(), NCOL = kRows * CS, WG = weightGroupB<N>();
    static_assert(N % 16 == 0 && N <= 64 && (NCOL & (NCOL - 1)) == 0 && NCOL <= 512, "TMEM layout");
    extern __shared__ __align__(1024) unsigned char smemRaw[];
    unsigned char *halo = smemRaw;                 // [2 groups][24 rows][130 nodes][16 B]
    unsigned char *wsm = smemRaw + kHaloB;         // [2 groups][27 taps][N][16 B]
    unsigned long long *full = reinterpret_cast<unsigned long long *>(wsm + 2 * WG);
    unsigned long long *mmaDone = full + 1;
    unsigned *tslot = reinterpret_cast<unsigned *>(full + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tilesY = a.H / kRY;
    const int z0 = (blockIdx.x / tilesY) * kRZ, y0 = (blockIdx.x % tilesY) * kRY;
    const int b = blockIdx.z, co0 = blockIdx.y * N;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(tslot)),
                     "r"(NCOL)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smemAddr(full)) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smemAddr(mmaDone)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fenceBefore();
    __syncthreads();
    fenceAfter();
    const unsigned tmem = *tslot;
    // kind::f16: D FP32 (bit 4), A and B BF16 (bits 7, 10), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
    const unsigned idesc = (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<unsigned>(N >> 3) << 17) | ((128u >> 4) << 24);
    const unsigned hb = smemAddr(halo), wb = smemAddr(wsm);
    const long long spin = a.spin > 0 ? a.spin : kSpin;
    // A wait that runs out must not leave the CTA while its copies or MMAs may still write
    // its shared memory or TMEM: before it leaves, the CTA drains -- it waits again on the
    // same barrier phase with a bound kDrain times as long -- and only then frees TMEM.
    constexpr long long kDrain = 64;
    bool ok = true;
    int chunk = 0;
    for (int ci0 = 0; ci0 < a.cin; ci0 += 16, ++chunk) {
        const bool lateTx = a.testLate == 1 && chunk == 0, lateCommit = a.testLate == 2 && chunk == 0;
        if (tid == 0) {
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(full)),
                         "r"(static_cast<unsigned>(kHaloB + 2 * WG + (lateTx ? 16 : 0)))
                         : "memory");
            for (int g = 0; g < 2; ++g) {
                tma5(hb + g * kGroupB, &mapX, ci0 + 8 * g, -1, y0 - 1, z0 - 1, b, smemAddr(full));
                tma3(wb + g * WG, &mapW, ci0 + 8 * g, co0, 0, smemAddr(full));
            }
        }
        const bool landed = waitParity(smemAddr(full), static_cast<unsigned>(chunk & 1), spin);
        if (!__syncthreads_and(landed)) {
            // drain: the copies of this chunk land before the CTA leaves (the test hook's
            // extra bytes are declared complete here, as late bytes would arrive)
            if (tid == 0 && lateTx)
                asm volatile("mbarrier.complete_tx.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(full)), "r"(16u)
                             : "memory");
            waitParity(smemAddr(full), static_cast<unsigned>(chunk & 1), kDrain * spin);
            __syncthreads();
            ok = false;
            break;
        }
        if (tid == 0) {
            for (int rr = 0; rr < kRows; ++rr) {
                const int oz = rr / kRY, oy = rr % kRY;
                for (int tap = 0; tap < 27; ++tap) {
                    const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
                    const int hr = (oz + dz) * kHY + oy + dy;
                    mma(tmem + static_cast<unsigned>(rr * CS),
                        sdesc(hb + static_cast<unsigned>(hr * kRowB + dx * 16), kGroupB, 128),
                        sdesc(wb + static_cast<unsigned>(tap * N * 16), WG, 128), idesc,
                        (ci0 > 0 || tap > 0) ? 1u : 0u);
                }
            }
            if (!lateCommit)
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smemAddr(mmaDone))
                             : "memory");
        }
        // this chunk's MMAs have read the buffers once the barrier's phase completes
        const bool done = waitParity(smemAddr(mmaDone), static_cast<unsigned>(chunk & 1), spin);
        ok = __syncthreads_and(done) != 0;
        if (!ok) {
            // drain: the MMAs issued for this chunk complete before TMEM is freed (the test
            // hook commits their completion only now, as a late completion would arrive)
            if (tid == 0 && lateCommit)
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smemAddr(mmaDone))
                             : "memory");
            waitParity(smemAddr(mmaDone), static_cast<unsigned>(chunk & 1), kDrain * spin);
            __syncthreads();
        }
        fenceAfter();
        if (!ok) break;
    }
    if (ok) {
        const int x = warp * 32 + lane;
        for (int rr = 0; rr < kRows; ++rr) {
            const int gz = z0 + rr / kRY, gy = y0 + rr % kRY;
            const long long node = ((static_cast<long long>(b) * a.D + gz) * a.H + gy) * 128 + x;
#pragma unroll
            for (int c0 = 0; c0 < N; c0 += 16) {
                unsigned r[16];
                const unsigned addr = tmem + ((static_cast<unsigned>(warp) * 32u) << 16) + static_cast<unsigned>(rr * CS + c0);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                      "=r"(r[15])
                    : "r"(addr)
                    : "memory");
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                float v[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    v[j] = __uint_as_float(r[j]);
                    if (a.bias) v[j] += a.bias[co0 + c0 + j];
                    if (a.relu) v[j] = fmaxf(v[j], 0.f);
                }
                bf16 *dst = a.y + node * a.cout + co0 + c0;
                if (a.mask) {
                    float m0[8], m1[8];
                    load8(m0, a.mask + node * a.cout + co0 + c0);
                    load8(m1, a.mask + node * a.cout + co0 + c0 + 8);
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        if (!(m0[j] > 0.f)) v[j] = 0.f;
                        if (!(m1[j] > 0.f)) v[8 + j] = 0.f;
                    }
                }
                float lo[8], hi[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    lo[j] = v[j];
                    hi[j] = v[8 + j];
                }
                store8(dst, lo);
                store8(dst + 8, hi);
            }
        }
    } else if (tid == 0 && a.status) {
        atomicExch(a.status, 1);
    }
    fenceBefore();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOL) : "memory");
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled encodeTiled() {
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

template <int N>
cudaError_t launchTc(const ConvArgs &a, cudaStream_t s) {
    EncodeTiled enc = encodeTiled();
    if (!enc) return cudaErrorNotSupported;
    // activations [B][D][H][128][cin] BF16: box of 8 channels x 130 nodes x 6 rows x 4 planes x 1 sample
    CUtensorMap mapX, mapW;
    const cuuint64_t dimX[5] = {static_cast<cuuint64_t>(a.cin), 128, static_cast<cuuint64_t>(a.H),
                                static_cast<cuuint64_t>(a.D), static_cast<cuuint64_t>(a.B)};
    const cuuint64_t strideX[4] = {static_cast<cuuint64_t>(a.cin) * 2, 128ull * a.cin * 2,
                                   static_cast<cuuint64_t>(a.H) * 128 * a.cin * 2,
                                   static_cast<cuuint64_t>(a.D) * a.H * 128 * a.cin * 2};
    const cuuint32_t boxX[5] = {8, kXN, kHY, kHZ, 1}, ones[5] = {1, 1, 1, 1, 1};
    if (enc(&mapX, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(a.x), dimX, strideX, boxX, ones,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    // weights [27][cout][cin] BF16: box of 8 channels in x N channels out x 27 taps
    const cuuint64_t dimW[3] = {static_cast<cuuint64_t>(a.cin), static_cast<cuuint64_t>(a.cout), 27};
    const cuuint64_t strideW[2] = {static_cast<cuuint64_t>(a.cin) * 2, static_cast<cuuint64_t>(a.cout) * a.cin * 2};
    const cuuint32_t boxW[3] = {8, static_cast<cuuint32_t>(N), 27};
    if (enc(&mapW, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<bf16 *>(a.w), dimW, strideW, boxW, ones,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    // the shared-memory limit is a per-device attribute: set it for the current device
    cudaError_t e = cudaFuncSetAttribute(convTcKernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, smemBytes<N>());
    if (e != cudaSuccess) return e;
    dim3 grid((a.D / kRZ) * (a.H / kRY), a.cout / N, a.B);
    convTcKernel<N><<<grid, 128, smemBytes<N>(), s>>>(a, mapX, mapW);
    return cudaGetLastError();
}
}  // namespace tc

int gridFor(long long n, int cap = 1 << 20) {
    long long b = (n + kThreads - 1) / kThreads;
    if (b < 1) b = 1;
    return static_cast<int>(b < cap ? b : cap);
}

template <int NB>
cudaError_t convOne(const ConvArgs &a, cudaStream_t s) {
    const int smem = (kHaloNodes + 27 * NB) * kRowHalfs * static_cast<int>(sizeof(bf16));
    // the shared-memory limit is a per-device attribute: set it for the current device
    cudaError_t e = cudaFuncSetAttribute(convKernel<NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    dim3 grid(tilesPerSample(a.D, a.H, a.W), a.cout / NB, a.B);
    convKernel<NB><<<grid, kThreads, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launchConv(const ConvArgs &a, cudaStream_t s) {
    if (a.cin % 16 || a.cout % 16 || a.B < 1) return cudaErrorInvalidValue;
    if (a.W == 128 && a.H % tc::kRY == 0 && a.D % tc::kRZ == 0) {
        switch (a.cout) {
            case 16: return tc::launchTc<16>(a, s);
            case 32: return tc::launchTc<32>(a, s);
            case 48: return tc::launchTc<48>(a, s);
            default:
                if (a.cout % 64 == 0) return tc::launchTc<64>(a, s);
                if (a.cout % 32 == 0) return tc::launchTc<32>(a, s);
                return tc::launchTc<16>(a, s);
        }
    }
    return a.cout % 32 == 0 ? convOne<32>(a, s) : convOne<16>(a, s);
}

cudaError_t launchWGrad(const WGradArgs &a, int numSMs, cudaStream_t s) {
    if (a.cin % 16 || a.cout % 16 || a.B < 1) return cudaErrorInvalidValue;
    const int smem = (kHaloNodes * kRowHalfs + 256 * (a.cout + 8)) * static_cast<int>(sizeof(bf16));
    // the shared-memory limit is a per-device attribute: set it for the current device
    cudaError_t e = cudaFuncSetAttribute(wgradKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const int warpsPerBlock = kThreads / 32;
    const int gy = (kTapGroups * (a.cout / 16) + warpsPerBlock - 1) / warpsPerBlock, gz = a.cin / 16;
    const int nTiles = tilesPerSample(a.D, a.H, a.W) * a.B;
    int gx = (4 * numSMs + gy * gz - 1) / (gy * gz);
    gx = gx < 1 ? 1 : (gx > nTiles ? nTiles : gx);
    wgradKernel<<<dim3(gx, gy, gz), kThreads, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launchBiasGrad(const bf16 *dy, int c, long long nodes, float *db, int numSMs, cudaStream_t s) {
    if (c < 1 || c > kThreads || kThreads % c) return cudaErrorInvalidValue;
    const long long slots = kThreads / c;
    long long blocks = (nodes + slots * 64 - 1) / (slots * 64);
    if (blocks > 4LL * numSMs) blocks = 4LL * numSMs;
    if (blocks < 1) blocks = 1;
    biasGradKernel<<<static_cast<int>(blocks), kThreads, 0, s>>>(dy, c, nodes, db);
    return cudaGetLastError();
}

cudaError_t launchPool(const bf16 *x, int C, int D, int H, int W, int B, bf16 *y, cudaStream_t s) {
    poolKernel<<<gridFor(static_cast<long long>(B) * (D / 2) * (H / 2) * (W / 2) * (C / 8)), kThreads, 0, s>>>(
        x, C, D, H, W, B, y);
    return cudaGetLastError();
}

cudaError_t launchUpcat(const bf16 *low, int c1, const bf16 *skip, int c2, int D, int H, int W, int B, bf16 *out,
                        cudaStream_t s) {
    upcatKernel<<<gridFor(static_cast<long long>(B) * D * H * W * ((c1 + c2) / 8)), kThreads, 0, s>>>(
        low, c1, skip, c2, D, H, W, B, out);
    return cudaGetLastError();
}

cudaError_t launchUpSumMask(const bf16 *dcat, int ccat, const bf16 *act, int c1, int Dl, int Hl, int Wl, int B,
                            bf16 *dpre, cudaStream_t s) {
    upSumMaskKernel<<<gridFor(static_cast<long long>(B) * Dl * Hl * Wl * (c1 / 8)), kThreads, 0, s>>>(
        dcat, ccat, act, c1, Dl, Hl, Wl, B, dpre);
    return cudaGetLastError();
}

cudaError_t launchCombineSkip(const bf16 *dcat, int ccat, int c1, const bf16 *dpool, const bf16 *skip, int c2,
                              int D, int H, int W, int B, bf16 *dpre, cudaStream_t s) {
    combineSkipKernel<<<gridFor(static_cast<long long>(B) * D * H * W * (c2 / 8)), kThreads, 0, s>>>(
        dcat, ccat, c1, dpool, skip, c2, D, H, W, B, dpre);
    return cudaGetLastError();
}

cudaError_t launchSlowness(const Sample *samples, Geometry g, int B, float *slow, cudaStream_t s) {
    slownessKernel<<<gridFor(static_cast<long long>(B) * g.nx * g.ny * g.nz), kThreads, 0, s>>>(samples, g, B, slow);
    return cudaGetLastError();
}

cudaError_t launchFeatures(const Sample *samples, const float *slow, Geometry g, int B, bf16 *feat, cudaStream_t s) {
    const long long n = static_cast<long long>(B) * g.nx * g.ny * g.nz;
    featuresKernel<<<static_cast<int>((n + kThreads - 1) / kThreads), kThreads, 0, s>>>(samples, slow, g, B, feat);
    return cudaGetLastError();
}

cudaError_t launchHeadLoss(const bf16 *h, const float *hw, const Sample *samples, const float *slow, Geometry g,
                           int B, double invN, float *dhw, bf16 *dpre, double *lossSum, cudaStream_t s) {
    const long long n = static_cast<long long>(B) * g.nx * g.ny * g.nz;
    headLossKernel<<<static_cast<int>((n + kThreads - 1) / kThreads), kThreads, 0, s>>>(h, hw, samples, slow, g, B,
                                                                                       invN, dhw, dpre, lossSum);
    return cudaGetLastError();
}

cudaError_t launchPredict(const bf16 *h, const float *hw, const Sample *samples, const float *slow, Geometry g, int B,
                          double inflate, float *out, double *lossSum, cudaStream_t s) {
    const long long n = static_cast<long long>(B) * g.nx * g.ny * g.nz;
    predictKernel<<<static_cast<int>((n + kThreads - 1) / kThreads), kThreads, 0, s>>>(
        h, hw, samples, slow, g, B, static_cast<float>(inflate), out, lossSum);
    return cudaGetLastError();
}

cudaError_t launchAdam(float *p, const float *g, float *m, float *v, bf16 *pb, long long n, float lr, float b1,
                       float b2, float eps, float bc1, float bc2, cudaStream_t s) {
    adamKernel<<<gridFor(n, 4096), kThreads, 0, s>>>(p, g, m, v, pb, n, lr, b1, b2, eps, bc1, bc2);
    return cudaGetLastError();
}

cudaError_t launchToBF16(const float *p, bf16 *pb, long long n, cudaStream_t s) {
    toBF16Kernel<<<gridFor(n, 4096), kThreads, 0, s>>>(p, pb, n);
    return cudaGetLastError();
}

cudaError_t launchFlipTranspose(const bf16 *w, int cout, int cin, bf16 *wt, cudaStream_t s) {
    flipTransposeKernel<<<gridFor(27LL * cout * cin, 4096), kThreads, 0, s>>>(w, cout, cin, wt);
    return cudaGetLastError();
}

}  // namespace net
}  // namespace eikx
