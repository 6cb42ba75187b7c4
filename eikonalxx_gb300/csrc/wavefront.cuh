// Shared machinery of the pipelined level-set sweep kernels.
//
// Layout of the work (one sweep of one batch of fields):
//   * Coordinates are sweep-permuted (x', y', z'): each axis the sweep runs in
//     decreasing order is mirrored, so every sweep proceeds towards +x', +y', +z' and
//     its levels are the planes x'+y'+z' = const (permuteGrid / Graph3D,
//     solverUtilities3d.hpp:1197-1257, src/graph3d.cpp:120-221).
//   * A warp owns an LY x LZ block of x'-pencils (lane = lz*LY + ly) and walks it in
//     steps: at step s lane (ly,lz) updates x' = s - ly - lz.  All nodes a warp
//     touches in one step lie on one level, so they are independent, and every node a
//     step reads lies on an earlier level: the warp reproduces the reference's serial
//     iz/iy/ix loop (include/private/solver3d.hpp:186-243) exactly.
//   * Values a lane needs from its upwind lanes come from a per-warp shared-memory ring
//     indexed by step; the upwind neighbours outside the block (the "halo" rows of the
//     upstream warp blocks) are prefetched from L2 PREF steps ahead by helper lanes.
//   * Blocks are taken from a queue sorted by start time; a block waits (bounded) on
//     release/acquire progress counters of its two upstream blocks, so blocks of a
//     field pipeline behind each other and blocks of different fields interleave.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace eikx {

constexpr int kRing = 16;     // ring slots per lane (power of two, >= kPref + 4)
constexpr int kPref = 4;      // halo prefetch distance in steps
constexpr int kPub = 4;       // publish own progress every kPub steps
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ unsigned ldAcquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void stRelease(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void fenceAcqRel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ int ldVolatile(const int *p) {
    return *reinterpret_cast<const volatile int *>(p);
}

// L2-coherent loads for data another warp of this launch wrote (the halo rows).
__device__ __forceinline__ float ldL2(const float *p) { return __ldcg(p); }
__device__ __forceinline__ double ldL2(const double *p) { return __ldcg(p); }

// Spin (bounded) until *flag >= need.  Returns false, after raising *abortFlag, when
// the bound runs out or another warp already raised it.  Only lane 0 calls this.
__device__ __forceinline__ bool waitAtLeast(const unsigned *flag, unsigned need, unsigned &known,
                                            int *abortFlag, unsigned long long spinLimit) {
    if (known >= need) return true;
    unsigned long long it = 0;
    while (true) {
        known = ldAcquire(flag);
        if (known >= need) return true;
        if ((++it & 63ull) == 0) {
            if (ldVolatile(abortFlag)) return false;
            if (it > spinLimit) {
                atomicExch(abortFlag, 1);
                return false;
            }
        }
        __nanosleep(64);
    }
}

// Reflect an index of an axis that the sweep runs in decreasing order.
__device__ __forceinline__ int reflect(int p, int n, int flip) { return flip ? n - 1 - p : p; }

// Inclusive update range of one axis in actual coordinates, as getLoopLimits
// (solverUtilities3d.hpp:944-1184, solverUtilities2d.hpp:939-1053): an increasing axis
// starts at 1 (at the source cell for the initialisation pass), a decreasing one at
// n-2 (at the cell above the source).
__device__ __forceinline__ void axisBounds(int n, int flip, int init, int is, int &lo, int &hi) {
    if (!flip) {
        lo = init ? max(1, is) : 1;
        hi = n - 1;
    } else {
        lo = 0;
        hi = init ? min(is + 1, n - 2) : n - 2;
    }
}

__device__ __forceinline__ double warpMax(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(kFull, v, o));
    return v;
}

}  // namespace eikx
