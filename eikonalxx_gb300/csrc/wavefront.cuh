// Shared machinery of the pipelined level-set sweep kernels.
//
// Layout of the work (one sweep of one batch of fields):
//   * Coordinates are sweep-permuted (x', y', z'): each axis the sweep runs in
//     decreasing order is mirrored, so every sweep proceeds towards +x', +y', +z' and
//     its levels are the planes x'+y'+z' = const (permuteGrid / Graph3D,
//     solverUtilities3d.hpp:1197-1257, src/graph3d.cpp:120-221).
//   * A warp owns a block of x'-pencils (3D: LY x LZ, lane = lz*LY + ly; 2D: 32 rows)
//     and walks it in steps: at step s lane (ly,lz) updates x' = s - ly - lz.  All nodes
//     a warp touches in one step lie on one level, so they are independent, and every
//     node a step reads lies on an earlier level: the warp reproduces the reference's
//     serial iz/iy/ix loop (include/private/solver3d.hpp:186-243) exactly.
//   * Values a lane needs from its upwind lanes come from a per-warp shared-memory ring
//     indexed by step.  Upwind values from outside the block are the last rows of the
//     upstream warp blocks: each block publishes its two downstream faces, node by node,
//     into a mailbox of 64-bit words (sweep tag << 32 | value bits).  A word is its own
//     flag -- its tag says which sweep wrote it -- so a consumer spins (bounded) on the
//     very word it needs and no fence or progress counter is involved.  Helper lanes
//     fetch the face values kPref steps ahead of their use.
//   * Own rows of travel times and slowness stream through registers in 16-byte chunks
//     fetched one chunk ahead.
//   * Blocks are taken from a queue sorted by the step at which they can start, so a
//     block only ever waits on blocks that were dequeued before it (and are running).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace eikx {

constexpr int kRing = 16;     // ring slots per lane (power of two, >= kPref + 4)
constexpr int kPref = 4;      // halo loads are issued kPref steps before their values are needed
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int ldVolatile(const int *p) {
    return *reinterpret_cast<const volatile int *>(p);
}
// Mailbox words are read and written with relaxed gpu-scope accesses: each 64-bit word
// is its own flag, so no ordering with other memory operations is needed.
__device__ __forceinline__ unsigned long long ldRelaxed(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ void stRelaxed(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v));
}

// Mailbox words of one value: FP32 fits in one tagged word, FP64 needs two.
template <class T> struct Mail;
template <> struct Mail<float> {
    static constexpr int kWords = 1;
    __device__ static void put(unsigned long long *w, unsigned tag, float v) {
        stRelaxed(w, (static_cast<unsigned long long>(tag) << 32) | __float_as_uint(v));
    }
    // Spin until the word carries `tag`; false when the bound runs out or another warp
    // raised the abort flag.
    __device__ static bool get(const unsigned long long *w, unsigned tag, float &v, int *abortFlag,
                               unsigned long long spinLimit) {
        unsigned long long it = 0;
        while (true) {
            const unsigned long long x = ldRelaxed(w);
            if (static_cast<unsigned>(x >> 32) == tag) {
                v = __uint_as_float(static_cast<unsigned>(x));
                return true;
            }
            if ((++it & 31ull) == 0) {
                if (ldVolatile(abortFlag)) return false;
                if (it > spinLimit) {
                    atomicExch(abortFlag, 1);
                    return false;
                }
            }
            __nanosleep(32);
        }
    }
};
template <> struct Mail<double> {
    static constexpr int kWords = 2;
    __device__ static void put(unsigned long long *w, unsigned tag, double v) {
        const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
        stRelaxed(w, (static_cast<unsigned long long>(tag) << 32) | (b & 0xffffffffull));
        stRelaxed(w + 1, (static_cast<unsigned long long>(tag) << 32) | (b >> 32));
    }
    __device__ static bool get(const unsigned long long *w, unsigned tag, double &v, int *abortFlag,
                               unsigned long long spinLimit) {
        unsigned long long it = 0;
        while (true) {
            const unsigned long long lo = ldRelaxed(w), hi = ldRelaxed(w + 1);
            if (static_cast<unsigned>(lo >> 32) == tag && static_cast<unsigned>(hi >> 32) == tag) {
                v = __longlong_as_double(static_cast<long long>((hi << 32) | (lo & 0xffffffffull)));
                return true;
            }
            if ((++it & 31ull) == 0) {
                if (ldVolatile(abortFlag)) return false;
                if (it > spinLimit) {
                    atomicExch(abortFlag, 1);
                    return false;
                }
            }
            __nanosleep(32);
        }
    }
};

// A mailbox read in flight: the word(s) are loaded when the slot is issued and checked
// when the value is needed, kPref steps later, so the L2 round trip overlaps the work of
// those steps.  A word not yet carrying the expected tag is then re-read (bounded spin).
template <class T> struct MailSlot {
    static constexpr int W = Mail<T>::kWords;
    unsigned long long w[W];
    __device__ __forceinline__ void issue(const unsigned long long *p) {
#pragma unroll
        for (int k = 0; k < W; ++k) w[k] = ldRelaxed(p + k);
    }
    __device__ __forceinline__ bool take(const unsigned long long *p, unsigned tag, T &v, int *abortFlag,
                                         unsigned long long spinLimit) const {
        bool ready = true;
#pragma unroll
        for (int k = 0; k < W; ++k) ready = ready && static_cast<unsigned>(w[k] >> 32) == tag;
        if (!ready) return Mail<T>::get(p, tag, v, abortFlag, spinLimit);
        if constexpr (W == 1) {
            v = __uint_as_float(static_cast<unsigned>(w[0]));
        } else {
            v = __longlong_as_double(static_cast<long long>((w[1] << 32) | (w[0] & 0xffffffffull)));
        }
        return true;
    }
};

// 16-byte chunk of a row: 4 floats or 2 doubles.
template <class T> struct Chunk {
    static constexpr int kN = 16 / sizeof(T);
    T v[kN];
    __device__ __forceinline__ void load(const T *p) {
        const uint4 u = *reinterpret_cast<const uint4 *>(p);
        *reinterpret_cast<uint4 *>(v) = u;
    }
    __device__ __forceinline__ T at(int i) const {
        T r = v[0];
#pragma unroll
        for (int k = 1; k < kN; ++k) r = (i == k) ? v[k] : r;
        return r;
    }
};

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
