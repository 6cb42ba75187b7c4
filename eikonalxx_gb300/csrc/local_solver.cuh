// Upwind local solvers of the eikonal equation, device side.
//
// These evaluate the same operators, in the same floating-point operation order, as
// the reference's finiteDifference functions:
//   3D uniform      include/private/solverUtilities3d.hpp:258-558
//   3D non-uniform  include/private/solverUtilities3d.hpp:562-824
//   2D uniform      include/private/solverUtilities2d.hpp:347-472
//   2D non-uniform  include/private/solverUtilities2d.hpp:474-614
// The translation unit is compiled with --fmad=false, -prec-sqrt=true and
// -prec-div=true, so each operation rounds exactly as the CPU code (IEEE binary32 /
// binary64, correctly rounded sqrt and division, no contraction) and a sweep
// reproduces the reference's travel times bit for bit.
#pragma once
#include <cuda_runtime.h>

namespace eikx {

template <class T> __device__ __forceinline__ T dmin(T a, T b);
template <> __device__ __forceinline__ float dmin(float a, float b) { return fminf(a, b); }
template <> __device__ __forceinline__ double dmin(double a, double b) { return fmin(a, b); }
template <class T> __device__ __forceinline__ T dmax(T a, T b);
template <> __device__ __forceinline__ float dmax(float a, float b) { return fmaxf(a, b); }
template <> __device__ __forceinline__ double dmax(double a, double b) { return fmax(a, b); }
// Minimum and maximum for operands known not to be negative (slowness values, which the model
// checks keep positive and finite; a maximum that includes a positive floor): for such doubles
// the IEEE order is the order of their bit patterns as signed 64-bit integers (a negative value
// only ever loses a maximum against a positive floor). So the selection runs on the integer
// pipe instead of GB300's narrow FP64 pipe, with the result fmin / fmax would give. FP32 keeps
// fminf / fmaxf.
template <class T> __device__ __forceinline__ T pmin(T a, T b) { return dmin(a, b); }
template <> __device__ __forceinline__ double pmin(double a, double b) {
    const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return __longlong_as_double(x < y ? x : y);
}
template <class T> __device__ __forceinline__ T pmax(T a, T b) { return dmax(a, b); }
template <> __device__ __forceinline__ double pmax(double a, double b) {
    const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return __longlong_as_double(x > y ? x : y);
}
// t0 <= min(a, b, c, d, e), for values that are not NaN.  FP64 compares order keys on the
// integer pipe: the bit pattern for x >= +0, minus its magnitude bits for x <= -0, which is
// monotone in x and equal for -0 and +0.
template <class T> __device__ __forceinline__ bool atMostAll(T t0, T a, T b, T c, T d, T e) {
    return t0 <= dmin(dmin(a, dmin(b, c)), dmin(d, e));
}
__device__ __forceinline__ long long orderKey(double x) {
    const long long v = __double_as_longlong(x);
    return v >= 0 ? v : -(v & 0x7fffffffffffffffLL);
}
template <> __device__ __forceinline__ bool atMostAll(double t0, double a, double b, double c, double d, double e) {
    const long long k = orderKey(t0);
    return (k <= orderKey(a)) & (k <= orderKey(b)) & (k <= orderKey(c)) & (k <= orderKey(d)) & (k <= orderKey(e));
}
__device__ __forceinline__ float dsqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ double dsqrt(double a) { return sqrt(a); }

// Per-sweep constants (getSweepFiniteDifferenceSigns, solverUtilities3d.hpp:843-925
// and solverUtilities2d.hpp:888-926): a flipped axis is swept in decreasing order,
// its analytic-time shift is +1 and its derivative sign -1.
struct SweepSigns {
    int ixShift, iyShift, izShift;
    int signX, signY, signZ;
};

// Source description as the sweep objects hold it (Solver3DSweep::setSourceInformation,
// include/private/solver3d.hpp:131-144): source cell, offsets from the origin and the
// source-cell slowness, all in the sweep's type.
template <class T> struct SourceT {
    int isx, isy, isz;
    T xs, ys, zs;
    T sSrc;
};


// Analytic homogeneous time and gradient (computeAnalyticalTravelTime,
// solverUtilities3d.hpp:138-208).
template <class T>
__device__ __forceinline__ T analyticT3(int ix, int iy, int iz, T dx, T dy, T dz, T xs, T ys,
                                        T zs, T s) {
    T x = ix * dx, y = iy * dy, z = iz * dz;
    T ddx = x - xs, ddy = y - ys, ddz = z - zs;
    T dist = dsqrt(ddx * ddx + ddy * ddy + ddz * ddz);
    return s * dist;
}
template <class T>
__device__ __forceinline__ void analyticTG3(int ix, int iy, int iz, T dx, T dy, T dz, T xs,
                                            T ys, T zs, T s, T &t, T &gx, T &gy, T &gz) {
    T x = ix * dx, y = iy * dy, z = iz * dz;
    T ddx = x - xs, ddy = y - ys, ddz = z - zs;
    T dist = dsqrt(ddx * ddx + ddy * ddy + ddz * ddz);
    t = s * dist;
    gx = 0; gy = 0; gz = 0;
    if (dist > 0) {
        gx = (s * ddx) / dist;
        gy = (s * ddy) / dist;
        gz = (s * ddz) / dist;
    }
}

// The neighbour naming of the reference's 3D stencil (gridToSurroundingTravelTimeIndices,
// solverUtilities3d.hpp:1460-1586; gridToSurroundingSlownessIndices, :1300-1442), with
// "up" = one step against the sweep direction along an axis:
//   t1 = x-up, t2 = x-up,y-up, t3 = y-up, t4 = z-up, t5 = x-up,z-up, t6 = all up,
//   t7 = y-up,z-up;  s0 = home cell, s1 = x-neighbour cell, s2 = x,y, s3 = y, s4 = z,
//   s5 = x,z, s7 = y,z.
template <class T> struct Stencil3 {
    T s0, s1, s2, s3, s4, s5, s7;
    T t1, t2, t3, t4, t5, t6, t7;
};

// The FP64 analytic factor of an FP32 sweep (eikx_options.near_fp64).  Within the
// factored radius the reference forms T0 = s0 |x - xs| (s0 the node's home-cell
// slowness), its gradient s0 (x - xs) / |x - xs|, the differences tau_k = t_k - T0_k at
// the 7 upwind neighbours and the candidate T0 + correction in the sweep type
// (solverUtilities3d.hpp:372-553); in FP32 the differences lose most of their digits to
// cancellation.  In this mode:
//   * D = |x - xs| and U = (x - xs) / D are formed in FP64 from FP64 offsets and spacing,
//     at the unclamped stencil positions, as the reference's analytic times are;
//   * T0_k = s0 D_k in FP64, carried as the float pair hi = fl(T0_k), lo = fl(T0_k - hi);
//   * tau_k = fl(fl(t_k - hi_k) - lo_k), the gradient fl(s0 U) (then the sweep's signs),
//     and the candidate fl(hi_0 + fl(correction + lo_0)), all FP32 operations;
//   * the quadratic solves stay in FP32.
// The pairs and gradient of every node within the radius depend on the node, the sweep
// ordering (its home cell and upwind neighbours) and the model only, so they are
// tabulated once per solve (FP64, `table`) and the sweep kernels read them: the kernels
// run no FP64 instruction.  Kept apart from SourceT, so the kernels without this mode
// carry none of it.
struct alignas(16) NearFactor {
    float hi[8], lo[8];   // T0 at the node (0) and at its upwind neighbours t1..t7 (1..7)
    float gx, gy, gz;     // the gradient of T0 (the sweep applies its signs)
    float pad;
};
struct SourceFp64 {
    double xs, ys, zs;          // source offsets from the origin (FP64)
    double dx, dy, dz;          // grid spacing (FP64)
    const NearFactor *table;    // [sweep][bz][by][bx] entries of the nodes within the radius
    int bx0, by0, bz0, bnx, bny, bnz;   // the table's node box
    // for filling the table: the model's unshifted edge-replicated FP32 slowness copy
    // (cell (cx, cy, cz) at (cz + 1) spPlane + (cy + 1) spPitch + cx + 1) and its cells
    const float *sp;
    long long spPlane;
    int spPitch, ncx, ncy, ncz;
};
// Largest factor table of one field (entries, 8 sweeps x nodes; 80 bytes each): factored
// radius 15, or a grid of 32,768 nodes, whatever the radius.  near_fp64 solves whose
// factored region needs more are rejected.
constexpr int kMaxFactorTable = 1 << 18;

// D of position (ix, iy, iz) in FP64, as analyticT3<double> forms the distance.
__host__ __device__ inline double factorDistance(const SourceFp64 &f, int ix, int iy, int iz, double *u = nullptr) {
    const double ddx = ix * f.dx - f.xs, ddy = iy * f.dy - f.ys, ddz = iz * f.dz - f.zs;
    const double d = sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
    if (u) {
        u[0] = d > 0 ? ddx / d : 0.0;
        u[1] = d > 0 ? ddy / d : 0.0;
        u[2] = d > 0 ? ddz / d : 0.0;
    }
    return d;
}
// The entry of node (ix, iy, iz) with home-cell slowness s0 (as the sweep holds it) in the
// sweep with signs sg.
__host__ __device__ inline NearFactor nearFactor(const SourceFp64 &f, float s0, const SweepSigns &sg, int ix, int iy,
                                                 int iz) {
    const int xu = ix + sg.ixShift, yu = iy + sg.iyShift, zu = iz + sg.izShift;
    const int px[8] = {ix, xu, xu, ix, ix, xu, xu, ix};
    const int py[8] = {iy, iy, yu, yu, iy, iy, yu, yu};
    const int pz[8] = {iz, iz, iz, iz, zu, zu, zu, zu};
    const double s = s0;
    NearFactor e;
    double u[3];
    for (int k = 0; k < 8; ++k) {
        const double t0 = s * factorDistance(f, px[k], py[k], pz[k], k == 0 ? u : nullptr);
        e.hi[k] = static_cast<float>(t0);
        e.lo[k] = static_cast<float>(t0 - static_cast<double>(e.hi[k]));
    }
    e.gx = static_cast<float>(s * u[0]);
    e.gy = static_cast<float>(s * u[1]);
    e.gz = static_cast<float>(s * u[2]);
    e.pad = 0;
    return e;
}
// Sweep ordering 0..7 of a set of signs (bit 0: x decreasing, 1: y, 2: z).
__host__ __device__ inline int sweepOf(const SweepSigns &sg) {
    return (sg.ixShift > 0 ? 1 : 0) | (sg.iyShift > 0 ? 2 : 0) | (sg.izShift > 0 ? 4 : 0);
}
// The table entry of node (ix, iy, iz), a node within the factored radius (inside the box).
__device__ __forceinline__ const NearFactor &nearFactorAt(const SourceFp64 &f, const SweepSigns &sg, int ix, int iy,
                                                          int iz) {
    const int bx = ix - f.bx0, by = iy - f.by0, bz = iz - f.bz0;
    return f.table[((static_cast<long long>(sweepOf(sg)) * f.bnz + bz) * f.bny + by) * f.bnx + bx];
}

// 3D uniform-grid update (solverUtilities3d.hpp:258-558), split at the reference's
// branch on the factored radius (:286-300): fd3UniformFar is the Cartesian branch, taken
// when the node is more than `radius` cells from the source cell along some axis;
// fd3UniformNear is the factored branch, the reference's as shipped (T0 built from the
// home-cell slowness s0).  Both evaluate the common head-wave prefix first, exactly as
// the reference does before it branches.
#define EIKX_FD3_UNIFORM_PREFIX                                                        \
    const T huge = static_cast<T>(1.e10);                                              \
    const T s0 = n.s0, s1 = n.s1, s2 = n.s2, s3 = n.s3, s4 = n.s4, s5 = n.s5, s7 = n.s7; \
    const T t1 = n.t1, t2 = n.t2, t3 = n.t3, t4 = n.t4, t5 = n.t5, t6 = n.t6, t7 = n.t7; \
    T tUpd;                                                                            \
    T minS0S3 = pmin(s0, s3);                                                          \
    T minS0S1 = pmin(s0, s1);                                                          \
    T minS0S4 = pmin(s0, s4);                                                          \
    T t1d1 = t1 + h * pmin(minS0S3, pmin(s4, s7));                                     \
    T t1d2 = t3 + h * pmin(minS0S4, pmin(s1, s5));                                     \
    T t1d3 = t4 + h * pmin(minS0S1, pmin(s2, s3));                                     \
    T t1d = dmin(dmin(t1d1, t1d2), t1d3);                                              \
    T hs03 = h * minS0S3;                                                              \
    T hs01 = h * minS0S1;                                                              \
    T hs04 = h * minS0S4;

template <class T>
__device__ __forceinline__ T fd3UniformFar(T h, const Stencil3<T> &n) {
    EIKX_FD3_UNIFORM_PREFIX
    {
        // 2D critically refracted (diagonal) operators in the XZ, YZ and XY planes.
        // Evaluated branch-free: every lane runs the same instructions and a failed
        // condition selects `huge`; a taken operator rounds exactly as the reference's.
        const T one = 1;
        T dXZ = t1 - t4;
        T detXZ = 2 * (hs03 * hs03) - dXZ * dXZ;
        const bool cXZ = detXZ > 0 && t4 <= t1 + hs03 && t1 <= t4 + hs03;
        const T rXZ = dsqrt(cXZ ? detXZ : one);
        T t2d = cXZ ? t5 + rXZ : huge;
        T dYZ = t3 - t4;
        T detYZ = 2 * (hs01 * hs01) - dYZ * dYZ;
        const bool cYZ = detYZ > 0 && t3 <= t4 + hs01 && t4 <= t3 + hs01;
        const T rYZ = dsqrt(cYZ ? detYZ : one);
        t2d = dmin(t2d, cYZ ? t7 + rYZ : huge);
        T dXY = t1 - t3;
        T detXY = 2 * (hs04 * hs04) - dXY * dXY;
        const bool cXY = detXY > 0 && t3 <= t1 + hs04 && t1 <= t3 + hs04;
        const T rXY = dsqrt(cXY ? detXY : one);
        t2d = dmin(t2d, cXY ? t2 + rXY : huge);
        // 8-point operator, taken only when the wave travels the sweep's way
        const T third = static_cast<T>(0.33333333333333333333333);
        const T half = static_cast<T>(0.5);
        T Tx = t1 + half * (-t4 + t5 - t3 + t2) - t7 + t6;
        T Ty = t3 + half * (-t4 + t7 - t1 + t2) - t5 + t6;
        T Tz = t4 + half * (-t1 + t5 - t3 + t7) - t2 + t6;
        T det = 27 * (h * s0) * (h * s0) - (Tx - Ty) * (Tx - Ty) - (Tx - Tz) * (Tx - Tz) -
                (Ty - Tz) * (Ty - Tz);
        const bool c3 = dmin(t1d, t2d) > dmax(dmax(t1, t4), t3) && det >= 0;
        const T r3 = dsqrt(c3 ? det : one);
        T t3d = c3 ? third * ((Tx + Ty + Tz) + r3) : huge;
        tUpd = dmin(t1d, dmin(t2d, t3d));
    }
    return tUpd;
}

// fd3UniformFar for a node whose current time is t0, for callers that keep min(t0, result):
// it returns t0 as soon as lower bounds show that no operator goes below t0, and evaluates
// an operator only where its bound leaves it a chance to.  The bounds hold for the rounded
// values, since round-to-nearest is monotone (u = unit roundoff: 2^-24 in FP32, less in
// FP64; all times are >= 0, M = max(t1..t7, 2^-100)).  The bounds are formed with fused
// multiply-adds: they only need to stay below the operators, which are evaluated unfused,
// as the reference does.
//   * a 2D operator, when its window is open, returns t_d + r (t_d = t5, t7, t2 for XZ, YZ,
//     XY) with r = sqrt(2 hs^2 - (t_a - t_b)^2) and |t_a - t_b| <= hs by its window (hs the
//     operator's h * min slowness, t_a, t_b its two axis neighbours).  The window test, the
//     determinant and the square root round with unit roundoff u: the test admits
//     |t_a - t_b| <= hs + u (t_a + t_b + hs), and the computed r is >= hs - u (t_a + t_b)
//     - 5 u hs up to second-order terms.  So r >= m with m = hs (1 - 2^-20) - 3 * 2^-20 M,
//     formed in T (3 M >= t1 + t3 + t4 >= t_a + t_b, so the margin is at least 10 u hs and
//     15 u (t_a + t_b), which covers the second-order terms and m's own rounding; m < 0
//     whenever the times are so large that the margin would not), and the operator is
//     >= L_d = t_d + m; a closed window returns huge;
//   * the 8-point operator returns third * (S + r3) with S = (Tx + Ty) + Tz, r3 >= 0, so it
//     is >= third * S (or huge when its window is closed).  In exact arithmetic Tx + Ty + Tz
//     = 3 t6.  Each of Tx, Ty, Tz is seven roundings of values within [-3M, 3M]: an error of
//     at most 9.5 u M; the two sums add 9 u M, and third = 1/3 (1 + d), |d| <= u, so
//     third * S >= t6 - 15 u M up to second-order terms.  lo3 = t6 - M 2^-18 (64 u M in FP32,
//     one rounding; M >= 2^-100 keeps the underflow of the halvings, 2^-150, far below the
//     margin) is a lower bound of it;
//   * if t0 <= min(t1d, L2, L5, L7, lo3), fd3UniformFar's result is >= t0;
//   * a 2D operator with L_d >= t0 and L_d > max(t1, t4, t3) is left out (taken as huge): it
//     is >= t0, so min(t0, .) does not see it, and it is above the 8-point window's
//     max(t1, t4, t3), so min(t1d, t2d) > max(t1, t4, t3) holds with it exactly when without;
//   * if lo3 >= min(t0, t1d, t2d), the 8-point operator is >= that minimum and is left out.
// So min(t0, result) is min(t0, fd3UniformFar(h, n)) bit for bit.  Over the refinement
// sweeps of the benchmark model the operators left out are 1.76 of the three 2D operators
// and 70 % of the 8-point operators per warp that reaches them.
__device__ __forceinline__ float fmaT(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmaT(double a, double b, double c) { return __fma_rn(a, b, c); }
// HS: the stencil's slowness values are the cells' slowness already multiplied by h (the FP64
// sweeps' scaled copies).  With h > 0, round-to-nearest multiplication is monotone, so h times
// a minimum is the minimum of the products, bit for bit: every term below is the one the
// unscaled form computes.
template <class T, bool HS = false>
__device__ __forceinline__ T fd3UniformFarBounded(T h, const Stencil3<T> &n, T t0) {
    const T huge = static_cast<T>(1.e10);
    const T s0 = n.s0, s1 = n.s1, s2 = n.s2, s3 = n.s3, s4 = n.s4, s5 = n.s5, s7 = n.s7;
    const T t1 = n.t1, t2 = n.t2, t3 = n.t3, t4 = n.t4, t5 = n.t5, t6 = n.t6, t7 = n.t7;
    auto byH = [h](T x) -> T {
        if constexpr (HS) return x;
        else return h * x;
    };
    const T minS0S3 = pmin(s0, s3), minS0S1 = pmin(s0, s1), minS0S4 = pmin(s0, s4);
    const T t1d1 = t1 + byH(pmin(minS0S3, pmin(s4, s7)));
    const T t1d2 = t3 + byH(pmin(minS0S4, pmin(s1, s5)));
    const T t1d3 = t4 + byH(pmin(minS0S1, pmin(s2, s3)));
    const T t1d = dmin(dmin(t1d1, t1d2), t1d3);
    const T hs03 = byH(minS0S3), hs01 = byH(minS0S1), hs04 = byH(minS0S4);
    const T c20 = static_cast<T>(1.0 - 1.0 / 1048576.0);
    const T M = pmax(pmax(pmax(t1, t2), pmax(t3, t4)),
                     pmax(pmax(t5, t6), pmax(t7, static_cast<T>(7.8886090522101181e-31))));   // 2^-100
    const T E = M * static_cast<T>(3.0 / 1048576.0);
    const T L2 = t2 + fmaT(hs04, c20, -E), L5 = t5 + fmaT(hs03, c20, -E), L7 = t7 + fmaT(hs01, c20, -E);
    const T lo3 = fmaT(M, static_cast<T>(-1.0 / 262144.0), t6);
    if (atMostAll(t0, t1d, L2, L5, L7, lo3)) return t0;
    const T m = dmax(dmax(t1, t4), t3);
    T t2d = huge;
    if (L5 < t0 || !(L5 > m)) {
        const T dXZ = t1 - t4;
        const T detXZ = 2 * (hs03 * hs03) - dXZ * dXZ;
        if (detXZ > 0 && t4 <= t1 + hs03 && t1 <= t4 + hs03) t2d = t5 + dsqrt(detXZ);
    }
    if (L7 < t0 || !(L7 > m)) {
        const T dYZ = t3 - t4;
        const T detYZ = 2 * (hs01 * hs01) - dYZ * dYZ;
        if (detYZ > 0 && t3 <= t4 + hs01 && t4 <= t3 + hs01) t2d = dmin(t2d, t7 + dsqrt(detYZ));
    }
    if (L2 < t0 || !(L2 > m)) {
        const T dXY = t1 - t3;
        const T detXY = 2 * (hs04 * hs04) - dXY * dXY;
        if (detXY > 0 && t3 <= t1 + hs04 && t1 <= t3 + hs04) t2d = dmin(t2d, t2 + dsqrt(detXY));
    }
    // the 8-point operator under fd3UniformFar's condition: min(t1d, t2d, huge) is
    // min(t1d, t2d)
    const T t12 = dmin(t1d, t2d);
    if (lo3 >= dmin(t0, t12) || !(t12 > m)) return t12;
    const T third = static_cast<T>(0.33333333333333333333333);
    const T half = static_cast<T>(0.5);
    const T Tx = t1 + half * (-t4 + t5 - t3 + t2) - t7 + t6;
    const T Ty = t3 + half * (-t4 + t7 - t1 + t2) - t5 + t6;
    const T Tz = t4 + half * (-t1 + t5 - t3 + t7) - t2 + t6;
    T det = 27 * byH(s0) * byH(s0) - (Tx - Ty) * (Tx - Ty) - (Tx - Tz) * (Tx - Tz) - (Ty - Tz) * (Ty - Tz);
    if (!(det >= 0)) return t12;
    return dmin(t1d, dmin(t2d, third * (((Tx + Ty) + Tz) + dsqrt(det))));
}

// F64: the analytic factor in FP64 (SourceFp64, eikx_options.near_fp64; FP32 sweeps only).
template <class T, bool F64 = false>
__device__ __forceinline__ T fd3UniformNear(T h, const SourceT<T> &src, const SweepSigns &sg,
                                            int ix, int iy, int iz, const Stencil3<T> &n,
                                            const SourceFp64 *f64 = nullptr) {
    EIKX_FD3_UNIFORM_PREFIX
    {
        const T xs = src.xs, ys = src.ys, zs = src.zs, sSrc = src.sSrc;
        T t0, dt0dx, dt0dy, dt0dz;
        T tau1, tau2, tau3, tau4, tau5, tau6, tau7;
        NearFactor nf;
        if constexpr (F64 && sizeof(T) == 4) {
            nf = nearFactorAt(*f64, sg, ix, iy, iz);
            t0 = nf.hi[0];
            tau1 = (t1 - nf.hi[1]) - nf.lo[1]; tau2 = (t2 - nf.hi[2]) - nf.lo[2];
            tau3 = (t3 - nf.hi[3]) - nf.lo[3]; tau4 = (t4 - nf.hi[4]) - nf.lo[4];
            tau5 = (t5 - nf.hi[5]) - nf.lo[5]; tau6 = (t6 - nf.hi[6]) - nf.lo[6];
            tau7 = (t7 - nf.hi[7]) - nf.lo[7];
            dt0dx = nf.gx; dt0dy = nf.gy; dt0dz = nf.gz;
        } else {
            analyticTG3(ix, iy, iz, h, h, h, xs, ys, zs, s0, t0, dt0dx, dt0dy, dt0dz);
            const int xu = ix + sg.ixShift, yu = iy + sg.iyShift, zu = iz + sg.izShift;
            tau1 = t1 - analyticT3(xu, iy, iz, h, h, h, xs, ys, zs, s0);
            tau2 = t2 - analyticT3(xu, yu, iz, h, h, h, xs, ys, zs, s0);
            tau3 = t3 - analyticT3(ix, yu, iz, h, h, h, xs, ys, zs, s0);
            tau4 = t4 - analyticT3(ix, iy, zu, h, h, h, xs, ys, zs, s0);
            tau5 = t5 - analyticT3(xu, iy, zu, h, h, h, xs, ys, zs, s0);
            tau6 = t6 - analyticT3(xu, yu, zu, h, h, h, xs, ys, zs, s0);
            tau7 = t7 - analyticT3(ix, yu, zu, h, h, h, xs, ys, zs, s0);
        }
        // T0 + correction: in FP64 when the factor is
        auto plusT0 = [&](T d) -> T {
            if constexpr (F64 && sizeof(T) == 4) return nf.hi[0] + (d + nf.lo[0]);
            else return t0 + d;
        };
        dt0dx = sg.signX * dt0dx;
        dt0dy = sg.signY * dt0dy;
        dt0dz = sg.signZ * dt0dz;
        const T half = static_cast<T>(0.5);
        T hi = 1 / h;
        T h2inv = 1 / (h * h);
        T a = h2inv;
        T pXZ = tau1 - tau4 + tau5;
        T qXZ = tau4 - tau1 + tau5;
        T b = (2 * hi) * (dt0dx + dt0dz) - (2 * h2inv) * tau5;
        T c = (half * h2inv) * (pXZ * pXZ + qXZ * qXZ) - (2 * hi) * (dt0dx * pXZ + dt0dz * qXZ) +
              2 * (sSrc * sSrc - s0 * s0 + dt0dy * dt0dy);
        T det = b * b - 4 * a * c;
        T t2d = huge;
        if (det > 0 && t4 <= t1 + hs03 && t1 <= t4 + hs03) {
            t2d = plusT0((-b + dsqrt(det)) / (2 * a));
            if (t2d < t1 || t2d < t4) t2d = huge;
        }
        T pYZ = tau3 - tau4 + tau7;
        T qYZ = tau4 - tau3 + tau7;
        b = (2 * hi) * (dt0dy + dt0dz) - (2 * h2inv) * tau7;
        c = (half * h2inv) * (pYZ * pYZ + qYZ * qYZ) - (2 * hi) * (dt0dy * pYZ + dt0dz * qYZ) +
            2 * (sSrc * sSrc - s0 * s0 + dt0dx * dt0dx);
        det = b * b - 4 * a * c;
        T t2d2 = huge;
        if (det >= 0 && t3 <= t4 + hs01 && t4 <= t3 + hs01) {
            t2d2 = plusT0((-b + dsqrt(det)) / (2 * a));
            if (t2d2 < t3 || t2d2 < t4) t2d2 = huge;
        }
        t2d = dmin(t2d, t2d2);
        T pXY = tau1 - tau3 + tau2;
        T qXY = tau3 - tau1 + tau2;
        b = (2 * hi) * (dt0dx + dt0dy) - (2 * h2inv) * tau2;
        c = (half * h2inv) * (pXY * pXY + qXY * qXY) - (2 * hi) * (dt0dx * pXY + dt0dy * qXY) +
            2 * (sSrc * sSrc - s0 * s0 + dt0dz * dt0dz);
        det = b * b - 4 * a * c;
        T t2d3 = huge;
        if (det >= 0 && t3 <= t1 + hs04 && t1 <= t3 + hs04) {
            t2d3 = plusT0((-b + dsqrt(det)) / (2 * a));
            if (t2d3 < t1 || t2d3 < t3) t2d3 = huge;
        }
        t2d = dmin(t2d, t2d3);
        T t3d = huge;
        if (dmin(t1d, t2d) > dmax(dmax(t1, t4), t3)) {
            T taux = tau1 + half * (-tau4 + tau5 - tau3 + tau2) - tau7 + tau6;
            T tauy = tau3 + half * (-tau4 + tau7 - tau1 + tau2) - tau5 + tau6;
            T tauz = tau4 + half * (-tau1 + tau5 - tau3 + tau7) - tau2 + tau6;
            a = 3 * h2inv;
            b = -2 * h2inv * (taux + tauy + tauz) + (6 * hi) * (dt0dx + dt0dy + dt0dz);
            c = h2inv * (taux * taux + tauy * tauy + tauz * tauz) -
                (6 * hi) * (dt0dx * taux + dt0dy * tauy + dt0dz * tauz) + 9 * (sSrc * sSrc - s0 * s0);
            det = b * b - 4 * a * c;
            if (det >= 0) t3d = plusT0((-b + dsqrt(det)) / (2 * a));
            if (t3d < t1 || t3d < t3 || t3d < t4) t3d = huge;
        }
        tUpd = dmin(t1d, dmin(t2d, t3d));
    }
    return tUpd;
}
#undef EIKX_FD3_UNIFORM_PREFIX

__device__ __forceinline__ bool nearSource(int radius, int isx, int isy, int isz, int ix, int iy, int iz) {
    return !(abs(isx - ix) > radius || abs(isy - iy) > radius || abs(isz - iz) > radius);
}

template <class T>
__device__ __forceinline__ T fd3Uniform(int radius, T h, const SourceT<T> &src,
                                        const SweepSigns &sg, int ix, int iy, int iz,
                                        const Stencil3<T> &n) {
    if (!nearSource(radius, src.isx, src.isy, src.isz, ix, iy, iz)) return fd3UniformFar(h, n);
    return fd3UniformNear(h, src, sg, ix, iy, iz, n);
}

// Grid constants of the non-uniform 3D solver (include/private/solver3d.hpp:247-261),
// computed on the host in the field type and passed by value.
template <class T> struct Spacing3 {
    T dx, dy, dz, dxInv, dyInv, dzInv, dx2Inv, dy2Inv, dz2Inv;
    T dx_dz, dz_dx, dy_dz, dz_dy, dx_dy, dy_dx;
    T dx2_p_dz2_inv, dy2_p_dz2_inv, dx2_p_dy2_inv;
};

// 3D non-uniform update (solverUtilities3d.hpp:562-824), split at the factored-radius
// branch like the uniform solver.
#define EIKX_FD3_NONUNIFORM_PREFIX                                                     \
    const T huge = static_cast<T>(1.e10);                                              \
    const T dx = g.dx, dy = g.dy, dz = g.dz;                                           \
    const T s0 = n.s0, s1 = n.s1, s2 = n.s2, s3 = n.s3, s4 = n.s4, s5 = n.s5, s7 = n.s7; \
    const T t1 = n.t1, t2 = n.t2, t3 = n.t3, t4 = n.t4, t5 = n.t5, t6 = n.t6, t7 = n.t7; \
    T tUpd;                                                                            \
    T minS0S3 = pmin(s0, s3);                                                          \
    T minS0S1 = pmin(s0, s1);                                                          \
    T minS0S4 = pmin(s0, s4);                                                          \
    T t1d1 = t1 + dx * pmin(minS0S3, pmin(s4, s7));                                    \
    T t1d2 = t3 + dy * pmin(minS0S4, pmin(s1, s5));                                    \
    T t1d3 = t4 + dz * pmin(minS0S1, pmin(s2, s3));                                    \
    T t1d = dmin(dmin(t1d1, t1d2), t1d3);

template <class T>
__device__ __forceinline__ T fd3NonUniformFar(const Spacing3<T> &g, const Stencil3<T> &n) {
    EIKX_FD3_NONUNIFORM_PREFIX
    {
        T dXZ = t1 - t4;
        T detXZ = (dx * dx + dz * dz) * (minS0S3 * minS0S3) - dXZ * dXZ;
        T t2d = huge;
        if (detXZ > 0 && t1 < t4 + dz * minS0S3 && t4 < t1 + dx * minS0S3) {
            T TxXZ = t1 - t4 + t5;
            T TzXZ = t4 - t1 + t5;
            t2d = (TxXZ * g.dz_dx + TzXZ * g.dx_dz) + 2 * dsqrt(detXZ);
            t2d = ((dx * dz) * g.dx2_p_dz2_inv) * t2d;
        }
        T dYZ = t3 - t4;
        T detYZ = (dy * dy + dz * dz) * (minS0S1 * minS0S1) - dYZ * dYZ;
        T t2d2 = huge;
        if (detYZ > 0 && t3 < t4 + dz * minS0S1 && t4 < t3 + dy * minS0S1) {
            T TyYZ = t3 - t4 + t7;
            T TzYZ = t4 - t3 + t7;
            t2d2 = (TyYZ * g.dz_dy + TzYZ * g.dy_dz) + 2 * dsqrt(detYZ);
            t2d2 = ((dy * dz) * g.dy2_p_dz2_inv) * t2d2;
        }
        t2d = dmin(t2d, t2d2);
        T dXY = t1 - t3;
        T detXY = (dx * dx + dy * dy) * (minS0S4 * minS0S4) - dXY * dXY;
        T t2d3 = huge;
        if (detXY > 0 && t3 < t1 + dx * minS0S4 && t1 < t3 + dy * minS0S4) {
            T TxXY = t1 - t3 + t2;
            T TyXY = t3 - t1 + t2;
            t2d3 = (TxXY * g.dy_dx + TyXY * g.dx_dy) + 2 * dsqrt(detXY);
            t2d3 = ((dx * dy) * g.dx2_p_dy2_inv) * t2d3;
        }
        t2d = dmin(t2d, t2d3);
        T t3d = huge;
        if (dmin(t1d, t2d) > dmax(dmax(t1, t4), t3)) {
            const T half = static_cast<T>(0.5);
            T Tx = t1 + half * (-t4 + t5 - t3 + t2) - t7 + t6;
            T Ty = t3 + half * (-t4 + t7 - t1 + t2) - t5 + t6;
            T Tz = t4 + half * (-t1 + t5 - t3 + t7) - t2 + t6;
            T det = 9 * (s0 * s0) * (g.dx2Inv + g.dy2Inv + g.dz2Inv) -
                    ((Tx - Tz) * (Tx - Tz)) * (g.dx2Inv * g.dz2Inv) -
                    ((Ty - Tz) * (Ty - Tz)) * (g.dy2Inv * g.dz2Inv) -
                    ((Tx - Ty) * (Tx - Ty)) * (g.dx2Inv * g.dy2Inv);
            if (det >= 0)
                t3d = (Tx * g.dx2Inv + Ty * g.dy2Inv + Tz * g.dz2Inv + dsqrt(det)) /
                      (g.dx2Inv + g.dy2Inv + g.dz2Inv);
        }
        tUpd = dmin(t1d, dmin(t2d, t3d));
    }
    return tUpd;
}

template <class T, bool F64 = false>
__device__ __forceinline__ T fd3NonUniformNear(const Spacing3<T> &g, const SourceT<T> &src,
                                               const SweepSigns &sg, int ix, int iy, int iz,
                                               const Stencil3<T> &n, const SourceFp64 *f64 = nullptr) {
    EIKX_FD3_NONUNIFORM_PREFIX
    {
        const T xs = src.xs, ys = src.ys, zs = src.zs, sSrc = src.sSrc;
        T t0, dt0dx, dt0dy, dt0dz;
        T tau1, tau2, tau3, tau4, tau5, tau6, tau7;
        NearFactor nf;
        if constexpr (F64 && sizeof(T) == 4) {
            nf = nearFactorAt(*f64, sg, ix, iy, iz);
            t0 = nf.hi[0];
            tau1 = (t1 - nf.hi[1]) - nf.lo[1]; tau2 = (t2 - nf.hi[2]) - nf.lo[2];
            tau3 = (t3 - nf.hi[3]) - nf.lo[3]; tau4 = (t4 - nf.hi[4]) - nf.lo[4];
            tau5 = (t5 - nf.hi[5]) - nf.lo[5]; tau6 = (t6 - nf.hi[6]) - nf.lo[6];
            tau7 = (t7 - nf.hi[7]) - nf.lo[7];
            dt0dx = nf.gx; dt0dy = nf.gy; dt0dz = nf.gz;
        } else {
            analyticTG3(ix, iy, iz, dx, dy, dz, xs, ys, zs, s0, t0, dt0dx, dt0dy, dt0dz);
            const int xu = ix + sg.ixShift, yu = iy + sg.iyShift, zu = iz + sg.izShift;
            tau1 = t1 - analyticT3(xu, iy, iz, dx, dy, dz, xs, ys, zs, s0);
            tau2 = t2 - analyticT3(xu, yu, iz, dx, dy, dz, xs, ys, zs, s0);
            tau3 = t3 - analyticT3(ix, yu, iz, dx, dy, dz, xs, ys, zs, s0);
            tau4 = t4 - analyticT3(ix, iy, zu, dx, dy, dz, xs, ys, zs, s0);
            tau5 = t5 - analyticT3(xu, iy, zu, dx, dy, dz, xs, ys, zs, s0);
            tau6 = t6 - analyticT3(xu, yu, zu, dx, dy, dz, xs, ys, zs, s0);
            tau7 = t7 - analyticT3(ix, yu, zu, dx, dy, dz, xs, ys, zs, s0);
        }
        auto plusT0 = [&](T d) -> T {
            if constexpr (F64 && sizeof(T) == 4) return nf.hi[0] + (d + nf.lo[0]);
            else return t0 + d;
        };
        dt0dx = sg.signX * dt0dx;
        dt0dy = sg.signY * dt0dy;
        dt0dz = sg.signZ * dt0dz;
        const T dxInv = g.dxInv, dyInv = g.dyInv, dzInv = g.dzInv;
        const T dx2Inv = g.dx2Inv, dy2Inv = g.dy2Inv, dz2Inv = g.dz2Inv;
        T p = tau1 - tau4 + tau5;
        T q = tau4 - tau1 + tau5;
        T a = dx2Inv + dz2Inv;
        T b = 4 * (dxInv * dt0dx + dzInv * dt0dz) - 2 * (p * dx2Inv + q * dz2Inv);
        T c = (p * p) * dx2Inv + (q * q) * dz2Inv - 4 * ((dt0dx * p) * dxInv + (dt0dz * q) * dzInv) +
              4 * (sSrc * sSrc - s0 * s0 + dt0dy * dt0dy);
        T det = b * b - 4 * a * c;
        T t2d = huge;
        if (det > 0 && t1 < t4 + dz * minS0S3 && t4 < t1 + dx * minS0S3) {
            t2d = plusT0((-b + dsqrt(det)) / (2 * a));
            if (t2d < t1 || t2d < t4) t2d = huge;
        }
        p = tau3 - tau4 + tau7;
        q = tau4 - tau3 + tau7;
        a = dy2Inv + dz2Inv;
        b = 4 * (dyInv * dt0dy + dzInv * dt0dz) - 2 * (p * dy2Inv + q * dz2Inv);
        c = (p * p) * dy2Inv + (q * q) * dz2Inv - 4 * ((dt0dy * p) * dyInv + (dt0dz * q) * dzInv) +
            4 * (sSrc * sSrc - s0 * s0 + dt0dx * dt0dx);
        det = b * b - 4 * a * c;
        T t2d2 = huge;
        if (det > 0 && t3 < t4 + dz * minS0S1 && t4 < t3 + dy * minS0S1) {
            t2d2 = plusT0((-b + dsqrt(det)) / (2 * a));
            if (t2d2 < t3 || t2d2 < t4) t2d2 = huge;
        }
        t2d = dmin(t2d, t2d2);
        p = tau1 - tau3 + tau2;
        q = tau3 - tau1 + tau2;
        a = dx2Inv + dy2Inv;
        b = 4 * (dxInv * dt0dx + dyInv * dt0dy) - 2 * (p * dx2Inv + q * dy2Inv);
        c = (p * p) * dx2Inv + (q * q) * dy2Inv - 4 * ((dt0dx * p) * dxInv + (dt0dy * q) * dyInv) +
            4 * (sSrc * sSrc - s0 * s0 + dt0dz * dt0dz);
        det = b * b - 4 * a * c;
        T t2d3 = huge;
        if (det > 0 && t3 < t1 + dx * minS0S4 && t1 < t3 + dy * minS0S4) {
            t2d3 = plusT0((-b + dsqrt(det)) / (2 * a));
            if (t2d3 < t1 || t2d3 < t3) t2d3 = huge;
        }
        t2d = dmin(t2d, t2d3);
        T t3d = huge;
        if (dmin(t1d, t2d) > dmax(dmax(t1, t4), t3)) {
            const T half = static_cast<T>(0.5);
            T taux = tau1 + half * (-tau4 + tau5 - tau3 + tau2) - tau7 + tau6;
            T tauy = tau3 + half * (-tau4 + tau7 - tau1 + tau2) - tau5 + tau6;
            T tauz = tau4 + half * (-tau1 + tau5 - tau3 + tau7) - tau2 + tau6;
            a = dx2Inv + dy2Inv + dz2Inv;
            b = -2 * (taux * dx2Inv + tauy * dy2Inv + tauz * dz2Inv) +
                6 * (dxInv * dt0dx + dyInv * dt0dy + dzInv * dt0dz);
            c = (taux * taux) * dx2Inv + (tauy * tauy) * dy2Inv + (tauz * tauz) * dz2Inv -
                6 * (dt0dx * taux * dxInv + dt0dy * tauy * dyInv + dt0dz * tauz * dzInv) +
                9 * (sSrc * sSrc - s0 * s0);
            det = b * b - 4 * a * c;
            if (det >= 0) t3d = plusT0((-b + dsqrt(det)) / (2 * a));
            if (t3d < t1 || t3d < t3 || t3d < t4) t3d = huge;
        }
        tUpd = dmin(t1d, dmin(t2d, t3d));
    }
    return tUpd;
}
#undef EIKX_FD3_NONUNIFORM_PREFIX

template <class T>
__device__ __forceinline__ T fd3NonUniform(int radius, const Spacing3<T> &g, const SourceT<T> &src,
                                           const SweepSigns &sg, int ix, int iy, int iz,
                                           const Stencil3<T> &n) {
    if (!nearSource(radius, src.isx, src.isy, src.isz, ix, iy, iz)) return fd3NonUniformFar(g, n);
    return fd3NonUniformNear(g, src, sg, ix, iy, iz, n);
}

// ---------------------------------------------------------------------------- 2D

// hypot by Borges, "An Improved Algorithm for hypot(a,b)", arXiv:1904.09481 (2019),
// fused correction step; the oracle uses the same steps so both sides round alike.
__device__ __forceinline__ double eikxHypot(double a, double b) {
    a = fabs(a); b = fabs(b);
    if (a < b) { double t = a; a = b; b = t; }
    if (b == 0) return a;
    double h = sqrt(fma(a, a, b * b));
    double h2 = h * h;
    double a2 = a * a;
    double x = fma(-b, b, h2 - a2) + fma(h, h, -h2) - fma(a, a, -a2);
    return h - x / (2 * h);
}
__device__ __forceinline__ float eikxHypot(float a, float b) {
    double da = a, db = b;
    return static_cast<float>(sqrt(da * da + db * db));
}

template <class T>
__device__ __forceinline__ T analyticT2(int ix, int iz, T dx, T dz, T xs, T zs, T s) {
    T x = ix * dx, z = iz * dz;
    T ddx = x - xs, ddz = z - zs;
    return s * eikxHypot(ddx, ddz);
}
template <class T>
__device__ __forceinline__ void analyticTG2(int ix, int iz, T dx, T dz, T xs, T zs, T s, T &t,
                                            T &gx, T &gz) {
    T x = ix * dx, z = iz * dz;
    T ddx = x - xs, ddz = z - zs;
    T dist = eikxHypot(ddx, ddz);
    t = s * dist;
    gx = 0; gz = 0;
    if (dist > 0) {
        gx = (s * ddx) / dist;
        gz = (s * ddz) / dist;
    }
}

// 2D grid constants (include/private/solver2d.hpp:41-46), host-computed.
template <class T> struct Spacing2 {
    T dx, dz, dx_dz, dz_dx, cosTheta, sinTheta;
};

// 2D uniform update (solverUtilities2d.hpp:347-472).  t1 = x-up, t2 = diagonal,
// t3 = z-up; s0 home cell, s1 x-neighbour cell, s3 z-neighbour cell.
template <class T>
__device__ __forceinline__ T fd2Uniform(int radius, T h, const SourceT<T> &src,
                                        const SweepSigns &sg, int ix, int iz, T s0, T s1, T s3,
                                        T t1, T t2, T t3) {
    const T huge = static_cast<T>(1.e10);
    const T sqrt1_2 = static_cast<T>(0.70710678118654752440);
    T tUpd;
    T t0x = t1 + h * dmin(s0, s3);
    T t0z = t3 + h * dmin(s0, s1);
    T t0Update1 = dmin(t0x, t0z);
    T hs0 = h * s0;
    T dTx = t3 - t2;
    T dTz = t1 - t2;
    T sx = sqrt1_2 * s0;
    T sz = sqrt1_2 * s0;
    if (abs(src.isx - ix) > radius || abs(src.isz - iz) > radius) {
        T t0a = huge;
        T deta = hs0 * hs0 - dTz * dTz;
        if (dTz >= 0 && deta >= 0 && dTz <= h * sz) t0a = t1 + h * dsqrt(deta);
        T t0b = huge;
        T detb = hs0 * hs0 - dTx * dTx;
        if (dTx >= 0 && detb >= 0 && dTx <= h * sx) t0b = t3 + h * dsqrt(detb);
        T t0Update2 = dmin(t0a, t0b);
        T dtCross = t1 - t3;
        T detc = 2 * (hs0 * hs0) - dtCross * dtCross;
        T t0Update3 = huge;
        if (dTx >= 0 && dTz >= 0 && detc > 0 && t3 <= t1 + hs0 && t1 <= t3 + hs0)
            t0Update3 = t2 + dsqrt(detc);
        tUpd = dmin(dmin(t0Update1, t0Update2), t0Update3);
    } else {
        T t0Update3 = huge;
        if (dTx >= 0 && dTz >= 0 && t1 < t3 + hs0 && t3 < t1 + hs0) {
            const T sSrc = src.sSrc;
            T dt0dx, dt0dz, t0;
            analyticTG2(ix, iz, h, h, src.xs, src.zs, sSrc, t0, dt0dx, dt0dz);
            T tau1 = t1 - analyticT2(ix + sg.ixShift, iz, h, h, src.xs, src.zs, sSrc);
            T tau2 = t2 - analyticT2(ix + sg.ixShift, iz + sg.izShift, h, h, src.xs, src.zs, sSrc);
            T tau3 = t3 - analyticT2(ix, iz + sg.izShift, h, h, src.xs, src.zs, sSrc);
            dt0dx = sg.signX * dt0dx;
            dt0dz = sg.signZ * dt0dz;
            T tauX = tau1 - tau3 + tau2;
            T tauZ = tau3 - tau1 + tau2;
            const T one = 1, two = 2, four = 4;
            T h2 = h * h;
            T a = one / h2;
            T b = two / h * (dt0dx + dt0dz) - two / h2 * tau2;
            T c = one / (two * h2) * (tauX * tauX + tauZ * tauZ) -
                  two / h * (dt0dx * tauX + dt0dz * tauZ) + two * (sSrc * sSrc - s0 * s0);
            T det = b * b - four * a * c;
            if (det >= 0) {
                T tau = (-b + dsqrt(det)) / (two * a);
                t0Update3 = t0 + tau;
            }
            if (t0Update3 < t1 || t0Update3 < t3) t0Update3 = huge;
        }
        tUpd = dmin(t0Update1, t0Update3);
    }
    return tUpd;
}

// 2D non-uniform update (solverUtilities2d.hpp:474-614).
template <class T>
__device__ __forceinline__ T fd2NonUniform(int radius, const Spacing2<T> &g, const SourceT<T> &src,
                                           const SweepSigns &sg, int ix, int iz, T s0, T s1, T s3,
                                           T t1, T t2, T t3) {
    const T huge = static_cast<T>(1.e10);
    const T dx = g.dx, dz = g.dz;
    T tUpd;
    T t0x = t1 + dx * dmin(s0, s3);
    T t0z = t3 + dz * dmin(s0, s1);
    T t0Update1 = dmin(t0x, t0z);
    T dTx = t3 - t2;
    T dTz = t1 - t2;
    T sx = g.cosTheta * s0;
    T sz = g.sinTheta * s0;
    T hxs0 = dx * s0;
    T hzs0 = dz * s0;
    if (abs(src.isx - ix) > radius || abs(src.isz - iz) > radius) {
        T t0a = huge;
        T deta = hzs0 * hzs0 - dTz * dTz;
        if (dTz >= 0 && deta >= 0 && dTz <= dz * sz) t0a = t1 + g.dx_dz * dsqrt(deta);
        T t0b = huge;
        T detb = hxs0 * hxs0 - dTx * dTx;
        if (dTx >= 0 && detb >= 0 && dTx <= dx * sx) t0b = t3 + g.dz_dx * dsqrt(detb);
        T t0Update2 = dmin(t0a, t0b);
        T dxdz = g.cosTheta * g.sinTheta;
        T tildeTx = t1 - t3 + t2;
        T tildeTz = t3 - t1 + t2;
        T dtCross = t1 - t3;
        T detc = hxs0 * hxs0 + hzs0 * hzs0 - dtCross * dtCross;
        T t0Update3 = huge;
        if (dTx >= 0 && dTz >= 0 && detc > 0 && t1 < t3 + hzs0 && t3 < t1 + hxs0) {
            t0Update3 = tildeTx * g.dz_dx + tildeTz * g.dx_dz + 2 * dsqrt(detc);
            t0Update3 = dxdz * t0Update3;
        }
        if (t0Update3 < 0) t0Update3 = huge;
        tUpd = dmin(dmin(t0Update1, t0Update2), t0Update3);
    } else {
        T t0Update3 = huge;
        if (dTx >= 0 && dTz >= 0 && t1 < t3 + hzs0 && t3 < t1 + hxs0) {
            const T sSrc = src.sSrc;
            T dt0dx, dt0dz, t0;
            analyticTG2(ix, iz, dx, dz, src.xs, src.zs, sSrc, t0, dt0dx, dt0dz);
            T tau1 = t1 - analyticT2(ix + sg.ixShift, iz, dx, dz, src.xs, src.zs, sSrc);
            T tau2 = t2 - analyticT2(ix + sg.ixShift, iz + sg.izShift, dx, dz, src.xs, src.zs, sSrc);
            T tau3 = t3 - analyticT2(ix, iz + sg.izShift, dx, dz, src.xs, src.zs, sSrc);
            dt0dx = sg.signX * dt0dx;
            dt0dz = sg.signZ * dt0dz;
            T tauX = tau1 - tau3 + tau2;
            T tauZ = tau3 - tau1 + tau2;
            const T one = 1, two = 2, four = 4;
            T hx2inv = one / (dx * dx);
            T hz2inv = one / (dz * dz);
            T dxinv = one / dx;
            T dzinv = one / dz;
            T a = hx2inv + hz2inv;
            T b = four * (dxinv * dt0dx + dzinv * dt0dz) - two * (tauX * hx2inv + tauZ * hz2inv);
            T c = (tauX * tauX) * hx2inv + (tauZ * tauZ) * hz2inv -
                  four * ((dt0dx * tauX) * dxinv + (dt0dz * tauZ) * dzinv) +
                  four * (sSrc * sSrc - s0 * s0);
            T det = b * b - four * a * c;
            if (det >= 0) {
                T tau = (-b + dsqrt(det)) / (two * a);
                t0Update3 = t0 + tau;
            }
            if (t0Update3 < t1 || t0Update3 < t3) t0Update3 = huge;
        }
        tUpd = dmin(t0Update1, t0Update3);
    }
    return tUpd;
}

}  // namespace eikx
