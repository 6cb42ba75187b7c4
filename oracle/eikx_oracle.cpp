// ORACLE — test infrastructure only.
//
// A CPU restatement of the reference's (uofuseismo/eikonalxx v0.2.0) level-set /
// fast-sweeping eikonal path, written for this project as the checker of the GPU
// kernels.  Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
// reference legs may load this library; the product path never does.
//
// Every function follows the reference's arithmetic in the same operation order so
// that, compiled with -O2 -ffp-contract=off (no FMA contraction) and IEEE sqrt, it is
// bit-identical to the reference's own code for the same inputs.  It is pinned
// against the reference itself (oracle/_ref, built from the reference's sources by
// oracle/build_ref.py) and against the golden vectors of the reference's tests
// (tests/golden/).
//
// Semantics of a solve (the reference's Solver2D::solve, src/solver2d.cpp:462-565,
// extended to 3D because Solver3D::solve is unfinished, src/solver3d.cpp:391-500):
//   1. T := HUGE (1e10), the 4 (2D) / 8 (3D) corners of the source cell := s_src*dist
//      (src/solver2d.cpp:61-105, src/solver3d.cpp:21-84);
//   2. one initialisation pass of all sweeps restricted to the source quadrant/octant
//      (getLoopLimits with source, solverUtilities3d.hpp:1075-1184);
//   3. nSweeps refinement iterations of all sweeps over the full grid; new: the solve
//      ends once each of the last 8 (3D) / 4 (2D) refinement sweeps decreased no node by
//      the tolerance or more.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <vector>

namespace {

constexpr double kHuge = 1.e10;  // include/private/solver3d.hpp:10

template <class T> inline T tmin(T a, T b) { return std::fmin(a, b); }
template <class T> inline T tmax(T a, T b) { return std::fmax(a, b); }

inline int clampi(int v, int lo, int hi) { return std::max(lo, std::min(hi, v)); }

//----------------------------------------------------------------------------//
//                                   3D                                       //
//----------------------------------------------------------------------------//

// Sweep e (0..7 = Sweep1..Sweep8): bit 0 flips x, bit 1 flips y, bit 2 flips z.
// getSweepFiniteDifferenceSigns, solverUtilities3d.hpp:843-925.
struct Sweep3 {
    int fx, fy, fz;            // 1 when the axis is swept in decreasing order
    int ixShift, iyShift, izShift;
    int signX, signY, signZ;
    explicit Sweep3(int e) {
        fx = e & 1; fy = (e >> 1) & 1; fz = (e >> 2) & 1;
        ixShift = fx ? 1 : -1; iyShift = fy ? 1 : -1; izShift = fz ? 1 : -1;
        signX = fx ? -1 : 1; signY = fy ? -1 : 1; signZ = fz ? -1 : 1;
    }
};

// computeAnalyticalTravelTime, solverUtilities3d.hpp:138-156 and :180-208.
template <class T>
T analyticT(int ix, int iy, int iz, T dx, T dy, T dz, T xs, T ys, T zs, T s) {
    T x = ix * dx, y = iy * dy, z = iz * dz;
    T ddx = x - xs, ddy = y - ys, ddz = z - zs;
    T dist = std::sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
    return s * dist;
}
template <class T>
void analyticTG(int ix, int iy, int iz, T dx, T dy, T dz, T xs, T ys, T zs, T s,
                T *t, T *gx, T *gy, T *gz) {
    T x = ix * dx, y = iy * dy, z = iz * dz;
    T ddx = x - xs, ddy = y - ys, ddz = z - zs;
    T dist = std::sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
    *t = s * dist;
    *gx = 0; *gy = 0; *gz = 0;
    if (dist > 0) {
        *gx = (s * ddx) / dist;
        *gy = (s * ddy) / dist;
        *gz = (s * ddz) / dist;
    }
}

struct Src3 {
    int isx, isy, isz;
    double xo, yo, zo;   // source offsets from the origin (m)
};
struct Grid3 {
    int nx, ny, nz;
    double dx, dy, dz;
};

// near_fp64 (FP32 sweeps; the GPU's eikx_options.near_fp64): the analytic factor of the
// factored branch in FP64.  D = |x - xs| and U = (x - xs) / D from FP64 offsets and
// spacing at the unclamped stencil positions; T0_k = s0 D_k in FP64, carried as the float
// pair hi = fl(T0_k), lo = fl(T0_k - hi); tau_k = fl(fl(t_k - hi_k) - lo_k), the gradient
// fl(s0 U) and the candidate fl(hi_0 + fl(correction + lo_0)); the quadratic solves stay
// in the sweep type.
struct FactorTerms {
    double d, ux, uy, uz;
};
inline FactorTerms factorTerms(const Grid3 &g, const Src3 &src, int ix, int iy, int iz) {
    const double ddx = ix * g.dx - src.xo, ddy = iy * g.dy - src.yo, ddz = iz * g.dz - src.zo;
    const double d = std::sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
    return {d, d > 0 ? ddx / d : 0.0, d > 0 ? ddy / d : 0.0, d > 0 ? ddz / d : 0.0};
}
// The node's float pair (hi0, lo0, returned through t0 / lo0), the gradient and tau_1..tau_7.
template <class T>
void factorFp64(const Grid3 &g, const Src3 &src, const Sweep3 &sw, int ix, int iy, int iz, T s0,
                T t1, T t2, T t3, T t4, T t5, T t6, T t7, T &t0, T &lo0, T &gx, T &gy, T &gz, T (&tau)[7]) {
    const double s = s0;
    const FactorTerms e0 = factorTerms(g, src, ix, iy, iz);
    const double T00 = s * e0.d;
    t0 = static_cast<T>(T00);
    lo0 = static_cast<T>(T00 - static_cast<double>(t0));
    gx = static_cast<T>(s * e0.ux);
    gy = static_cast<T>(s * e0.uy);
    gz = static_cast<T>(s * e0.uz);
    auto tauOf = [&](T t, int x, int y, int z) {
        const double T0k = s * factorTerms(g, src, x, y, z).d;
        const T hi = static_cast<T>(T0k), lo = static_cast<T>(T0k - static_cast<double>(hi));
        return static_cast<T>(static_cast<T>(t - hi) - lo);
    };
    const int xu = ix + sw.ixShift, yu = iy + sw.iyShift, zu = iz + sw.izShift;
    tau[0] = tauOf(t1, xu, iy, iz);
    tau[1] = tauOf(t2, xu, yu, iz);
    tau[2] = tauOf(t3, ix, yu, iz);
    tau[3] = tauOf(t4, ix, iy, zu);
    tau[4] = tauOf(t5, xu, iy, zu);
    tau[5] = tauOf(t6, xu, yu, zu);
    tau[6] = tauOf(t7, ix, yu, zu);
}

// Uniform-grid local solver, solverUtilities3d.hpp:258-558 (debug prints removed).
template <class T>
T fd3Uniform(int radius, T huge, T h, T sSrc, int ix, int iy, int iz, const Sweep3 &sw,
             const Src3 &src, T xs, T ys, T zs,
             T s0, T s1, T s2, T s3, T s4, T s5, T s7,
             T t1, T t2, T t3, T t4, T t5, T t6, T t7, const Grid3 *g64 = nullptr) {
    T tUpd = huge;
    T minS0S3 = tmin(s0, s3);
    T minS0S1 = tmin(s0, s1);
    T minS0S4 = tmin(s0, s4);
    T t1d1 = t1 + h * tmin(minS0S3, tmin(s4, s7));
    T t1d2 = t3 + h * tmin(minS0S4, tmin(s1, s5));
    T t1d3 = t4 + h * tmin(minS0S1, tmin(s2, s3));
    T t1d = tmin(tmin(t1d1, t1d2), t1d3);
    T hs03 = h * minS0S3;
    T hs01 = h * minS0S1;
    T hs04 = h * minS0S4;
    if (std::abs(src.isx - ix) > radius || std::abs(src.isy - iy) > radius ||
        std::abs(src.isz - iz) > radius) {
        T dtCrossXZ = t1 - t4;
        T detXZ = 2 * (hs03 * hs03) - dtCrossXZ * dtCrossXZ;
        T t2d1 = huge;
        if (detXZ > 0 && t4 <= t1 + hs03 && t1 <= t4 + hs03) t2d1 = t5 + std::sqrt(detXZ);
        T t2d = t2d1;
        T dtCrossYZ = t3 - t4;
        T detYZ = 2 * (hs01 * hs01) - dtCrossYZ * dtCrossYZ;
        T t2d2 = huge;
        if (detYZ > 0 && t3 <= t4 + hs01 && t4 <= t3 + hs01) t2d2 = t7 + std::sqrt(detYZ);
        t2d = tmin(t2d, t2d2);
        T dtCrossXY = t1 - t3;
        T detXY = 2 * (hs04 * hs04) - dtCrossXY * dtCrossXY;
        T t2d3 = huge;
        if (detXY > 0 && t3 <= t1 + hs04 && t1 <= t3 + hs04) t2d3 = t2 + std::sqrt(detXY);
        t2d = tmin(t2d, t2d3);
        T t3d = huge;
        if (tmin(t1d, t2d) > tmax(tmax(t1, t4), t3)) {
            constexpr T third = 0.33333333333333333333333;
            constexpr T half = 0.5;
            T Tx = t1 + half * (-t4 + t5 - t3 + t2) - t7 + t6;
            T Ty = t3 + half * (-t4 + t7 - t1 + t2) - t5 + t6;
            T Tz = t4 + half * (-t1 + t5 - t3 + t7) - t2 + t6;
            T det = 27 * (h * s0) * (h * s0) - (Tx - Ty) * (Tx - Ty) - (Tx - Tz) * (Tx - Tz) -
                    (Ty - Tz) * (Ty - Tz);
            if (det >= 0) t3d = third * ((Tx + Ty + Tz) + std::sqrt(det));
        }
        tUpd = tmin(t1d, tmin(t2d, t3d));
    } else {
        // Factored ("spherical") branch exactly as the reference ships it: T0 uses the
        // home-cell slowness s0 (solverUtilities3d.hpp:373-378).
        T t0, dt0dx, dt0dy, dt0dz;
        T tau1, tau2, tau3, tau4, tau5, tau6, tau7;
        T lo0 = 0;
        if (g64) {
            T tau[7];
            factorFp64<T>(*g64, src, sw, ix, iy, iz, s0, t1, t2, t3, t4, t5, t6, t7, t0, lo0, dt0dx, dt0dy, dt0dz, tau);
            tau1 = tau[0]; tau2 = tau[1]; tau3 = tau[2]; tau4 = tau[3]; tau5 = tau[4]; tau6 = tau[5]; tau7 = tau[6];
        } else {
            analyticTG(ix, iy, iz, h, h, h, xs, ys, zs, s0, &t0, &dt0dx, &dt0dy, &dt0dz);
            tau1 = t1 - analyticT(ix + sw.ixShift, iy, iz, h, h, h, xs, ys, zs, s0);
            tau2 = t2 - analyticT(ix + sw.ixShift, iy + sw.iyShift, iz, h, h, h, xs, ys, zs, s0);
            tau3 = t3 - analyticT(ix, iy + sw.iyShift, iz, h, h, h, xs, ys, zs, s0);
            tau4 = t4 - analyticT(ix, iy, iz + sw.izShift, h, h, h, xs, ys, zs, s0);
            tau5 = t5 - analyticT(ix + sw.ixShift, iy, iz + sw.izShift, h, h, h, xs, ys, zs, s0);
            tau6 = t6 - analyticT(ix + sw.ixShift, iy + sw.iyShift, iz + sw.izShift, h, h, h, xs, ys, zs, s0);
            tau7 = t7 - analyticT(ix, iy + sw.iyShift, iz + sw.izShift, h, h, h, xs, ys, zs, s0);
        }
        auto plusT0 = [&](T d) -> T { return g64 ? static_cast<T>(t0 + static_cast<T>(d + lo0)) : t0 + d; };
        dt0dx = sw.signX * dt0dx;
        dt0dy = sw.signY * dt0dy;
        dt0dz = sw.signZ * dt0dz;
        T dTauTxXZ = tau1 - tau4 + tau5;
        T dTauTzXZ = tau4 - tau1 + tau5;
        constexpr T half = 0.5;
        T hi = 1 / h;
        T h2inv = 1 / (h * h);
        T a = h2inv;
        T b = (2 * hi) * (dt0dx + dt0dz) - (2 * h2inv) * tau5;
        T c = (half * h2inv) * (dTauTxXZ * dTauTxXZ + dTauTzXZ * dTauTzXZ) -
              (2 * hi) * (dt0dx * dTauTxXZ + dt0dz * dTauTzXZ) +
              2 * (sSrc * sSrc - s0 * s0 + dt0dy * dt0dy);
        T detXZ = b * b - 4 * a * c;
        T tau = 0;
        T t2d1 = huge;
        if (detXZ > 0 && t4 <= t1 + hs03 && t1 <= t4 + hs03) {
            tau = (-b + std::sqrt(detXZ)) / (2 * a);
            t2d1 = plusT0(tau);
            if (t2d1 < t1 || t2d1 < t4) t2d1 = huge;
        }
        T t2d = t2d1;
        T dTauTyYZ = tau3 - tau4 + tau7;
        T dTauTzYZ = tau4 - tau3 + tau7;
        b = (2 * hi) * (dt0dy + dt0dz) - (2 * h2inv) * tau7;
        c = (half * h2inv) * (dTauTyYZ * dTauTyYZ + dTauTzYZ * dTauTzYZ) -
            (2 * hi) * (dt0dy * dTauTyYZ + dt0dz * dTauTzYZ) +
            2 * (sSrc * sSrc - s0 * s0 + dt0dx * dt0dx);
        T detYZ = b * b - 4 * a * c;
        T t2d2 = huge;
        if (detYZ >= 0 && t3 <= t4 + hs01 && t4 <= t3 + hs01) {
            tau = (-b + std::sqrt(detYZ)) / (2 * a);
            t2d2 = plusT0(tau);
            if (t2d2 < t3 || t2d2 < t4) t2d2 = huge;
        }
        t2d = tmin(t2d, t2d2);
        T dTauTxXY = tau1 - tau3 + tau2;
        T dTauTyXY = tau3 - tau1 + tau2;
        b = (2 * hi) * (dt0dx + dt0dy) - (2 * h2inv) * tau2;
        c = (half * h2inv) * (dTauTxXY * dTauTxXY + dTauTyXY * dTauTyXY) -
            (2 * hi) * (dt0dx * dTauTxXY + dt0dy * dTauTyXY) +
            2 * (sSrc * sSrc - s0 * s0 + dt0dz * dt0dz);
        T detXY = b * b - 4 * a * c;
        T t2d3 = huge;
        if (detXY >= 0 && t3 <= t1 + hs04 && t1 <= t3 + hs04) {
            tau = (-b + std::sqrt(detXY)) / (2 * a);
            t2d3 = plusT0(tau);
            if (t2d3 < t1 || t2d3 < t3) t2d3 = huge;
        }
        t2d = tmin(t2d, t2d3);
        T t3d = huge;
        if (tmin(t1d, t2d) > tmax(tmax(t1, t4), t3)) {
            T taux = tau1 + half * (-tau4 + tau5 - tau3 + tau2) - tau7 + tau6;
            T tauy = tau3 + half * (-tau4 + tau7 - tau1 + tau2) - tau5 + tau6;
            T tauz = tau4 + half * (-tau1 + tau5 - tau3 + tau7) - tau2 + tau6;
            a = 3 * h2inv;
            b = -2 * h2inv * (taux + tauy + tauz) + (6 * hi) * (dt0dx + dt0dy + dt0dz);
            c = h2inv * (taux * taux + tauy * tauy + tauz * tauz) -
                (6 * hi) * (dt0dx * taux + dt0dy * tauy + dt0dz * tauz) +
                9 * (sSrc * sSrc - s0 * s0);
            T det = b * b - 4 * a * c;
            if (det >= 0) t3d = plusT0((-b + std::sqrt(det)) / (2 * a));
            if (t3d < t1 || t3d < t3 || t3d < t4) t3d = huge;
        }
        tUpd = tmin(t1d, tmin(t2d, t3d));
    }
    return tUpd;
}

// Non-uniform-grid local solver, solverUtilities3d.hpp:562-824.
template <class T>
struct NonUniform3 {
    T dx, dy, dz, dxInv, dyInv, dzInv, dx2Inv, dy2Inv, dz2Inv;
    T dx_dz, dz_dx, dy_dz, dz_dy, dx_dy, dy_dx;
    T dx2_p_dz2_inv, dy2_p_dz2_inv, dx2_p_dy2_inv;
    NonUniform3(T dx_, T dy_, T dz_) {
        // include/private/solver3d.hpp:247-261
        dx = dx_; dy = dy_; dz = dz_;
        dxInv = 1 / dx; dyInv = 1 / dy; dzInv = 1 / dz;
        dx2Inv = 1 / (dx * dx); dy2Inv = 1 / (dy * dy); dz2Inv = 1 / (dz * dz);
        dx_dz = dx / dz; dz_dx = dz / dx; dy_dz = dy / dz; dz_dy = dz / dy;
        dx_dy = dx / dy; dy_dx = dy / dx;
        dx2_p_dz2_inv = 1 / (dx * dx + dz * dz);
        dy2_p_dz2_inv = 1 / (dy * dy + dz * dz);
        dx2_p_dy2_inv = 1 / (dx * dx + dy * dy);
    }
};

template <class T>
T fd3NonUniform(int radius, T huge, const NonUniform3<T> &g, T sSrc, int ix, int iy, int iz,
                const Sweep3 &sw, const Src3 &src, T xs, T ys, T zs,
                T s0, T s1, T s2, T s3, T s4, T s5, T s7,
                T t1, T t2, T t3, T t4, T t5, T t6, T t7, const Grid3 *g64 = nullptr) {
    const T dx = g.dx, dy = g.dy, dz = g.dz;
    T tUpd = huge;
    T minS0S3 = tmin(s0, s3);
    T minS0S1 = tmin(s0, s1);
    T minS0S4 = tmin(s0, s4);
    T t1d1 = t1 + dx * tmin(minS0S3, tmin(s4, s7));
    T t1d2 = t3 + dy * tmin(minS0S4, tmin(s1, s5));
    T t1d3 = t4 + dz * tmin(minS0S1, tmin(s2, s3));
    T t1d = tmin(tmin(t1d1, t1d2), t1d3);
    if (std::abs(src.isx - ix) > radius || std::abs(src.isy - iy) > radius ||
        std::abs(src.isz - iz) > radius) {
        T dtCrossXZ = t1 - t4;
        T detXZ = (dx * dx + dz * dz) * (minS0S3 * minS0S3) - dtCrossXZ * dtCrossXZ;
        T t2d1 = huge;
        if (detXZ > 0 && t1 < t4 + dz * minS0S3 && t4 < t1 + dx * minS0S3) {
            T TxXZ = t1 - t4 + t5;
            T TzXZ = t4 - t1 + t5;
            t2d1 = (TxXZ * g.dz_dx + TzXZ * g.dx_dz) + 2 * std::sqrt(detXZ);
            t2d1 = ((dx * dz) * g.dx2_p_dz2_inv) * t2d1;
        }
        T t2d = t2d1;
        T dtCrossYZ = t3 - t4;
        T detYZ = (dy * dy + dz * dz) * (minS0S1 * minS0S1) - dtCrossYZ * dtCrossYZ;
        T t2d2 = huge;
        if (detYZ > 0 && t3 < t4 + dz * minS0S1 && t4 < t3 + dy * minS0S1) {
            T TyYZ = t3 - t4 + t7;
            T TzYZ = t4 - t3 + t7;
            t2d2 = (TyYZ * g.dz_dy + TzYZ * g.dy_dz) + 2 * std::sqrt(detYZ);
            t2d2 = ((dy * dz) * g.dy2_p_dz2_inv) * t2d2;
        }
        t2d = tmin(t2d, t2d2);
        T dtCrossXY = t1 - t3;
        T detXY = (dx * dx + dy * dy) * (minS0S4 * minS0S4) - dtCrossXY * dtCrossXY;
        T t2d3 = huge;
        if (detXY > 0 && t3 < t1 + dx * minS0S4 && t1 < t3 + dy * minS0S4) {
            T TxXY = t1 - t3 + t2;
            T TyXY = t3 - t1 + t2;
            t2d3 = (TxXY * g.dy_dx + TyXY * g.dx_dy) + 2 * std::sqrt(detXY);
            t2d3 = ((dx * dy) * g.dx2_p_dy2_inv) * t2d3;
        }
        t2d = tmin(t2d, t2d3);
        T t3d = huge;
        if (tmin(t1d, t2d) > tmax(tmax(t1, t4), t3)) {
            constexpr T half = 0.5;
            T Tx = t1 + half * (-t4 + t5 - t3 + t2) - t7 + t6;
            T Ty = t3 + half * (-t4 + t7 - t1 + t2) - t5 + t6;
            T Tz = t4 + half * (-t1 + t5 - t3 + t7) - t2 + t6;
            T det = 9 * (s0 * s0) * (g.dx2Inv + g.dy2Inv + g.dz2Inv) -
                    ((Tx - Tz) * (Tx - Tz)) * (g.dx2Inv * g.dz2Inv) -
                    ((Ty - Tz) * (Ty - Tz)) * (g.dy2Inv * g.dz2Inv) -
                    ((Tx - Ty) * (Tx - Ty)) * (g.dx2Inv * g.dy2Inv);
            if (det >= 0)
                t3d = (Tx * g.dx2Inv + Ty * g.dy2Inv + Tz * g.dz2Inv + std::sqrt(det)) /
                      (g.dx2Inv + g.dy2Inv + g.dz2Inv);
        }
        tUpd = tmin(t1d, tmin(t2d, t3d));
    } else {
        T t0, dt0dx, dt0dy, dt0dz;
        T tau1, tau2, tau3, tau4, tau5, tau6, tau7;
        T lo0 = 0;
        if (g64) {
            T tau[7];
            factorFp64<T>(*g64, src, sw, ix, iy, iz, s0, t1, t2, t3, t4, t5, t6, t7, t0, lo0, dt0dx, dt0dy, dt0dz, tau);
            tau1 = tau[0]; tau2 = tau[1]; tau3 = tau[2]; tau4 = tau[3]; tau5 = tau[4]; tau6 = tau[5]; tau7 = tau[6];
        } else {
            analyticTG(ix, iy, iz, dx, dy, dz, xs, ys, zs, s0, &t0, &dt0dx, &dt0dy, &dt0dz);
            tau1 = t1 - analyticT(ix + sw.ixShift, iy, iz, dx, dy, dz, xs, ys, zs, s0);
            tau2 = t2 - analyticT(ix + sw.ixShift, iy + sw.iyShift, iz, dx, dy, dz, xs, ys, zs, s0);
            tau3 = t3 - analyticT(ix, iy + sw.iyShift, iz, dx, dy, dz, xs, ys, zs, s0);
            tau4 = t4 - analyticT(ix, iy, iz + sw.izShift, dx, dy, dz, xs, ys, zs, s0);
            tau5 = t5 - analyticT(ix + sw.ixShift, iy, iz + sw.izShift, dx, dy, dz, xs, ys, zs, s0);
            tau6 = t6 - analyticT(ix + sw.ixShift, iy + sw.iyShift, iz + sw.izShift, dx, dy, dz, xs, ys, zs, s0);
            tau7 = t7 - analyticT(ix, iy + sw.iyShift, iz + sw.izShift, dx, dy, dz, xs, ys, zs, s0);
        }
        auto plusT0 = [&](T d) -> T { return g64 ? static_cast<T>(t0 + static_cast<T>(d + lo0)) : t0 + d; };
        dt0dx = sw.signX * dt0dx;
        dt0dy = sw.signY * dt0dy;
        dt0dz = sw.signZ * dt0dz;
        const T dxInv = g.dxInv, dyInv = g.dyInv, dzInv = g.dzInv;
        const T dx2Inv = g.dx2Inv, dy2Inv = g.dy2Inv, dz2Inv = g.dz2Inv;
        T dTauTxXZ = tau1 - tau4 + tau5;
        T dTauTzXZ = tau4 - tau1 + tau5;
        T a = dx2Inv + dz2Inv;
        T b = 4 * (dxInv * dt0dx + dzInv * dt0dz) - 2 * (dTauTxXZ * dx2Inv + dTauTzXZ * dz2Inv);
        T c = (dTauTxXZ * dTauTxXZ) * dx2Inv + (dTauTzXZ * dTauTzXZ) * dz2Inv -
              4 * ((dt0dx * dTauTxXZ) * dxInv + (dt0dz * dTauTzXZ) * dzInv) +
              4 * (sSrc * sSrc - s0 * s0 + dt0dy * dt0dy);
        T detXZ = b * b - 4 * a * c;
        T t2d1 = huge;
        if (detXZ > 0 && t1 < t4 + dz * minS0S3 && t4 < t1 + dx * minS0S3) {
            t2d1 = plusT0((-b + std::sqrt(detXZ)) / (2 * a));
            if (t2d1 < t1 || t2d1 < t4) t2d1 = huge;
        }
        T t2d = t2d1;
        T dTauTyYZ = tau3 - tau4 + tau7;
        T dTauTzYZ = tau4 - tau3 + tau7;
        a = dy2Inv + dz2Inv;
        b = 4 * (dyInv * dt0dy + dzInv * dt0dz) - 2 * (dTauTyYZ * dy2Inv + dTauTzYZ * dz2Inv);
        c = (dTauTyYZ * dTauTyYZ) * dy2Inv + (dTauTzYZ * dTauTzYZ) * dz2Inv -
            4 * ((dt0dy * dTauTyYZ) * dyInv + (dt0dz * dTauTzYZ) * dzInv) +
            4 * (sSrc * sSrc - s0 * s0 + dt0dx * dt0dx);
        T detYZ = b * b - 4 * a * c;
        T t2d2 = huge;
        if (detYZ > 0 && t3 < t4 + dz * minS0S1 && t4 < t3 + dy * minS0S1) {
            t2d2 = plusT0((-b + std::sqrt(detYZ)) / (2 * a));
            if (t2d2 < t3 || t2d2 < t4) t2d2 = huge;
        }
        t2d = tmin(t2d, t2d2);
        T dTauTxXY = tau1 - tau3 + tau2;
        T dTauTyXY = tau3 - tau1 + tau2;
        a = dx2Inv + dy2Inv;
        b = 4 * (dxInv * dt0dx + dyInv * dt0dy) - 2 * (dTauTxXY * dx2Inv + dTauTyXY * dy2Inv);
        c = (dTauTxXY * dTauTxXY) * dx2Inv + (dTauTyXY * dTauTyXY) * dy2Inv -
            4 * ((dt0dx * dTauTxXY) * dxInv + (dt0dy * dTauTyXY) * dyInv) +
            4 * (sSrc * sSrc - s0 * s0 + dt0dz * dt0dz);
        T detXY = b * b - 4 * a * c;
        T t2d3 = huge;
        if (detXY > 0 && t3 < t1 + dx * minS0S4 && t1 < t3 + dy * minS0S4) {
            t2d3 = plusT0((-b + std::sqrt(detXY)) / (2 * a));
            if (t2d3 < t1 || t2d3 < t3) t2d3 = huge;
        }
        t2d = tmin(t2d, t2d3);
        T t3d = huge;
        if (tmin(t1d, t2d) > tmax(tmax(t1, t4), t3)) {
            constexpr T half = 0.5;
            T taux = tau1 + half * (-tau4 + tau5 - tau3 + tau2) - tau7 + tau6;
            T tauy = tau3 + half * (-tau4 + tau7 - tau1 + tau2) - tau5 + tau6;
            T tauz = tau4 + half * (-tau1 + tau5 - tau3 + tau7) - tau2 + tau6;
            a = dx2Inv + dy2Inv + dz2Inv;
            b = -2 * (taux * dx2Inv + tauy * dy2Inv + tauz * dz2Inv) +
                6 * (dxInv * dt0dx + dyInv * dt0dy + dzInv * dt0dz);
            c = (taux * taux) * dx2Inv + (tauy * tauy) * dy2Inv + (tauz * tauz) * dz2Inv -
                6 * (dt0dx * taux * dxInv + dt0dy * tauy * dyInv + dt0dz * tauz * dzInv) +
                9 * (sSrc * sSrc - s0 * s0);
            T det = b * b - 4 * a * c;
            if (det >= 0) t3d = plusT0((-b + std::sqrt(det)) / (2 * a));
            if (t3d < t1 || t3d < t3 || t3d < t4) t3d = huge;
        }
        tUpd = tmin(t1d, tmin(t2d, t3d));
    }
    return tUpd;
}


// getLoopLimits (full, solverUtilities3d.hpp:944-1052) and the source-limited
// variant used by the initialisation sweeps (:1075-1184), both expressed as
// [first, stop) with a direction.
void loopLimits3(const Grid3 &g, const Sweep3 &sw, bool init, const Src3 &src,
                 int *x0, int *x1, int *dx, int *y0, int *y1, int *dy, int *z0, int *z1,
                 int *dz) {
    auto axis = [&](int n, int flip, int is, int *a0, int *a1, int *ad) {
        if (!flip) {
            *a0 = init ? std::max(1, is) : 1;
            *a1 = n;
            *ad = 1;
        } else {
            *a0 = init ? std::min(is + 1, n - 2) : n - 2;
            *a1 = -1;
            *ad = -1;
        }
    };
    axis(g.nx, sw.fx, src.isx, x0, x1, dx);
    axis(g.ny, sw.fy, src.isy, y0, y1, dy);
    axis(g.nz, sw.fz, src.isz, z0, z1, dz);
}

// Solver3DSweep<T,E>::updateFSM, include/private/solver3d.hpp:150-326, with the
// stencil addressing of gridToSurroundingSlownessIndices (:1300-1442) and
// gridToSurroundingTravelTimeIndices (:1460-1586).  Returns the largest decrease.
// near_fp64 (FP32 solves): the analytic factor of the factored branch in FP64 -- the
// GPU's eikx_options.near_fp64 (factorFp64 below).
int gNearFp64 = 0;

template <class T>
double sweep3(int e, bool init, const Grid3 &g, int radius, const Src3 &src, T sSrc,
              const T *slow, T *tt) {
    Sweep3 sw(e);
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int ncx = nx - 1, ncy = ny - 1, ncz = nz - 1;
    int x0, x1, xd, y0, y1, yd, z0, z1, zd;
    loopLimits3(g, sw, init, src, &x0, &x1, &xd, &y0, &y1, &yd, &z0, &z1, &zd);
    const T huge = static_cast<T>(kHuge);
    const T xs = static_cast<T>(src.xo), ys = static_cast<T>(src.yo), zs = static_cast<T>(src.zo);
    const double eps = std::numeric_limits<T>::epsilon() * 100;
    const bool uniform = std::abs(g.dx - g.dy) < eps && std::abs(g.dx - g.dz) < eps;
    const T h = static_cast<T>(g.dx);
    NonUniform3<T> nu(static_cast<T>(g.dx), static_cast<T>(g.dy), static_cast<T>(g.dz));
    double diffMax = 0;
    auto cidx = [&](int cx, int cy, int cz) {
        return static_cast<size_t>(cz) * ncx * ncy + static_cast<size_t>(cy) * ncx + cx;
    };
    auto gidx = [&](int ix, int iy, int iz) {
        return static_cast<size_t>(iz) * nx * ny + static_cast<size_t>(iy) * nx + ix;
    };
    for (int iz = z0; iz != z1; iz += zd) {
        for (int iy = y0; iy != y1; iy += yd) {
            for (int ix = x0; ix != x1; ix += xd) {
                // cell indices: increasing axis -> update cell = i-1, offset = update+1;
                // decreasing axis -> update cell = i, offset = update-1; all clamped.
                int cxu = sw.fx ? clampi(ix, 0, ncx - 1) : clampi(ix - 1, 0, ncx - 1);
                int cxo = sw.fx ? clampi(cxu - 1, 0, ncx - 1) : clampi(cxu + 1, 0, ncx - 1);
                int cyu = sw.fy ? clampi(iy, 0, ncy - 1) : clampi(iy - 1, 0, ncy - 1);
                int cyo = sw.fy ? clampi(cyu - 1, 0, ncy - 1) : clampi(cyu + 1, 0, ncy - 1);
                int czu = sw.fz ? clampi(iz, 0, ncz - 1) : clampi(iz - 1, 0, ncz - 1);
                int czo = sw.fz ? clampi(czu - 1, 0, ncz - 1) : clampi(czu + 1, 0, ncz - 1);
                T s0 = slow[cidx(cxu, cyu, czu)];
                T s1 = slow[cidx(cxo, cyu, czu)];
                T s2 = slow[cidx(cxo, cyo, czu)];
                T s3 = slow[cidx(cxu, cyo, czu)];
                T s4 = slow[cidx(cxu, cyu, czo)];
                T s5 = slow[cidx(cxo, cyu, czo)];
                T s7 = slow[cidx(cxu, cyo, czo)];
                int xsft = clampi(ix + sw.ixShift, 0, nx - 1);
                int ysft = clampi(iy + sw.iyShift, 0, ny - 1);
                int zsft = clampi(iz + sw.izShift, 0, nz - 1);
                size_t i0 = gidx(ix, iy, iz);
                T t0 = tt[i0];
                T t1 = tt[gidx(xsft, iy, iz)];
                T t2 = tt[gidx(xsft, ysft, iz)];
                T t3 = tt[gidx(ix, ysft, iz)];
                T t4 = tt[gidx(ix, iy, zsft)];
                T t5 = tt[gidx(xsft, iy, zsft)];
                T t6 = tt[gidx(xsft, ysft, zsft)];
                T t7 = tt[gidx(ix, ysft, zsft)];
                // near_fp64 (FP32 sweeps): the analytic factor in FP64
                const Grid3 *g64 = gNearFp64 && sizeof(T) == 4 ? &g : nullptr;
                T tUpd = uniform
                    ? fd3Uniform<T>(radius, huge, h, sSrc, ix, iy, iz, sw, src, xs, ys, zs,
                                    s0, s1, s2, s3, s4, s5, s7, t1, t2, t3, t4, t5, t6, t7, g64)
                    : fd3NonUniform<T>(radius, huge, nu, sSrc, ix, iy, iz, sw, src, xs, ys, zs,
                                       s0, s1, s2, s3, s4, s5, s7, t1, t2, t3, t4, t5, t6, t7, g64);
                if (tUpd < t0) {
                    tt[i0] = tUpd;
                    // decrease formed in T (exact by Sterbenz whenever it is below t0/2),
                    // maximum kept in FP64 -- as the GPU kernels do
                    diffMax = std::max(diffMax, static_cast<double>(static_cast<T>(t0 - tUpd)));
                }
            }
        }
    }
    return diffMax;
}

// Solver3D::initializeTravelTimes, src/solver3d.cpp:21-84.  initFp64 computes the
// eight corner times in double precision before rounding to T (the GPU default);
// otherwise they are computed in T as the reference does.
template <class T>
void init3(const Grid3 &g, const Src3 &src, const T *slow, bool initFp64, T *tt) {
    const size_t n = static_cast<size_t>(g.nx) * g.ny * g.nz;
    std::fill(tt, tt + n, static_cast<T>(kHuge));
    const int ncx = g.nx - 1, ncy = g.ny - 1;
    const size_t scell = static_cast<size_t>(src.isz) * ncx * ncy + static_cast<size_t>(src.isy) * ncx + src.isx;
    for (int k = 0; k < 2; ++k)
        for (int j = 0; j < 2; ++j)
            for (int i = 0; i < 2; ++i) {
                int ix = src.isx + i, iy = src.isy + j, iz = src.isz + k;
                size_t idx = static_cast<size_t>(iz) * g.nx * g.ny + static_cast<size_t>(iy) * g.nx + ix;
                if (initFp64) {
                    tt[idx] = static_cast<T>(analyticT<double>(
                        ix, iy, iz, g.dx, g.dy, g.dz, src.xo, src.yo, src.zo,
                        static_cast<double>(slow[scell])));
                } else {
                    tt[idx] = analyticT<T>(ix, iy, iz, static_cast<T>(g.dx), static_cast<T>(g.dy),
                                           static_cast<T>(g.dz), static_cast<T>(src.xo),
                                           static_cast<T>(src.yo), static_cast<T>(src.zo), slow[scell]);
                }
            }
}

template <class T>
int solve3(const Grid3 &g, const Src3 &src, const T *slow, int nSweeps, int radius,
           double tol, int initFp64, int doInitSweeps, T *tt, double *residuals, int *nIter) {
    init3<T>(g, src, slow, initFp64 != 0, tt);
    const int ncx = g.nx - 1, ncy = g.ny - 1;
    T sSrc = slow[static_cast<size_t>(src.isz) * ncx * ncy + static_cast<size_t>(src.isy) * ncx + src.isx];
    if (doInitSweeps)
        for (int e = 0; e < 8; ++e) sweep3<T>(e, true, g, radius, src, sSrc, slow, tt);
    // the solve ends once each of the last 8 refinement sweeps (a window that may span two
    // iterations) decreased no node by tol or more; *nIter = refinement iterations begun
    int k = 0, quiet = 0;
    bool done = false;
    for (; k < nSweeps && !done; ++k) {
        for (int e = 0; e < 8; ++e) {
            double r = sweep3<T>(e, false, g, radius, src, sSrc, slow, tt);
            if (residuals) residuals[k * 8 + e] = r;
            quiet = r < tol ? quiet + 1 : 0;
            if (quiet >= 8) {
                done = true;
                break;
            }
        }
    }
    if (nIter) *nIter = k;
    return 0;
}

// solve3 in pieces, for the CPU baselines, which time real cold-start solves a bounded
// number of sweeps at a time.  *pos counts the schedule sweeps done (0 = not started:
// the field is initialised first; then the 8 initialisation sweeps, then refinement
// sweeps), *quiet the current run of refinement sweeps that decreased no node by tol or
// more.  Runs at most maxSweeps more sweeps of the schedule; returns 1 once the solve has
// ended (the convergence rule of solve3, or nSweeps iterations), else 0.  Run to the end,
// the field is solve3's, bit for bit.
template <class T>
int advance3(const Grid3 &g, const Src3 &src, const T *slow, int nSweeps, int radius, double tol, int initFp64,
             T *tt, int *pos, int *quiet, int maxSweeps) {
    const int ncx = g.nx - 1, ncy = g.ny - 1;
    const T sSrc = slow[static_cast<size_t>(src.isz) * ncx * ncy + static_cast<size_t>(src.isy) * ncx + src.isx];
    if (*pos == 0) {
        init3<T>(g, src, slow, initFp64 != 0, tt);
        *quiet = 0;
    }
    const int total = 8 * (1 + nSweeps);
    for (int n = 0; n < maxSweeps && *pos < total && *quiet < 8; ++n) {
        const int e = *pos % 8;
        if (*pos < 8) {
            sweep3<T>(e, true, g, radius, src, sSrc, slow, tt);
        } else {
            const double r = sweep3<T>(e, false, g, radius, src, sSrc, slow, tt);
            *quiet = r < tol ? *quiet + 1 : 0;
        }
        ++*pos;
    }
    return (*pos >= total || *quiet >= 8) ? 1 : 0;
}

//----------------------------------------------------------------------------//
//                                   2D                                       //
//----------------------------------------------------------------------------//

// A hypot shared with the GPU kernels so both sides round identically: Borges,
// "An Improved Algorithm for hypot(a,b)", arXiv:1904.09481 (2019), the fused
// correction step, with std::fma as the exact fused multiply-add.
inline double eikxHypot(double a, double b) {
    a = std::fabs(a); b = std::fabs(b);
    if (a < b) std::swap(a, b);
    if (b == 0) return a;
    double h = std::sqrt(std::fma(a, a, b * b));
    double h2 = h * h;
    double a2 = a * a;
    double x = std::fma(-b, b, h2 - a2) + std::fma(h, h, -h2) - std::fma(a, a, -a2);
    return h - x / (2 * h);
}
inline float eikxHypot(float a, float b) {
    // Exact in double then a single rounding: the float result is correctly rounded
    // except in double-rounding corner cases, identically on both sides.
    double da = a, db = b;
    return static_cast<float>(std::sqrt(da * da + db * db));
}

// Which hypot the 2D analytic times use: 0 = std::hypot (what the reference calls,
// for pinning against oracle/_ref), 1 = eikxHypot (what the GPU kernels call).
int gHypotMode = 1;
template <class T> inline T hypot2(T a, T b) {
    return gHypotMode ? eikxHypot(a, b) : std::hypot(a, b);
}

// 2D analytic times, solverUtilities2d.hpp:159-215.
template <class T>
T analyticT2(int ix, int iz, T dx, T dz, T xs, T zs, T s) {
    T x = ix * dx, z = iz * dz;
    T ddx = x - xs, ddz = z - zs;
    T dist = hypot2(ddx, ddz);
    return s * dist;
}
template <class T>
void analyticTG2(int ix, int iz, T dx, T dz, T xs, T zs, T s, T *t, T *gx, T *gz) {
    T x = ix * dx, z = iz * dz;
    T ddx = x - xs, ddz = z - zs;
    T dist = hypot2(ddx, ddz);
    *t = s * dist;
    *gx = 0; *gz = 0;
    if (dist > 0) {
        *gx = (s * ddx) / dist;
        *gz = (s * ddz) / dist;
    }
}

struct Sweep2 {
    int fx, fz, ixShift, izShift, signX, signZ;
    explicit Sweep2(int e) {
        // getSweepFiniteDifferenceSigns 2D, solverUtilities2d.hpp:888-926
        fx = e & 1; fz = (e >> 1) & 1;
        ixShift = fx ? 1 : -1; izShift = fz ? 1 : -1;
        signX = fx ? -1 : 1; signZ = fz ? -1 : 1;
    }
};

struct Src2 {
    int isx, isz;
    double xo, zo;
};

constexpr double kSqrt1_2 = 0.70710678118654752440;  // M_SQRT1_2

// Uniform 2D local solver, solverUtilities2d.hpp:347-472.
template <class T>
T fd2Uniform(int radius, T huge, T h, T sSrc, int ix, int iz, const Sweep2 &sw,
             const Src2 &src, T xs, T zs, T s0, T s1, T s3, T t1, T t2, T t3) {
    T tUpd = huge;
    T t0x = t1 + h * tmin(s0, s3);
    T t0z = t3 + h * tmin(s0, s1);
    T t0Update1 = tmin(t0x, t0z);
    T hs0 = h * s0;
    T dTx = t3 - t2;
    T dTz = t1 - t2;
    T sx = static_cast<T>(kSqrt1_2) * s0;
    T sz = static_cast<T>(kSqrt1_2) * s0;
    if (std::abs(src.isx - ix) > radius || std::abs(src.isz - iz) > radius) {
        T t0a = huge;
        T deta = hs0 * hs0 - dTz * dTz;
        if (dTz >= 0 && deta >= 0 && dTz <= h * sz) t0a = t1 + h * std::sqrt(deta);
        T t0b = huge;
        T detb = hs0 * hs0 - dTx * dTx;
        if (dTx >= 0 && detb >= 0 && dTx <= h * sx) t0b = t3 + h * std::sqrt(detb);
        T t0Update2 = tmin(t0a, t0b);
        T dtCross = t1 - t3;
        T detc = 2 * (hs0 * hs0) - dtCross * dtCross;
        T t0Update3 = huge;
        if (dTx >= 0 && dTz >= 0 && detc > 0 && t3 <= t1 + hs0 && t1 <= t3 + hs0)
            t0Update3 = t2 + std::sqrt(detc);
        tUpd = tmin(tmin(t0Update1, t0Update2), t0Update3);
    } else {
        T t0Update3 = huge;
        if (dTx >= 0 && dTz >= 0 && t1 < t3 + hs0 && t3 < t1 + hs0) {
            T dt0dx, dt0dz, t0;
            analyticTG2(ix, iz, h, h, xs, zs, sSrc, &t0, &dt0dx, &dt0dz);
            T tau1 = t1 - analyticT2(ix + sw.ixShift, iz, h, h, xs, zs, sSrc);
            T tau2 = t2 - analyticT2(ix + sw.ixShift, iz + sw.izShift, h, h, xs, zs, sSrc);
            T tau3 = t3 - analyticT2(ix, iz + sw.izShift, h, h, xs, zs, sSrc);
            dt0dx = sw.signX * dt0dx;
            dt0dz = sw.signZ * dt0dz;
            T tauX = tau1 - tau3 + tau2;
            T tauZ = tau3 - tau1 + tau2;
            constexpr T one = 1, two = 2, four = 4;
            T h2 = h * h;
            T a = one / h2;
            T b = two / h * (dt0dx + dt0dz) - two / h2 * tau2;
            T c = one / (two * h2) * (tauX * tauX + tauZ * tauZ) -
                  two / h * (dt0dx * tauX + dt0dz * tauZ) + two * (sSrc * sSrc - s0 * s0);
            T det = b * b - four * a * c;
            if (det >= 0) {
                T tau = (-b + std::sqrt(det)) / (two * a);
                t0Update3 = t0 + tau;
            }
            if (t0Update3 < t1 || t0Update3 < t3) t0Update3 = huge;
        }
        tUpd = tmin(t0Update1, t0Update3);
    }
    return tUpd;
}

template <class T>
struct NonUniform2 {
    T dx, dz, dx_dz, dz_dx, cosTheta, sinTheta;
};

// Non-uniform 2D local solver, solverUtilities2d.hpp:474-614.
template <class T>
T fd2NonUniform(int radius, T huge, const NonUniform2<T> &g, T sSrc, int ix, int iz,
                const Sweep2 &sw, const Src2 &src, T xs, T zs, T s0, T s1, T s3, T t1,
                T t2, T t3) {
    const T dx = g.dx, dz = g.dz;
    T tUpd = huge;
    T t0x = t1 + dx * tmin(s0, s3);
    T t0z = t3 + dz * tmin(s0, s1);
    T t0Update1 = tmin(t0x, t0z);
    T dTx = t3 - t2;
    T dTz = t1 - t2;
    T sx = g.cosTheta * s0;
    T sz = g.sinTheta * s0;
    T hxs0 = dx * s0;
    T hzs0 = dz * s0;
    if (std::abs(src.isx - ix) > radius || std::abs(src.isz - iz) > radius) {
        T t0a = huge;
        T deta = hzs0 * hzs0 - dTz * dTz;
        if (dTz >= 0 && deta >= 0 && dTz <= dz * sz) t0a = t1 + g.dx_dz * std::sqrt(deta);
        T t0b = huge;
        T detb = hxs0 * hxs0 - dTx * dTx;
        if (dTx >= 0 && detb >= 0 && dTx <= dx * sx) t0b = t3 + g.dz_dx * std::sqrt(detb);
        T t0Update2 = tmin(t0a, t0b);
        T dxdz_dx2_p_dz2 = g.cosTheta * g.sinTheta;
        T tildeTx = t1 - t3 + t2;
        T tildeTz = t3 - t1 + t2;
        T dtCross = t1 - t3;
        T detc = hxs0 * hxs0 + hzs0 * hzs0 - dtCross * dtCross;
        T t0Update3 = huge;
        if (dTx >= 0 && dTz >= 0 && detc > 0 && t1 < t3 + hzs0 && t3 < t1 + hxs0) {
            t0Update3 = tildeTx * g.dz_dx + tildeTz * g.dx_dz + 2 * std::sqrt(detc);
            t0Update3 = dxdz_dx2_p_dz2 * t0Update3;
        }
        if (t0Update3 < 0) t0Update3 = huge;
        tUpd = tmin(tmin(t0Update1, t0Update2), t0Update3);
    } else {
        T t0Update3 = huge;
        if (dTx >= 0 && dTz >= 0 && t1 < t3 + hzs0 && t3 < t1 + hxs0) {
            T dt0dx, dt0dz, t0;
            analyticTG2(ix, iz, dx, dz, xs, zs, sSrc, &t0, &dt0dx, &dt0dz);
            T tau1 = t1 - analyticT2(ix + sw.ixShift, iz, dx, dz, xs, zs, sSrc);
            T tau2 = t2 - analyticT2(ix + sw.ixShift, iz + sw.izShift, dx, dz, xs, zs, sSrc);
            T tau3 = t3 - analyticT2(ix, iz + sw.izShift, dx, dz, xs, zs, sSrc);
            dt0dx = sw.signX * dt0dx;
            dt0dz = sw.signZ * dt0dz;
            T tauX = tau1 - tau3 + tau2;
            T tauZ = tau3 - tau1 + tau2;
            constexpr T one = 1, two = 2, four = 4;
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
                T tau = (-b + std::sqrt(det)) / (two * a);
                t0Update3 = t0 + tau;
            }
            if (t0Update3 < t1 || t0Update3 < t3) t0Update3 = huge;
        }
        tUpd = tmin(t0Update1, t0Update3);
    }
    return tUpd;
}

struct Grid2 {
    int nx, nz;
    double dx, dz;
};

// Solver2DSweep<T,E>::updateFSM, include/private/solver2d.hpp:203-327, with
// gridToSurroundingSlowness (solverUtilities2d.hpp:1279-1370) and the unclamped
// gridToSurroundingTravelTimes (:1383-1422).
template <class T>
double sweep2(int e, bool init, const Grid2 &g, int radius, const Src2 &src, T sSrc,
              const T *slow, T *tt) {
    Sweep2 sw(e);
    const int nx = g.nx, nz = g.nz, ncx = nx - 1, ncz = nz - 1;
    int x0, x1, xd, z0, z1, zd;
    // getLoopLimits 2D, solverUtilities2d.hpp:939-1053
    if (!sw.fx) { x0 = init ? std::max(src.isx, 1) : 1; x1 = nx; xd = 1; }
    else { x0 = init ? std::min(src.isx + 1, nx - 2) : nx - 2; x1 = -1; xd = -1; }
    if (!sw.fz) { z0 = init ? std::max(src.isz, 1) : 1; z1 = nz; zd = 1; }
    else { z0 = init ? std::min(src.isz + 1, nz - 2) : nz - 2; z1 = -1; zd = -1; }
    const T huge = static_cast<T>(kHuge);
    const T xs = static_cast<T>(src.xo), zs = static_cast<T>(src.zo);
    const bool uniform = std::abs(g.dx - g.dz) < std::numeric_limits<T>::epsilon() * 100;
    const T h = static_cast<T>(g.dx);
    // include/private/solver2d.hpp:41-46
    NonUniform2<T> nu{static_cast<T>(g.dx), static_cast<T>(g.dz), static_cast<T>(g.dx / g.dz),
                      static_cast<T>(g.dz / g.dx), static_cast<T>(g.dx / std::hypot(g.dx, g.dz)),
                      static_cast<T>(g.dz / std::hypot(g.dx, g.dz))};
    double diffMax = 0;
    for (int iz = z0; iz != z1; iz += zd) {
        for (int ix = x0; ix != x1; ix += xd) {
            int c0x, c1x, c3x, c0z, c1z, c3z;
            if (!sw.fx) {
                c0x = std::max(0, ix - 1);
                c1x = std::min(ncx - 1, c0x + 1);
                if (ix == 0) c1x = 0;
            } else {
                c0x = ix;
                c1x = std::max(0, c0x - 1);
                if (ix == ncx) { c0x = ix - 1; c1x = ix - 1; }
            }
            c3x = c0x;
            if (!sw.fz) {
                c0z = std::max(0, iz - 1);
                c3z = std::min(ncz - 1, c0z + 1);
                if (iz == 0) c3z = 0;
            } else {
                c0z = iz;
                c3z = std::max(0, c0z - 1);
                if (iz == ncz) { c0z = iz - 1; c3z = iz - 1; }
            }
            c1z = c0z;
            T s0 = slow[static_cast<size_t>(c0z) * ncx + c0x];
            T s1 = slow[static_cast<size_t>(c1z) * ncx + c1x];
            T s3 = slow[static_cast<size_t>(c3z) * ncx + c3x];
            size_t i0 = static_cast<size_t>(iz) * nx + ix;
            int xsft = ix + sw.ixShift, zsft = iz + sw.izShift;
            T t0 = tt[i0];
            T t1 = tt[static_cast<size_t>(iz) * nx + xsft];
            T t2 = tt[static_cast<size_t>(zsft) * nx + xsft];
            T t3 = tt[static_cast<size_t>(zsft) * nx + ix];
            T tUpd = uniform
                ? fd2Uniform<T>(radius, huge, h, sSrc, ix, iz, sw, src, xs, zs, s0, s1, s3, t1, t2, t3)
                : fd2NonUniform<T>(radius, huge, nu, sSrc, ix, iz, sw, src, xs, zs, s0, s1, s3, t1, t2, t3);
            if (tUpd < t0) {
                tt[i0] = tUpd;
                diffMax = std::max(diffMax, static_cast<double>(static_cast<T>(t0 - tUpd)));
            }
        }
    }
    return diffMax;
}

// Solver2D::initializeTravelTimes, src/solver2d.cpp:61-105.
template <class T>
void init2(const Grid2 &g, const Src2 &src, const T *slow, bool initFp64, T *tt) {
    const size_t n = static_cast<size_t>(g.nx) * g.nz;
    std::fill(tt, tt + n, static_cast<T>(kHuge));
    const int ncx = g.nx - 1;
    const T s = slow[static_cast<size_t>(src.isz) * ncx + src.isx];
    for (int k = 0; k < 2; ++k)
        for (int i = 0; i < 2; ++i) {
            int ix = src.isx + i, iz = src.isz + k;
            size_t idx = static_cast<size_t>(iz) * g.nx + ix;
            if (initFp64)
                tt[idx] = static_cast<T>(analyticT2<double>(ix, iz, g.dx, g.dz, src.xo, src.zo,
                                                            static_cast<double>(s)));
            else
                tt[idx] = analyticT2<T>(ix, iz, static_cast<T>(g.dx), static_cast<T>(g.dz),
                                        static_cast<T>(src.xo), static_cast<T>(src.zo), s);
        }
}

template <class T>
int solve2(const Grid2 &g, const Src2 &src, const T *slow, int nSweeps, int radius,
           double tol, int initFp64, int doInitSweeps, T *tt, double *residuals, int *nIter) {
    init2<T>(g, src, slow, initFp64 != 0, tt);
    T sSrc = slow[static_cast<size_t>(src.isz) * (g.nx - 1) + src.isx];
    if (doInitSweeps)
        for (int e = 0; e < 4; ++e) sweep2<T>(e, true, g, radius, src, sSrc, slow, tt);
    // as solve3, with a window of the last 4 refinement sweeps
    int k = 0, quiet = 0;
    bool done = false;
    for (; k < nSweeps && !done; ++k) {
        for (int e = 0; e < 4; ++e) {
            double r = sweep2<T>(e, false, g, radius, src, sSrc, slow, tt);
            if (residuals) residuals[k * 4 + e] = r;
            quiet = r < tol ? quiet + 1 : 0;
            if (quiet >= 4) {
                done = true;
                break;
            }
        }
    }
    if (nIter) *nIter = k;
    return 0;
}

//----------------------------------------------------------------------------//
//                         Level-set tables (Graph3D)                         //
//----------------------------------------------------------------------------//

// Graph3D<E>::initialize, src/graph3d.cpp:120-221: levels are the planes
// jx+jy+jz = const of the sweep-permuted coordinates (permuteGrid,
// solverUtilities3d.hpp:1197-1257); nodes of a level are sorted by natural index;
// indexToLevel is filled by node position (graph3d.cpp:177).
int graph3(int e, int nx, int ny, int nz, int *levelStart, int *nodeToIndex, int *toX,
           int *toY, int *toZ, int *indexToLevel, int *maxLevelSize) {
    if (nx < 3 || ny < 3 || nz < 3) return -1;
    const int nLevels = nx + ny + nz - 2;
    const int fx = e & 1, fy = (e >> 1) & 1, fz = (e >> 2) & 1;
    levelStart[0] = 0;
    int maxSize = 0;
    for (int level = 0; level < nLevels; ++level) {
        int offset = levelStart[level];
        int count = 0;
        int k1 = std::min(std::max(0, level - (nx - 1) - (ny - 1)), nz - 1);
        int k2 = std::min(nz - 1, level);
        for (int iz = k1; iz <= k2; ++iz) {
            int j1 = std::min(std::max(0, level - iz - (nx - 1)), ny - 1);
            int j2 = std::min(ny - 1, level - iz);
            for (int iy = j1; iy <= j2; ++iy) {
                int i1 = std::min(std::max(0, level - iz - iy), nx - 1);
                int i2 = std::min(nx - 1, level - iz - iy);
                for (int ix = i1; ix <= i2; ++ix) {
                    int jx = fx ? nx - 1 - ix : ix;
                    int jy = fy ? ny - 1 - iy : iy;
                    int jz = fz ? nz - 1 - iz : iz;
                    nodeToIndex[offset + count] = jz * nx * ny + jy * nx + jx;
                    indexToLevel[offset + count] = level;
                    ++count;
                }
            }
        }
        maxSize = std::max(maxSize, count);
        levelStart[level + 1] = offset + count;
        std::sort(nodeToIndex + offset, nodeToIndex + offset + count);
        for (int i = 0; i < count; ++i) {
            int idx = nodeToIndex[offset + i];
            int iz = idx / (nx * ny);
            int iy = (idx - iz * nx * ny) / nx;
            toX[offset + i] = idx - iz * nx * ny - iy * nx;
            toY[offset + i] = iy;
            toZ[offset + i] = iz;
        }
    }
    *maxLevelSize = maxSize;
    return nLevels;
}

//----------------------------------------------------------------------------//
//                            Analytic solutions                              //
//----------------------------------------------------------------------------//

// LinearGradient3D / LinearGradient2D, src/analytic/linearGradient3d.cpp:12-116 and
// linearGradient2d.cpp:12-124 (z-gradient only); Homogeneous when vTop == vBottom.
void linearGradient3(int nx, int ny, int nz, double dx, double dy, double dz, double xs,
                     double ys, double zs, double vTop, double vBottom, double *tt) {
    const double gz = (vBottom - vTop) / ((nz - 1) * dz);
    const double absG2 = gz * gz;
    const double absG = std::sqrt(absG2);
    const double v0 = vTop + gz * zs;
    const double s0 = 1 / v0;
    for (int iz = 0; iz < nz; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix) {
                size_t idx = static_cast<size_t>(iz) * nx * ny + static_cast<size_t>(iy) * nx + ix;
                if (std::abs(vTop - vBottom) > 1.e-14) {
                    double ddx = ix * dx - xs, ddy = iy * dy - ys, ddz = iz * dz - zs;
                    double dist2 = ddx * ddx + ddy * ddy + ddz * ddz;
                    double vel = v0 + 0 * ddx + 0 * ddy + gz * ddz;
                    double arg = 1 + (s0 * absG2 * dist2) / (2 * vel);
                    tt[idx] = std::acosh(arg) / absG;
                } else {
                    double ddx = xs - ix * dx, ddy = ys - iy * dy, ddz = zs - iz * dz;
                    tt[idx] = std::sqrt(ddx * ddx + ddy * ddy + ddz * ddz) * s0;
                }
            }
}

void linearGradient2(int nx, int nz, double dx, double dz, double xs, double zs, double vTop,
                     double vBottom, double *tt) {
    const double gz = (vBottom - vTop) / ((nz - 1) * dz);
    const double absG2 = gz * gz;
    const double absG = std::sqrt(absG2);
    const double v0 = vTop + gz * zs;
    const double s0 = 1 / v0;
    for (int iz = 0; iz < nz; ++iz)
        for (int ix = 0; ix < nx; ++ix) {
            size_t idx = static_cast<size_t>(iz) * nx + ix;
            if (std::abs(vTop - vBottom) > 1.e-14) {
                double ddx = ix * dx - xs, ddz = iz * dz - zs;
                double dist2 = ddx * ddx + ddz * ddz;
                double vel = v0 + 0 * ddx + gz * ddz;
                double arg = 1 + (s0 * absG2 * dist2) / (2 * vel);
                tt[idx] = std::acosh(arg) / absG;
            } else {
                double ddx = xs - ix * dx, ddz = zs - iz * dz;
                tt[idx] = std::hypot(ddx, ddz) * s0;
            }
        }
}

// Model3D::setNodalVelocities -> interpolate3d, src/model3d.cpp:46-151 (natural and
// XYZ orderings): cell slowness = 8/(sum of the 8 corner velocities), summed in
// pairs in the reference's order.
template <class T>
void nodalToCell3(int nx, int ny, int nz, const T *v, int ordering, T *slow) {
    const size_t ncx = nx - 1, ncy = ny - 1, ncz = nz - 1;
    const T eight = 8;
    for (size_t iz = 0; iz < ncz; ++iz)
        for (size_t iy = 0; iy < ncy; ++iy)
            for (size_t ix = 0; ix < ncx; ++ix) {
                size_t dst = iz * ncx * ncy + iy * ncx + ix;
                size_t i1, i2, i3, i4, i5, i6, i7, i8;
                if (ordering == 0) {
                    i1 = iz * (ncx + 1) * (ncy + 1) + iy * (ncx + 1) + ix;
                    i2 = i1 + 1; i3 = i1 + (ncx + 1); i4 = i3 + 1;
                    i5 = i1 + (ncx + 1) * (ncy + 1); i6 = i2 + (ncx + 1) * (ncy + 1);
                    i7 = i3 + (ncx + 1) * (ncy + 1); i8 = i4 + (ncx + 1) * (ncy + 1);
                } else {
                    i1 = ix * (ncz + 1) * (ncy + 1) + iy * (ncz + 1) + iz;
                    i2 = i1 + 1; i3 = i1 + (ncz + 1); i4 = i3 + 1;
                    i5 = i1 + (ncz + 1) * (ncy + 1); i6 = i2 + (ncz + 1) * (ncy + 1);
                    i7 = i3 + (ncz + 1) * (ncy + 1); i8 = i4 + (ncz + 1) * (ncy + 1);
                }
                T sum1 = v[i1] + v[i2], sum2 = v[i3] + v[i4];
                T sum3 = v[i5] + v[i6], sum4 = v[i7] + v[i8];
                slow[dst] = eight / (sum1 + sum2 + sum3 + sum4);
            }
}

// Model2D::setNodalVelocities -> interpolate2d, src/model2d.cpp:46-125.
template <class T>
void nodalToCell2(int nx, int nz, const T *v, int ordering, T *slow) {
    const size_t ncx = nx - 1, ncz = nz - 1;
    const T four = 4;
    for (size_t iz = 0; iz < ncz; ++iz)
        for (size_t ix = 0; ix < ncx; ++ix) {
            size_t dst = iz * ncx + ix;
            size_t i1, i2, i3, i4;
            if (ordering == 0) {
                i1 = iz * (ncx + 1) + ix; i2 = i1 + 1; i3 = i1 + (ncx + 1); i4 = i3 + 1;
            } else {
                i1 = ix * (ncz + 1) + iz; i2 = i1 + 1; i3 = i1 + (ncz + 1); i4 = i3 + 1;
            }
            T sum1 = v[i1] + v[i2], sum2 = v[i3] + v[i4];
            slow[dst] = four / (sum1 + sum2);
        }
}

}  // namespace

//----------------------------------------------------------------------------//
//                                 C entry points                             //
//----------------------------------------------------------------------------//
//----------------------------------------------------------------------------//
//                 Products of a solved field: gradient, stations             //
//----------------------------------------------------------------------------//

// Travel-time gradient of a solved field, the reference's 2D finiteDifference with
// central differences (src/gradient.hpp:20-289): interior nodes (u[i+1] - u[i-1]) / 2h,
// the first and last node of an axis the second-order one-sided differences
// (-3 u0 + 4 u1 - u2) / 2h and (u[n-3] - 4 u[n-2] + 3 u[n-1]) / 2h, and -- when the
// source is off the cell corner by more than 1e-7 m -- the analytic constant-slowness
// gradient at the corners of the source cell.  The 3D form applies the same rule per
// axis and at the 8 corners.  Output interleaved per node: (d/dx, d/dz) or (d/dx, d/dy, d/dz).
template <class T>
T axisDerivative(const T *t, size_t i, size_t stride, int k, int n, T twodi) {
    if (k == 0) return (-3 * t[i] + 4 * t[i + stride] - t[i + 2 * stride]) * twodi;
    if (k == n - 1) return (t[i - 2 * stride] - 4 * t[i - stride] + 3 * t[i]) * twodi;
    return (t[i + stride] - t[i - stride]) * twodi;
}

template <class T>
void gradient3(const Grid3 &g, const Src3 &src, T slow0, const T *t, T *grad) {
    const T twodxi = static_cast<T>(1. / (2. * g.dx));
    const T twodyi = static_cast<T>(1. / (2. * g.dy));
    const T twodzi = static_cast<T>(1. / (2. * g.dz));
    const size_t sx = 1, sy = g.nx, sz = static_cast<size_t>(g.nx) * g.ny;
    for (int iz = 0; iz < g.nz; ++iz)
        for (int iy = 0; iy < g.ny; ++iy)
            for (int ix = 0; ix < g.nx; ++ix) {
                const size_t i = iz * sz + iy * sy + ix;
                grad[3 * i] = axisDerivative(t, i, sx, ix, g.nx, twodxi);
                grad[3 * i + 1] = axisDerivative(t, i, sy, iy, g.ny, twodyi);
                grad[3 * i + 2] = axisDerivative(t, i, sz, iz, g.nz, twodzi);
            }
    constexpr double tol = 1.e-7;
    const double d0[3] = {src.isx * g.dx - src.xo, src.isy * g.dy - src.yo, src.isz * g.dz - src.zo};
    const double d1[3] = {(src.isx + 1) * g.dx - src.xo, (src.isy + 1) * g.dy - src.yo, (src.isz + 1) * g.dz - src.zo};
    const bool doAxis[3] = {std::abs(d0[0]) > tol, std::abs(d0[1]) > tol, std::abs(d0[2]) > tol};
    if (!(doAxis[0] || doAxis[1] || doAxis[2])) return;
    for (int k = 0; k < 2; ++k)
        for (int j = 0; j < 2; ++j)
            for (int i = 0; i < 2; ++i) {
                const double a = i ? d1[0] : d0[0], b = j ? d1[1] : d0[1], c = k ? d1[2] : d0[2];
                const double r = std::sqrt(a * a + b * b + c * c);
                const size_t n = (src.isz + k) * sz + (src.isy + j) * sy + (src.isx + i);
                if (doAxis[0]) grad[3 * n] = static_cast<T>((a / r) * slow0);
                if (doAxis[1]) grad[3 * n + 1] = static_cast<T>((b / r) * slow0);
                if (doAxis[2]) grad[3 * n + 2] = static_cast<T>((c / r) * slow0);
            }
}

template <class T>
void gradient2(const Grid2 &g, const Src2 &src, T slow0, const T *t, T *grad) {
    const T twodxi = static_cast<T>(1. / (2. * g.dx));
    const T twodzi = static_cast<T>(1. / (2. * g.dz));
    for (int iz = 0; iz < g.nz; ++iz)
        for (int ix = 0; ix < g.nx; ++ix) {
            const size_t i = static_cast<size_t>(iz) * g.nx + ix;
            grad[2 * i] = axisDerivative(t, i, 1, ix, g.nx, twodxi);
            grad[2 * i + 1] = axisDerivative(t, i, g.nx, iz, g.nz, twodzi);
        }
    constexpr double tol = 1.e-7;
    const double dx0 = src.isx * g.dx - src.xo, dx1 = (src.isx + 1) * g.dx - src.xo;
    const double dz0 = src.isz * g.dz - src.zo, dz1 = (src.isz + 1) * g.dz - src.zo;
    const bool doX = std::abs(dx0) > tol, doZ = std::abs(dz0) > tol;
    if (!(doX || doZ)) return;
    for (int k = 0; k < 2; ++k)
        for (int i = 0; i < 2; ++i) {
            const double a = i ? dx1 : dx0, c = k ? dz1 : dz0;
            const double r = std::sqrt(a * a + c * c);
            const size_t n = static_cast<size_t>(src.isz + k) * g.nx + (src.isx + i);
            if (doX) grad[2 * n] = static_cast<T>((a / r) * slow0);
            if (doZ) grad[2 * n + 1] = static_cast<T>((c / r) * slow0);
        }
}

// Travel times at stations (Solver2D::interpolateTravelTimes, src/solver2d.cpp:106-167,
// with bilinear() of src/ray/bilinear.hpp): a station in the source cell gets the
// straight-ray time |x - x_s| * s_src; any other station the bilinear (2D) / trilinear
// (3D, x then y then z) interpolation of the 4 / 8 corner times of its cell, in double.
// Stations are located as sources are: offset = x - x0, cell = min(nCell - 1, offset / d).
template <class T>
double station3(const Grid3 &g, const Src3 &src, double sSrc, const T *t, int cx, int cy, int cz, double xi,
                double yi, double zi) {
    if (cx == src.isx && cy == src.isy && cz == src.isz) {
        const double a = xi - src.xo, b = yi - src.yo, c = zi - src.zo;
        return std::sqrt(a * a + b * b + c * c) * sSrc;
    }
    const size_t sy = g.nx, sz = static_cast<size_t>(g.nx) * g.ny;
    const size_t i0 = cz * sz + cy * sy + cx;
    auto f = [&](int i, int j, int k) { return static_cast<double>(t[i0 + k * sz + j * sy + i]); };
    const double dxi = 1. / g.dx, dyi = 1. / g.dy, dzi = 1. / g.dz;
    const double x1 = cx * g.dx, x2 = (cx + 1) * g.dx, y1 = cy * g.dy, y2 = (cy + 1) * g.dy;
    const double z1 = cz * g.dz, z2 = (cz + 1) * g.dz;
    const double x2mx = x2 - xi, xmx1 = xi - x1;
    const double f11 = dxi * (x2mx * f(0, 0, 0) + xmx1 * f(1, 0, 0));
    const double f21 = dxi * (x2mx * f(0, 1, 0) + xmx1 * f(1, 1, 0));
    const double f12 = dxi * (x2mx * f(0, 0, 1) + xmx1 * f(1, 0, 1));
    const double f22 = dxi * (x2mx * f(0, 1, 1) + xmx1 * f(1, 1, 1));
    const double y2my = y2 - yi, ymy1 = yi - y1;
    const double fz1 = dyi * (y2my * f11 + ymy1 * f21);
    const double fz2 = dyi * (y2my * f12 + ymy1 * f22);
    return dzi * ((z2 - zi) * fz1 + (zi - z1) * fz2);
}

template <class T>
double station2(const Grid2 &g, const Src2 &src, double sSrc, const T *t, int cx, int cz, double xi, double zi) {
    if (cx == src.isx && cz == src.isz) return eikxHypot(xi - src.xo, zi - src.zo) * sSrc;
    const size_t i00 = static_cast<size_t>(cz) * g.nx + cx;
    const double f00 = t[i00], f10 = t[i00 + 1], f01 = t[i00 + g.nx], f11 = t[i00 + g.nx + 1];
    const double dxi = 1. / g.dx, dzi = 1. / g.dz;
    const double x1 = cx * g.dx, x2 = (cx + 1) * g.dx, z1 = cz * g.dz, z2 = (cz + 1) * g.dz;
    const double x2mx = x2 - xi, xmx1 = xi - x1;
    const double fxz1 = dxi * (x2mx * f00 + xmx1 * f10);
    const double fxz2 = dxi * (x2mx * f01 + xmx1 * f11);
    return dzi * ((z2 - zi) * fxz1 + (zi - z1) * fxz2);
}

//----------------------------------------------------------------------------//
//                       2D gradient ray tracer                               //
//----------------------------------------------------------------------------//

// Ray::GradientTracer2D::trace (src/ray/gradientTracer2d.cpp:339-600) for one station:
// march from the station down the travel-time gradient (bilinear, src/ray/bilinear.hpp)
// with the radius-scaled step lengths of GradientTracerOptions
// (src/ray/gradientTracerOptions.cpp), until the ray ends within one cell of the source
// cell; then turn the march around and heal it into segments that end on cell walls
// (intersect, gradientTracer2d.cpp:137-196).  Positions are offsets from the origin;
// segments are written in absolute coordinates as (x0, z0, x1, z1, slowness, cell), cell
// -1 where the reference leaves it unset.  Returns the number of segments, -1 when the
// march did not reach the source within maxSteps, -2 when the path needs more than
// `capacity` segments, -3 when the march left the grid (the reference reads outside its
// arrays there).  Gradient nodes past the end of the array read as 0: they are used only
// with weight 0.  hypot is eikxHypot, as on the GPU (the reference uses std::hypot).
template <class T>
int traceRay2(int nx, int nz, double dx, double dz, double x0, double z0, const T *grad, const double *slow,
              int isx, int isz, double xs, double zs, double xr, double zr, int nRsf, const int *rsfRadius,
              const double *rsfScale, int maxSteps, double *pos, int capacity, double *seg) {
    const int ncx = nx - 1, ncz = nz - 1;
    auto slowAt = [&](int cx, int cz) {
        cx = clampi(cx, 0, ncx - 1);
        cz = clampi(cz, 0, ncz - 1);
        return slow[static_cast<size_t>(cz) * ncx + cx];
    };
    const double dxi = 1. / dx, dzi = 1. / dz;
    const double hmin = std::min(dx, dz);
    const int scx = std::min(nx - 2, static_cast<int>(xr / dx)), scz = std::min(nz - 2, static_cast<int>(zr / dz));
    const double sourceSlowness = slowAt(isx, isz), stationSlowness = slowAt(scx, scz);
    int nSeg = 0;
    auto put = [&](double ax, double az, double bx, double bz, double s, int cell) {
        if (nSeg >= capacity) return false;
        double *o = seg + 6 * static_cast<size_t>(nSeg++);
        o[0] = ax; o[1] = az; o[2] = bx; o[3] = bz; o[4] = s; o[5] = cell;
        return true;
    };
    if (scz * ncx + scx == isz * ncx + isx) {
        return put(x0 + xs, z0 + zs, x0 + xr, z0 + zr, stationSlowness, scz * ncx + scx) ? 1 : -2;
    }
    const long long nGrad = 2LL * nx * nz;
    auto g = [&](long long i) { return i >= 0 && i < nGrad ? static_cast<double>(grad[i]) : 0.0; };
    auto bilinear = [&](double x, double z, double x1, double x2, double z1, double z2, double f00, double f01,
                        double f10, double f11) {
        const double x2mx = x2 - x, xmx1 = x - x1;
        const double fxz1 = dxi * (x2mx * f00 + xmx1 * f10);
        const double fxz2 = dxi * (x2mx * f01 + xmx1 * f11);
        const double z2mz = z2 - z, zmz1 = z - z1;
        return dzi * (z2mz * fxz1 + zmz1 * fxz2);
    };
    double xs0 = xr, zs0 = zr;
    int cx0 = -1, cz0 = -1;
    double gx000 = 1.e10, gz000 = 1.e10, gx100 = 1.e10, gz100 = 1.e10;
    double gx010 = 1.e10, gz010 = 1.e10, gx110 = 1.e10, gz110 = 1.e10;
    double stepLength0 = rsfScale[nRsf - 1] * hmin;
    int m = 0;   // march points p_0 .. p_m
    pos[0] = xr; pos[1] = zr;
    bool converged = false;
    for (int step = 0; step < maxSteps; ++step) {
        const int cxs = static_cast<int>(xs0 / dx), czs = static_cast<int>(zs0 / dz);
        if (cxs < 0 || cxs > nx - 1 || czs < 0 || czs > nz - 1) return -3;
        double stepLength = stepLength0;
        double gx00 = gx000, gz00 = gz000, gx10 = gx100, gz10 = gz100;
        double gx01 = gx010, gz01 = gz010, gx11 = gx110, gz11 = gz110;
        if (cxs != cx0 || czs != cz0) {
            const int dist = std::min(std::abs(isx - cxs), std::abs(isz - czs));
            stepLength = rsfScale[nRsf - 1] * hmin;
            for (int k = 0; k < nRsf; ++k)
                if (rsfRadius[k] >= dist) {
                    stepLength = rsfScale[k] * hmin;
                    break;
                }
            const long long i00 = 2LL * (static_cast<long long>(czs) * nx + cxs);
            const long long i10 = 2LL * (static_cast<long long>(czs) * nx + cxs + 1);
            const long long i11 = 2LL * (static_cast<long long>(czs + 1) * nx + cxs + 1);
            const long long i01 = 2LL * (static_cast<long long>(czs + 1) * nx + cxs);
            gx00 = g(i00); gz00 = g(i00 + 1);
            gx10 = g(i10); gz10 = g(i10 + 1);
            gx01 = g(i01); gz01 = g(i01 + 1);
            gx11 = g(i11); gz11 = g(i11 + 1);
        }
        const double gx = bilinear(xs0, zs0, cxs * dx, (cxs + 1) * dx, czs * dz, (czs + 1) * dz, gx00, gx01, gx10, gx11);
        const double gz = bilinear(xs0, zs0, cxs * dx, (cxs + 1) * dx, czs * dz, (czs + 1) * dz, gz00, gz01, gz10, gz11);
        const double gNorm = eikxHypot(gx, gz);
        const double gStep = stepLength / gNorm;
        const double xe = xs0 - gx * gStep, ze = zs0 - gz * gStep;
        ++m;
        pos[2 * m] = xe; pos[2 * m + 1] = ze;
        const int cxe = static_cast<int>(xe / dx), cze = static_cast<int>(ze / dz);
        if (std::abs(cxe - isx) < 2 && std::abs(cze - isz) < 2) {
            converged = true;
            break;
        }
        stepLength0 = stepLength;
        xs0 = xe; zs0 = ze;
        cx0 = cxs; cz0 = czs;
        gx000 = gx00; gz000 = gz00; gx100 = gx10; gz100 = gz10;
        gx010 = gx01; gz010 = gz01; gx110 = gx11; gz110 = gz11;
    }
    if (!converged) return -1;
    // reversed march: R_0 = source -> p_m, R_j = p_{m-j+1} -> p_{m-j} (j = 1..m)
    auto cellOf = [&](int k, int &cx, int &cz) {
        cx = static_cast<int>(pos[2 * k] / dx);
        cz = static_cast<int>(pos[2 * k + 1] / dz);
    };
    double xa = xs, za = zs;
    for (int j = 0; j <= m; ++j) {
        if (j == m) {
            if (!put(x0 + xa, z0 + za, x0 + xr, z0 + zr, stationSlowness, -1)) return -2;
            break;
        }
        int c0x, c0z, c1x, c1z;
        double ax, az, bx, bz;
        if (j == 0) {
            c0x = isx; c0z = isz;
            cellOf(m, c1x, c1z);
            ax = xs; az = zs; bx = pos[2 * m]; bz = pos[2 * m + 1];
        } else {
            cellOf(m - j + 1, c0x, c0z);
            cellOf(m - j, c1x, c1z);
            ax = pos[2 * (m - j + 1)]; az = pos[2 * (m - j + 1) + 1];
            bx = pos[2 * (m - j)]; bz = pos[2 * (m - j) + 1];
        }
        if (c0x != c1x || c0z != c1z) {
            double gx = bx - ax, gz = bz - az;
            const double gnorm = eikxHypot(gx, gz);
            gx = gx / gnorm;
            gz = gz / gnorm;
            // intersect: where the line from (xa, za) along (gx, gz) leaves cell (c0x, c0z)
            double ti = 1.e10, tj = 1.e10;
            const double wx0 = c0x * dx, wx1 = (c0x + 1) * dx, wz0 = c0z * dz, wz1 = (c0z + 1) * dz;
            if (gx > 0) ti = (wx1 - xa) / gx;
            else if (gx < 0) ti = (wx0 - xa) / gx;
            if (gz > 0) tj = (wz1 - za) / gz;
            else if (gz < 0) tj = (wz0 - za) / gz;
            const double fxi = xa + gx * ti, fzi = za + gz * ti;
            const double fxj = xa + gx * tj, fzj = za + gz * tj;
            const double li = (fxi - xa) * (fxi - xa) + (fzi - za) * (fzi - za);
            const double lj = (fxj - xa) * (fxj - xa) + (fzj - za) * (fzj - za);
            const double xb = li < lj ? fxi : fxj, zb = li < lj ? fzi : fzj;
            const double s = j == 0 ? sourceSlowness : slowAt(c0x, c0z);
            if (!put(x0 + xa, z0 + za, x0 + xb, z0 + zb, s, -1)) return -2;
            xa = xb;
            za = zb;
        }
    }
    return nSeg;
}

extern "C" {

int oracle_solve3d_f64(int nx, int ny, int nz, double dx, double dy, double dz, int isx,
                       int isy, int isz, double xo, double yo, double zo, const double *slow,
                       int nSweeps, int radius, double tol, int initFp64, int doInitSweeps,
                       double *tt, double *residuals, int *nIter) {
    Grid3 g{nx, ny, nz, dx, dy, dz};
    Src3 s{isx, isy, isz, xo, yo, zo};
    return solve3<double>(g, s, slow, nSweeps, radius, tol, initFp64, doInitSweeps, tt, residuals, nIter);
}

int oracle_solve3d_f32(int nx, int ny, int nz, double dx, double dy, double dz, int isx,
                       int isy, int isz, double xo, double yo, double zo, const float *slow,
                       int nSweeps, int radius, double tol, int initFp64, int doInitSweeps,
                       float *tt, double *residuals, int *nIter) {
    Grid3 g{nx, ny, nz, dx, dy, dz};
    Src3 s{isx, isy, isz, xo, yo, zo};
    return solve3<float>(g, s, slow, nSweeps, radius, tol, initFp64, doInitSweeps, tt, residuals, nIter);
}

int oracle_advance3d_f32(int nx, int ny, int nz, double dx, double dy, double dz, int isx, int isy, int isz,
                        double xo, double yo, double zo, const float *slow, int nSweeps, int radius, double tol,
                        int initFp64, float *tt, int *pos, int *quiet, int maxSweeps) {
    Grid3 g{nx, ny, nz, dx, dy, dz};
    Src3 s{isx, isy, isz, xo, yo, zo};
    return advance3<float>(g, s, slow, nSweeps, radius, tol, initFp64, tt, pos, quiet, maxSweeps);
}

// One sweep (e = 0..7) on an existing field; returns the largest decrease.
double oracle_sweep3d_f32(int e, int init, int nx, int ny, int nz, double dx, double dy,
                          double dz, int isx, int isy, int isz, double xo, double yo, double zo,
                          int radius, const float *slow, float *tt) {
    Grid3 g{nx, ny, nz, dx, dy, dz};
    Src3 s{isx, isy, isz, xo, yo, zo};
    float sSrc = slow[static_cast<size_t>(isz) * (nx - 1) * (ny - 1) + static_cast<size_t>(isy) * (nx - 1) + isx];
    return sweep3<float>(e, init != 0, g, radius, s, sSrc, slow, tt);
}

double oracle_sweep3d_f64(int e, int init, int nx, int ny, int nz, double dx, double dy,
                          double dz, int isx, int isy, int isz, double xo, double yo, double zo,
                          int radius, const double *slow, double *tt) {
    Grid3 g{nx, ny, nz, dx, dy, dz};
    Src3 s{isx, isy, isz, xo, yo, zo};
    double sSrc = slow[static_cast<size_t>(isz) * (nx - 1) * (ny - 1) + static_cast<size_t>(isy) * (nx - 1) + isx];
    return sweep3<double>(e, init != 0, g, radius, s, sSrc, slow, tt);
}

int oracle_solve2d_f64(int nx, int nz, double dx, double dz, int isx, int isz, double xo,
                       double zo, const double *slow, int nSweeps, int radius, double tol,
                       int initFp64, int doInitSweeps, double *tt, double *residuals, int *nIter) {
    Grid2 g{nx, nz, dx, dz};
    Src2 s{isx, isz, xo, zo};
    return solve2<double>(g, s, slow, nSweeps, radius, tol, initFp64, doInitSweeps, tt, residuals, nIter);
}

int oracle_solve2d_f32(int nx, int nz, double dx, double dz, int isx, int isz, double xo,
                       double zo, const float *slow, int nSweeps, int radius, double tol,
                       int initFp64, int doInitSweeps, float *tt, double *residuals, int *nIter) {
    Grid2 g{nx, nz, dx, dz};
    Src2 s{isx, isz, xo, zo};
    return solve2<float>(g, s, slow, nSweeps, radius, tol, initFp64, doInitSweeps, tt, residuals, nIter);
}

int oracle_graph3d(int e, int nx, int ny, int nz, int *levelStart, int *nodeToIndex, int *toX,
                   int *toY, int *toZ, int *indexToLevel, int *maxLevelSize) {
    return graph3(e, nx, ny, nz, levelStart, nodeToIndex, toX, toY, toZ, indexToLevel, maxLevelSize);
}

void oracle_linear_gradient3d(int nx, int ny, int nz, double dx, double dy, double dz,
                              double xs, double ys, double zs, double vTop, double vBottom,
                              double *tt) {
    linearGradient3(nx, ny, nz, dx, dy, dz, xs, ys, zs, vTop, vBottom, tt);
}

void oracle_linear_gradient2d(int nx, int nz, double dx, double dz, double xs, double zs,
                              double vTop, double vBottom, double *tt) {
    linearGradient2(nx, nz, dx, dz, xs, zs, vTop, vBottom, tt);
}

void oracle_nodal_to_cell3d_f64(int nx, int ny, int nz, const double *v, int ordering, double *s) {
    nodalToCell3<double>(nx, ny, nz, v, ordering, s);
}
void oracle_nodal_to_cell3d_f32(int nx, int ny, int nz, const float *v, int ordering, float *s) {
    nodalToCell3<float>(nx, ny, nz, v, ordering, s);
}
void oracle_nodal_to_cell2d_f64(int nx, int nz, const double *v, int ordering, double *s) {
    nodalToCell2<double>(nx, nz, v, ordering, s);
}

double oracle_hypot(double a, double b) { return eikxHypot(a, b); }
void oracle_set_near_fp64(int on) { gNearFp64 = on; }

// Rays from n stations (absolute x, z) to a source (absolute x, z) through a gradient
// field (nz x nx x 2, natural); segments [station][capacity][6]; counts[station].
int oracle_trace_rays2d(int precision, int nx, int nz, double dx, double dz, double x0, double z0, const void *grad,
                        const double *slow, double sx, double sz, int n, const double *stations, int nRsf,
                        const int *rsfRadius, const double *rsfScale, int maxSteps, int capacity, double *segments,
                        int *counts) {
    const double xs = sx - x0, zs = sz - z0;
    const int isx = std::min(nx - 2, static_cast<int>(xs / dx)), isz = std::min(nz - 2, static_cast<int>(zs / dz));
    std::vector<double> pos(2 * static_cast<size_t>(maxSteps + 2));
    for (int i = 0; i < n; ++i) {
        const double xr = stations[2 * i] - x0, zr = stations[2 * i + 1] - z0;
        double *seg = segments + static_cast<size_t>(i) * capacity * 6;
        counts[i] = precision == 0
            ? traceRay2<float>(nx, nz, dx, dz, x0, z0, static_cast<const float *>(grad), slow, isx, isz, xs, zs, xr, zr,
                               nRsf, rsfRadius, rsfScale, maxSteps, pos.data(), capacity, seg)
            : traceRay2<double>(nx, nz, dx, dz, x0, z0, static_cast<const double *>(grad), slow, isx, isz, xs, zs, xr,
                                zr, nRsf, rsfRadius, rsfScale, maxSteps, pos.data(), capacity, seg);
    }
    return 0;
}

// 0: the 2D analytic times use std::hypot (as the reference); 1: eikxHypot (as the GPU).
void oracle_set_hypot_mode(int mode) { gHypotMode = mode; }


int oracle_gradient3d_f32(int nx, int ny, int nz, double dx, double dy, double dz, int isx, int isy, int isz,
                          double xo, double yo, double zo, float slow0, const float *tt, float *grad) {
    gradient3<float>(Grid3{nx, ny, nz, dx, dy, dz}, Src3{isx, isy, isz, xo, yo, zo}, slow0, tt, grad);
    return 0;
}
int oracle_gradient3d_f64(int nx, int ny, int nz, double dx, double dy, double dz, int isx, int isy, int isz,
                          double xo, double yo, double zo, double slow0, const double *tt, double *grad) {
    gradient3<double>(Grid3{nx, ny, nz, dx, dy, dz}, Src3{isx, isy, isz, xo, yo, zo}, slow0, tt, grad);
    return 0;
}
int oracle_gradient2d_f32(int nx, int nz, double dx, double dz, int isx, int isz, double xo, double zo, float slow0,
                          const float *tt, float *grad) {
    gradient2<float>(Grid2{nx, nz, dx, dz}, Src2{isx, isz, xo, zo}, slow0, tt, grad);
    return 0;
}
int oracle_gradient2d_f64(int nx, int nz, double dx, double dz, int isx, int isz, double xo, double zo, double slow0,
                          const double *tt, double *grad) {
    gradient2<double>(Grid2{nx, nz, dx, dz}, Src2{isx, isz, xo, zo}, slow0, tt, grad);
    return 0;
}
// Station times; stations given as (cell x, cell y, cell z) and offsets from the origin.
int oracle_stations3d(int precision, int nx, int ny, int nz, double dx, double dy, double dz, int isx, int isy, int isz,
                      double xo, double yo, double zo, double sSrc, const void *tt, int n, const int *cells,
                      const double *offs, double *out) {
    Grid3 g{nx, ny, nz, dx, dy, dz};
    Src3 s{isx, isy, isz, xo, yo, zo};
    for (int i = 0; i < n; ++i)
        out[i] = precision == 0
            ? station3<float>(g, s, sSrc, static_cast<const float *>(tt), cells[3 * i], cells[3 * i + 1],
                              cells[3 * i + 2], offs[3 * i], offs[3 * i + 1], offs[3 * i + 2])
            : station3<double>(g, s, sSrc, static_cast<const double *>(tt), cells[3 * i], cells[3 * i + 1],
                               cells[3 * i + 2], offs[3 * i], offs[3 * i + 1], offs[3 * i + 2]);
    return 0;
}
int oracle_stations2d(int precision, int nx, int nz, double dx, double dz, int isx, int isz, double xo, double zo,
                      double sSrc, const void *tt, int n, const int *cells, const double *offs, double *out) {
    Grid2 g{nx, nz, dx, dz};
    Src2 s{isx, isz, xo, zo};
    for (int i = 0; i < n; ++i)
        out[i] = precision == 0
            ? station2<float>(g, s, sSrc, static_cast<const float *>(tt), cells[2 * i], cells[2 * i + 1],
                              offs[2 * i], offs[2 * i + 1])
            : station2<double>(g, s, sSrc, static_cast<const double *>(tt), cells[2 * i], cells[2 * i + 1],
                               offs[2 * i], offs[2 * i + 1]);
    return 0;
}
}  // extern "C"
