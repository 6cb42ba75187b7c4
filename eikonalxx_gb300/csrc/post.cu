// Products of a solved travel-time field, computed where the field lives (HBM):
//   * the travel-time gradient -- the reference's central-difference finiteDifference
//     (src/gradient.hpp:20-289): (u[i+1] - u[i-1]) / 2h inside, the second-order
//     one-sided differences (-3 u0 + 4 u1 - u2) / 2h and (u[n-3] - 4 u[n-2] + 3 u[n-1]) / 2h
//     on the first and last node of an axis, and the analytic constant-slowness gradient
//     at the corners of the source cell; in 3D the same rule per axis and at 8 corners;
//   * travel times at stations (Solver2D::interpolateTravelTimes, src/solver2d.cpp:106-167,
//     bilinear() of src/ray/bilinear.hpp): the straight-ray time in the source cell,
//     bilinear (2D) or trilinear (3D; x, then y, then z) interpolation elsewhere, in FP64.
// The gradient is one HBM-bound pass (read the field, write 2 or 3 values per node).
#include "sweep.h"

namespace eikx {


// ---------------------------------------------------------------------------------------
// Self-test of the Cartesian operator's shortcuts (eikx_selftest_operator3d): on stencils
// built to sit at the edges of the shortcuts -- node times within a few units in the last
// place of the operator's own value, neighbour differences at the 2D windows' limits
// |t_a - t_b| = hs, homogeneous slowness, unreached (huge) neighbours -- min(t0, bounded)
// must equal min(t0, fd3UniformFar) bit for bit.
__device__ __forceinline__ unsigned long long splitmix(unsigned long long &x) {
    unsigned long long z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double uni(unsigned long long &x) {
    return static_cast<double>(splitmix(x) >> 11) * (1.0 / 9007199254740992.0);
}
template <class T> __device__ __forceinline__ T ulpStep(T v, int k) {
    T r = v;
    const T dir = k > 0 ? static_cast<T>(1.e30) : static_cast<T>(-1.e30);
    for (int i = 0; i < (k > 0 ? k : -k); ++i) r = nextafter(r, dir);
    return r;
}
template <class T> __device__ __forceinline__ bool sameBits(T a, T b) {
    if constexpr (sizeof(T) == 4) return __float_as_uint(a) == __float_as_uint(b);
    else return __double_as_longlong(a) == __double_as_longlong(b);
}

template <class T>
__global__ void operatorSelftestKernel(long long n, unsigned long long seed, unsigned long long *counts) {
    unsigned long long local[4] = {0, 0, 0, 0};   // evaluated, mismatches, shortcut exits, t0 = operator
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        unsigned long long x = seed ^ (static_cast<unsigned long long>(i) * 0xD1B54A32D192ED03ull);
        const double hs[4] = {10.0, 25.0, 50.0, 100.0};
        const T h = static_cast<T>(hs[splitmix(x) & 3]);
        Stencil3<T> st;
        T *s = &st.s0;
        const bool homogeneous = (splitmix(x) & 3) == 0;
        const double v0 = 1500.0 + 6500.0 * uni(x);
        for (int k = 0; k < 7; ++k) s[k] = static_cast<T>(1.0 / (homogeneous ? v0 : 1500.0 + 6500.0 * uni(x)));
        const double base = (splitmix(x) & 7) == 0 ? 1e-3 * uni(x) : 40.0 * uni(x);
        const double hsMin = static_cast<double>(h) / 8000.0, hsMax = static_cast<double>(h) / 1500.0;
        T *t = &st.t1;
        for (int k = 0; k < 7; ++k) {
            const unsigned r = static_cast<unsigned>(splitmix(x) & 15);
            double off;
            if (r < 4) off = (uni(x) * 3.0 - 1.0) * hsMax;                            // anywhere near
            else if (r < 8) off = (r & 1 ? 1.0 : -1.0) * static_cast<double>(h) * s[k]; // at a window's edge
            else if (r < 10) off = static_cast<double>(h) * s[0] * (r & 1 ? 1.4142135623730951 : 1.7320508075688772);
            else if (r < 11) off = 0.0;
            else off = (uni(x) * 2.0 - 0.5) * hsMin;
            t[k] = static_cast<T>(base + off > 0 ? base + off : 0.0);
            if ((splitmix(x) & 31) == 0) t[k] = static_cast<T>(1.e10);               // unreached
            if (splitmix(x) & 1) t[k] = ulpStep(t[k], static_cast<int>(splitmix(x) % 5) - 2);
        }
        const T r = fd3UniformFar<T>(h, st);
        T t0;
        const unsigned mode = static_cast<unsigned>(splitmix(x) % 6);
        if (mode == 0) t0 = r;
        else if (mode == 1) t0 = ulpStep(r, static_cast<int>(splitmix(x) % 9) - 4);
        else if (mode == 2) t0 = static_cast<T>(base + (uni(x) * 3.0 - 1.0) * hsMax);
        else if (mode == 3) t0 = static_cast<T>(1.e10);
        else if (mode == 4) t0 = static_cast<T>(static_cast<double>(r) * (1.0 + (uni(x) * 2.0 - 1.0) * 1e-6));
        else t0 = ulpStep(t[splitmix(x) % 7], static_cast<int>(splitmix(x) % 9) - 4);
        if (!(t0 >= 0)) t0 = 0;
        const T b = fd3UniformFarBounded<T>(h, st, t0);
        const T m1 = b < t0 ? b : t0, m2 = r < t0 ? r : t0;
        local[0] += 1;
        local[1] += sameBits(m1, m2) ? 0 : 1;
        local[2] += sameBits(b, t0) ? 1 : 0;
        local[3] += sameBits(r, t0) ? 1 : 0;
    }
    for (int k = 0; k < 4; ++k) atomicAdd(counts + k, local[k]);
}

namespace {

constexpr int kThreads = 256;

inline int blocksFor(long long n) {
    long long b = (n + kThreads - 1) / kThreads;
    if (b < 1) b = 1;
    if (b > 152LL * 32) b = 152LL * 32;
    return static_cast<int>(b);
}

template <class T>
__device__ __forceinline__ T axisDerivative(const T *t, long long i, long long stride, int k, int n, T twodi) {
    if (k == 0) return (-3 * t[i] + 4 * t[i + stride] - t[i + 2 * stride]) * twodi;
    if (k == n - 1) return (t[i - 2 * stride] - 4 * t[i - stride] + 3 * t[i]) * twodi;
    return (t[i + stride] - t[i - stride]) * twodi;
}

// grad[3 i + (0, 1, 2)] at natural node i; the field has row pitch Px.
template <class T>
__global__ void gradient3Kernel(const T *tt, int Px, int nx, int ny, int nz, T twodxi, T twodyi, T twodzi, T *grad) {
    const long long n = static_cast<long long>(nx) * ny * nz;
    const long long sy = Px, sz = static_cast<long long>(Px) * ny;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int ix = static_cast<int>(i % nx);
        const long long r = i / nx;
        const int iy = static_cast<int>(r % ny), iz = static_cast<int>(r / ny);
        const long long p = iz * sz + iy * sy + ix;
        grad[3 * i] = axisDerivative(tt, p, 1, ix, nx, twodxi);
        grad[3 * i + 1] = axisDerivative(tt, p, sy, iy, ny, twodyi);
        grad[3 * i + 2] = axisDerivative(tt, p, sz, iz, nz, twodzi);
    }
}

template <class T>
__global__ void gradient2Kernel(const T *tt, int Px, int nx, int nz, T twodxi, T twodzi, T *grad) {
    const long long n = static_cast<long long>(nx) * nz;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int ix = static_cast<int>(i % nx), iz = static_cast<int>(i / nx);
        const long long p = static_cast<long long>(iz) * Px + ix;
        grad[2 * i] = axisDerivative(tt, p, 1, ix, nx, twodxi);
        grad[2 * i + 1] = axisDerivative(tt, p, Px, iz, nz, twodzi);
    }
}

// The source cell's corners (one thread each): the analytic gradient of a constant-slowness
// cell, for the axes along which the source is off the corner by more than 1e-7 m.
template <class T>
__global__ void sourceCorners3Kernel(T *grad, int nx, int ny, Corner3 c, double dx, double dy, double dz, int dim) {
    const int t = threadIdx.x;
    if (t >= (dim == 3 ? 8 : 4)) return;
    const int i = t & 1, j = dim == 3 ? (t >> 1) & 1 : 0, k = dim == 3 ? t >> 2 : (t >> 1) & 1;
    const double tol = 1.e-7;
    const double d0x = c.isx * dx - c.xo, d0y = c.isy * dy - c.yo, d0z = c.isz * dz - c.zo;
    const bool doX = fabs(d0x) > tol, doY = dim == 3 && fabs(d0y) > tol, doZ = fabs(d0z) > tol;
    if (!(doX || doY || doZ)) return;
    const double a = i ? (c.isx + 1) * dx - c.xo : d0x;
    const double b = j ? (c.isy + 1) * dy - c.yo : d0y;
    const double e = k ? (c.isz + 1) * dz - c.zo : d0z;
    const T slow0 = static_cast<T>(c.s);
    if (dim == 3) {
        const double r = sqrt(a * a + b * b + e * e);
        const long long n = (static_cast<long long>(c.isz + k) * ny + (c.isy + j)) * nx + (c.isx + i);
        if (doX) grad[3 * n] = static_cast<T>((a / r) * slow0);
        if (doY) grad[3 * n + 1] = static_cast<T>((b / r) * slow0);
        if (doZ) grad[3 * n + 2] = static_cast<T>((e / r) * slow0);
    } else {
        const double r = sqrt(a * a + e * e);
        const long long n = static_cast<long long>(c.isz + k) * nx + (c.isx + i);
        if (doX) grad[2 * n] = static_cast<T>((a / r) * slow0);
        if (doZ) grad[2 * n + 1] = static_cast<T>((e / r) * slow0);
    }
}

// Station times: cells (cx, cy, cz) and offsets (x, y, z) from the origin per station.
template <class T>
__global__ void stations3Kernel(const T *tt, int Px, int ny, double dx, double dy, double dz, Corner3 src, int n,
                                const int *cells, const double *offs, double *out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int cx = cells[3 * s], cy = cells[3 * s + 1], cz = cells[3 * s + 2];
    const double xi = offs[3 * s], yi = offs[3 * s + 1], zi = offs[3 * s + 2];
    const double sSrc = src.s;
    if (cx == src.isx && cy == src.isy && cz == src.isz) {
        const double a = xi - src.xo, b = yi - src.yo, c = zi - src.zo;
        out[s] = sqrt(a * a + b * b + c * c) * sSrc;
        return;
    }
    const long long sy = Px, sz = static_cast<long long>(Px) * ny;
    const long long i0 = cz * sz + cy * sy + cx;
    auto f = [&](int i, int j, int k) { return static_cast<double>(tt[i0 + k * sz + j * sy + i]); };
    const double dxi = 1. / dx, dyi = 1. / dy, dzi = 1. / dz;
    const double x1 = cx * dx, x2 = (cx + 1) * dx, y1 = cy * dy, y2 = (cy + 1) * dy;
    const double z1 = cz * dz, z2 = (cz + 1) * dz;
    const double x2mx = x2 - xi, xmx1 = xi - x1;
    const double f11 = dxi * (x2mx * f(0, 0, 0) + xmx1 * f(1, 0, 0));
    const double f21 = dxi * (x2mx * f(0, 1, 0) + xmx1 * f(1, 1, 0));
    const double f12 = dxi * (x2mx * f(0, 0, 1) + xmx1 * f(1, 0, 1));
    const double f22 = dxi * (x2mx * f(0, 1, 1) + xmx1 * f(1, 1, 1));
    const double y2my = y2 - yi, ymy1 = yi - y1;
    const double fz1 = dyi * (y2my * f11 + ymy1 * f21);
    const double fz2 = dyi * (y2my * f12 + ymy1 * f22);
    out[s] = dzi * ((z2 - zi) * fz1 + (zi - z1) * fz2);
}

template <class T>
__global__ void stations2Kernel(const T *tt, int Px, double dx, double dz, Corner3 src, int n, const int *cells,
                                const double *offs, double *out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int cx = cells[2 * s], cz = cells[2 * s + 1];
    const double xi = offs[2 * s], zi = offs[2 * s + 1];
    if (cx == src.isx && cz == src.isz) {
        out[s] = eikxHypot(xi - src.xo, zi - src.zo) * src.s;
        return;
    }
    const long long i00 = static_cast<long long>(cz) * Px + cx;
    const double f00 = tt[i00], f10 = tt[i00 + 1], f01 = tt[i00 + Px], f11 = tt[i00 + Px + 1];
    const double dxi = 1. / dx, dzi = 1. / dz;
    const double x1 = cx * dx, x2 = (cx + 1) * dx, z1 = cz * dz, z2 = (cz + 1) * dz;
    const double x2mx = x2 - xi, xmx1 = xi - x1;
    const double fxz1 = dxi * (x2mx * f00 + xmx1 * f10);
    const double fxz2 = dxi * (x2mx * f01 + xmx1 * f11);
    out[s] = dzi * ((z2 - zi) * fxz1 + (zi - z1) * fxz2);
}

}  // namespace

template <class T>
cudaError_t launchGradient(const T *tt, int dim, int Px, int nx, int ny, int nz, double dx, double dy, double dz,
                           const Corner3 &src, T *grad, cudaStream_t s) {
    const long long n = static_cast<long long>(nx) * ny * nz;
    const T twodxi = static_cast<T>(1. / (2. * dx)), twodyi = static_cast<T>(1. / (2. * dy));
    const T twodzi = static_cast<T>(1. / (2. * dz));
    if (dim == 3) gradient3Kernel<T><<<blocksFor(n), kThreads, 0, s>>>(tt, Px, nx, ny, nz, twodxi, twodyi, twodzi, grad);
    else gradient2Kernel<T><<<blocksFor(n), kThreads, 0, s>>>(tt, Px, nx, nz, twodxi, twodzi, grad);
    sourceCorners3Kernel<T><<<1, 32, 0, s>>>(grad, nx, ny, src, dx, dy, dz, dim);
    return cudaGetLastError();
}

template <class T>
cudaError_t launchStations(const T *tt, int dim, int Px, int ny, double dx, double dy, double dz, const Corner3 &src,
                           int n, const int *cells, const double *offs, double *out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int blocks = (n + kThreads - 1) / kThreads;
    if (dim == 3) stations3Kernel<T><<<blocks, kThreads, 0, s>>>(tt, Px, ny, dx, dy, dz, src, n, cells, offs, out);
    else stations2Kernel<T><<<blocks, kThreads, 0, s>>>(tt, Px, dx, dz, src, n, cells, offs, out);
    return cudaGetLastError();
}

template cudaError_t launchGradient<float>(const float *, int, int, int, int, int, double, double, double,
                                           const Corner3 &, float *, cudaStream_t);
template cudaError_t launchGradient<double>(const double *, int, int, int, int, int, double, double, double,
                                            const Corner3 &, double *, cudaStream_t);
template cudaError_t launchStations<float>(const float *, int, int, int, double, double, double, const Corner3 &, int,
                                           const int *, const double *, double *, cudaStream_t);
template cudaError_t launchStations<double>(const double *, int, int, int, double, double, double, const Corner3 &,
                                            int, const int *, const double *, double *, cudaStream_t);

// The operator self-test (see operatorSelftestKernel): counts[4] on the device.
cudaError_t launchOperatorSelftest(int precision, long long n, unsigned long long seed, unsigned long long *counts,
                                   cudaStream_t s) {
    const int blocks = 152 * 8;
    if (precision == 0) operatorSelftestKernel<float><<<blocks, 256, 0, s>>>(n, seed, counts);
    else operatorSelftestKernel<double><<<blocks, 256, 0, s>>>(n, seed, counts);
    return cudaGetLastError();
}

}  // namespace eikx

