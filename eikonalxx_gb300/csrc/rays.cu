// 2D gradient ray tracing (Ray::GradientTracer2D::trace, src/ray/gradientTracer2d.cpp:339-600),
// one thread per station:
//   * march from the station down the travel-time gradient, bilinearly interpolated in the
//     current cell (src/ray/bilinear.hpp), with step lengths scaled by the distance in cells
//     from the source (GradientTracerOptions, src/ray/gradientTracerOptions.cpp), until the
//     ray ends within one cell of the source cell;
//   * turn the march around and heal it into segments that end where the ray leaves a cell
//     (intersect, gradientTracer2d.cpp:137-196), each with the slowness of its cell.
// All arithmetic is FP64.  The march points of a station live in a scratch row of
// `maxSteps + 1` points; the march is bounded by maxSteps (the reference has no bound).
#include "sweep.h"

namespace eikx {

namespace {

__device__ __forceinline__ int clampCell(int v, int n) { return v < 0 ? 0 : (v > n - 1 ? n - 1 : v); }

template <class T>
__global__ void traceRays2Kernel(RayTrace2Args a, const T *grad, int n, const double *stations, double *pos,
                                 double *segments, int *counts) {
    const int st = blockIdx.x * blockDim.x + threadIdx.x;
    if (st >= n) return;
    const int nx = a.nx, nz = a.nz, ncx = nx - 1, ncz = nz - 1;
    const double dx = a.dx, dz = a.dz, dxi = 1. / dx, dzi = 1. / dz, hmin = fmin(dx, dz);
    const double xs = a.xs, zs = a.zs;
    const int isx = a.isx, isz = a.isz;
    const double xr = stations[2 * st] - a.x0, zr = stations[2 * st + 1] - a.z0;
    double *seg = segments + static_cast<long long>(st) * a.capacity * 6;
    double *p = pos + static_cast<long long>(st) * (a.maxSteps + 1) * 2;
    auto slowAt = [&](int cx, int cz) {
        return a.slow[static_cast<long long>(clampCell(cz, ncz)) * ncx + clampCell(cx, ncx)];
    };
    const int scx = min(nx - 2, static_cast<int>(xr / dx)), scz = min(nz - 2, static_cast<int>(zr / dz));
    const double sourceSlowness = slowAt(isx, isz), stationSlowness = slowAt(scx, scz);
    int nSeg = 0;
    auto put = [&](double ax, double az, double bx, double bz, double s, int cell) {
        if (nSeg >= a.capacity) return false;
        double *o = seg + 6 * static_cast<long long>(nSeg++);
        o[0] = ax; o[1] = az; o[2] = bx; o[3] = bz; o[4] = s; o[5] = cell;
        return true;
    };
    // source and station in one cell: the straight segment
    if (scz * ncx + scx == isz * ncx + isx) {
        counts[st] = put(a.x0 + xs, a.z0 + zs, a.x0 + xr, a.z0 + zr, stationSlowness, scz * ncx + scx) ? 1 : -2;
        return;
    }
    // gradient nodes past the end of the array are used only with weight 0 (rays on the
    // last row or column): they read as 0
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
    double xa = xr, za = zr;
    int cx0 = -1, cz0 = -1;
    double gx000 = 1.e10, gz000 = 1.e10, gx100 = 1.e10, gz100 = 1.e10;
    double gx010 = 1.e10, gz010 = 1.e10, gx110 = 1.e10, gz110 = 1.e10;
    double stepLength0 = a.rsfScale[a.nRsf - 1] * hmin;
    int m = 0;
    p[0] = xr; p[1] = zr;
    bool converged = false;
    for (int step = 0; step < a.maxSteps; ++step) {
        const int cxs = static_cast<int>(xa / dx), czs = static_cast<int>(za / dz);
        if (cxs < 0 || cxs > nx - 1 || czs < 0 || czs > nz - 1) {
            counts[st] = -3;   // the march left the grid
            return;
        }
        double stepLength = stepLength0;
        double gx00 = gx000, gz00 = gz000, gx10 = gx100, gz10 = gz100;
        double gx01 = gx010, gz01 = gz010, gx11 = gx110, gz11 = gz110;
        if (cxs != cx0 || czs != cz0) {
            const int dist = min(abs(isx - cxs), abs(isz - czs));
            stepLength = a.rsfScale[a.nRsf - 1] * hmin;
            for (int k = 0; k < a.nRsf; ++k)
                if (a.rsfRadius[k] >= dist) {
                    stepLength = a.rsfScale[k] * hmin;
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
        const double gx = bilinear(xa, za, cxs * dx, (cxs + 1) * dx, czs * dz, (czs + 1) * dz, gx00, gx01, gx10, gx11);
        const double gz = bilinear(xa, za, cxs * dx, (cxs + 1) * dx, czs * dz, (czs + 1) * dz, gz00, gz01, gz10, gz11);
        const double gStep = stepLength / eikxHypot(gx, gz);
        const double xe = xa - gx * gStep, ze = za - gz * gStep;
        ++m;
        p[2 * m] = xe; p[2 * m + 1] = ze;
        const int cxe = static_cast<int>(xe / dx), cze = static_cast<int>(ze / dz);
        if (abs(cxe - isx) < 2 && abs(cze - isz) < 2) {
            converged = true;
            break;
        }
        stepLength0 = stepLength;
        xa = xe; za = ze;
        cx0 = cxs; cz0 = czs;
        gx000 = gx00; gz000 = gz00; gx100 = gx10; gz100 = gz10;
        gx010 = gx01; gz010 = gz01; gx110 = gx11; gz110 = gz11;
    }
    if (!converged) {
        counts[st] = -1;   // did not reach the source within maxSteps
        return;
    }
    // healing, from the source: R_0 = source -> p_m, R_j = p_{m-j+1} -> p_{m-j}
    double ha = xs, hz = zs;
    for (int j = 0; j <= m; ++j) {
        if (j == m) {
            if (!put(a.x0 + ha, a.z0 + hz, a.x0 + xr, a.z0 + zr, stationSlowness, -1)) {
                counts[st] = -2;
                return;
            }
            break;
        }
        const int kb = m - j;          // end point of R_j
        const double bx = p[2 * kb], bz = p[2 * kb + 1];
        const double ax = j == 0 ? xs : p[2 * (kb + 1)], az = j == 0 ? zs : p[2 * (kb + 1) + 1];
        const int c0x = j == 0 ? isx : static_cast<int>(ax / dx), c0z = j == 0 ? isz : static_cast<int>(az / dz);
        const int c1x = static_cast<int>(bx / dx), c1z = static_cast<int>(bz / dz);
        if (c0x != c1x || c0z != c1z) {
            double ux = bx - ax, uz = bz - az;
            const double un = eikxHypot(ux, uz);
            ux = ux / un;
            uz = uz / un;
            double ti = 1.e10, tj = 1.e10;
            const double wx0 = c0x * dx, wx1 = (c0x + 1) * dx, wz0 = c0z * dz, wz1 = (c0z + 1) * dz;
            if (ux > 0) ti = (wx1 - ha) / ux;
            else if (ux < 0) ti = (wx0 - ha) / ux;
            if (uz > 0) tj = (wz1 - hz) / uz;
            else if (uz < 0) tj = (wz0 - hz) / uz;
            const double fxi = ha + ux * ti, fzi = hz + uz * ti;
            const double fxj = ha + ux * tj, fzj = hz + uz * tj;
            const double li = (fxi - ha) * (fxi - ha) + (fzi - hz) * (fzi - hz);
            const double lj = (fxj - ha) * (fxj - ha) + (fzj - hz) * (fzj - hz);
            const double xb = li < lj ? fxi : fxj, zb = li < lj ? fzi : fzj;
            if (!put(a.x0 + ha, a.z0 + hz, a.x0 + xb, a.z0 + zb, j == 0 ? sourceSlowness : slowAt(c0x, c0z), -1)) {
                counts[st] = -2;
                return;
            }
            ha = xb;
            hz = zb;
        }
    }
    counts[st] = nSeg;
}

}  // namespace

template <class T>
cudaError_t launchTraceRays2(const RayTrace2Args &a, const T *grad, int n, const double *stations, double *pos,
                             double *segments, int *counts, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    traceRays2Kernel<T><<<(n + 63) / 64, 64, 0, s>>>(a, grad, n, stations, pos, segments, counts);
    return cudaGetLastError();
}

template cudaError_t launchTraceRays2<float>(const RayTrace2Args &, const float *, int, const double *, double *,
                                             double *, int *, cudaStream_t);
template cudaError_t launchTraceRays2<double>(const RayTrace2Args &, const double *, int, const double *, double *,
                                              double *, int *, cudaStream_t);

}  // namespace eikx
