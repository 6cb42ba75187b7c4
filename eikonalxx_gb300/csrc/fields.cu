// Per-field kernels around the sweeps: source initialisation, model preparation,
// solve-state reset, the per-iteration convergence check and the analytic fields.
// All are single-pass and HBM-bound; grids are sized in multiples of the SM count by
// the caller's grid-stride loops.
#include "sweep.h"
#include <cmath>

namespace eikx {

namespace {

constexpr int kThreads = 256;

inline int gridFor(long long n, int threads = kThreads) {
    long long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 152LL * 32) b = 152LL * 32;
    return static_cast<int>(b);
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return max(lo, min(hi, v)); }

// Raises *flag when a velocity or slowness is not a positive finite number (Model3D
// rejects non-positive velocities, src/model3d.cpp:301-305).
template <class U>
__global__ void positiveKernel(const U *s, long long n, int *flag) {
    bool bad = false;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const U v = s[i];
        bad = bad || !(v > 0) || !isfinite(v);
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// Travel-time initialisation (Solver3D::initializeTravelTimes, src/solver3d.cpp:21-84):
// every node := HUGE, the 8 corners of the source cell := s_src * |x - x_s|, the
// distance and product evaluated in FP64 (fp64 = 1) or in the field type.  Two passes:
// a streaming fill of HUGE over every field (16-byte stores; the pitched rows' padding
// included), then one thread per source-cell corner.
template <class T>
__global__ void fillHugeKernel(uint4 *tt, long long n16) {
    const T huge = static_cast<T>(1.e10);
    uint4 v;
    T *e = reinterpret_cast<T *>(&v);
#pragma unroll
    for (int k = 0; k < static_cast<int>(16 / sizeof(T)); ++k) e[k] = huge;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n16;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        tt[i] = v;
}
template <class T>
__global__ void init3CornerKernel(T *tt, int nFields, long long fieldStride, int pitch, int nx, int ny, int nz,
                                  double dx, double dy, double dz, const Corner3 *corners, int fp64) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 8 * nFields) return;
    const int f = i >> 3, k = i & 7;
    const Corner3 cn = corners[f];
    const int ix = cn.isx + (k & 1), iy = cn.isy + ((k >> 1) & 1), iz = cn.isz + ((k >> 2) & 1);
    if (ix >= nx || iy >= ny || iz >= nz) return;
    T v;
    if (fp64) {
        v = static_cast<T>(analyticT3<double>(ix, iy, iz, dx, dy, dz, cn.xo, cn.yo, cn.zo, cn.s));
    } else {
        v = analyticT3<T>(ix, iy, iz, static_cast<T>(dx), static_cast<T>(dy), static_cast<T>(dz),
                          static_cast<T>(cn.xo), static_cast<T>(cn.yo), static_cast<T>(cn.zo),
                          static_cast<T>(cn.s));
    }
    tt[static_cast<long long>(f) * fieldStride + (static_cast<long long>(iz) * ny + iy) * pitch + ix] = v;
}

// Warm start of a 3D solve from an initial field (natural order): the field is taken as
// given except where the local solver shows it underestimates.  For every node the
// upwind update is evaluated from the initial field in all 8 sweep orderings (the
// stencils of Solver3DSweep::updateFSM, neighbours clamped to the grid); a node whose
// initial time lies more than gateTol below the smallest of them is lower than any of
// its neighbourhoods supports -- sweeps only lower times, so it could never recover --
// and is reset to HUGE.  A corner of the source cell keeps the smaller of its initial
// value and the analytic initialisation (the cold start begins at the analytic value and
// its sweeps may lower it, so a converged field starts where it ended); one the gate
// rejects takes the analytic value.  Only values of the initial field are read, so the
// pass is order-independent.
template <class T, bool UNIFORM>
__global__ void warmInit3Kernel(T *tt, const T *init, int nFields, long long fieldStride, int pitch, int nx, int ny,
                                int nz, double dx, double dy, double dz, const Corner3 *corners,
                                const SourceT<T> *srcs, const double *slow, int radius, T h, Spacing3<T> g,
                                double gateTol, int twoSided, int fp64, const SourceFp64 *srcs64,
                                unsigned long long *nReset) {
    const long long perField = static_cast<long long>(nx) * ny * nz;
    const long long n = perField * nFields;
    const int ncx = nx - 1, ncy = ny - 1, ncz = nz - 1;
    unsigned long long resets = 0;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int f = static_cast<int>(i / perField);
        const long long r = i - f * perField;
        const int ix = static_cast<int>(r % nx);
        const int iy = static_cast<int>((r / nx) % ny);
        const int iz = static_cast<int>(r / (static_cast<long long>(nx) * ny));
        const Corner3 cn = corners[f];
        const T *fi = init + static_cast<long long>(f) * perField;
        const bool corner = ix - cn.isx >= 0 && ix - cn.isx <= 1 && iy - cn.isy >= 0 && iy - cn.isy <= 1 &&
                            iz - cn.isz >= 0 && iz - cn.isz <= 1;
        T v = fi[r];
        {
            const SourceT<T> src = srcs[f];
            T uMin = static_cast<T>(1.e10);
            for (int e = 0; e < 8; ++e) {
                const int fx = e & 1, fy = (e >> 1) & 1, fz = (e >> 2) & 1;
                SweepSigns sg;
                sg.ixShift = fx ? 1 : -1; sg.iyShift = fy ? 1 : -1; sg.izShift = fz ? 1 : -1;
                sg.signX = fx ? -1 : 1; sg.signY = fy ? -1 : 1; sg.signZ = fz ? -1 : 1;
                auto clampi_ = [](int a, int lo, int hi) { return a < lo ? lo : (a > hi ? hi : a); };
                const int cxu = fx ? clampi_(ix, 0, ncx - 1) : clampi_(ix - 1, 0, ncx - 1);
                const int cxo = fx ? clampi_(cxu - 1, 0, ncx - 1) : clampi_(cxu + 1, 0, ncx - 1);
                const int cyu = fy ? clampi_(iy, 0, ncy - 1) : clampi_(iy - 1, 0, ncy - 1);
                const int cyo = fy ? clampi_(cyu - 1, 0, ncy - 1) : clampi_(cyu + 1, 0, ncy - 1);
                const int czu = fz ? clampi_(iz, 0, ncz - 1) : clampi_(iz - 1, 0, ncz - 1);
                const int czo = fz ? clampi_(czu - 1, 0, ncz - 1) : clampi_(czu + 1, 0, ncz - 1);
                auto cell = [&](int x, int y, int z) {
                    return static_cast<T>(slow[(static_cast<long long>(z) * ncy + y) * ncx + x]);
                };
                const int xs = clampi_(ix + sg.ixShift, 0, nx - 1), ys = clampi_(iy + sg.iyShift, 0, ny - 1);
                const int zs = clampi_(iz + sg.izShift, 0, nz - 1);
                auto tv = [&](int x, int y, int z) { return fi[(static_cast<long long>(z) * ny + y) * nx + x]; };
                Stencil3<T> st;
                st.s0 = cell(cxu, cyu, czu); st.s1 = cell(cxo, cyu, czu); st.s2 = cell(cxo, cyo, czu);
                st.s3 = cell(cxu, cyo, czu); st.s4 = cell(cxu, cyu, czo); st.s5 = cell(cxo, cyu, czo);
                st.s7 = cell(cxu, cyo, czo);
                st.t1 = tv(xs, iy, iz); st.t2 = tv(xs, ys, iz); st.t3 = tv(ix, ys, iz); st.t4 = tv(ix, iy, zs);
                st.t5 = tv(xs, iy, zs); st.t6 = tv(xs, ys, zs); st.t7 = tv(ix, ys, zs);
                // a near_fp64 solve gates with the FP64 analytic factor its sweeps use
                T u;
                if (srcs64 && nearSource(radius, src.isx, src.isy, src.isz, ix, iy, iz)) {
                    u = UNIFORM ? fd3UniformNear<T, true>(h, src, sg, ix, iy, iz, st, srcs64 + f)
                                : fd3NonUniformNear<T, true>(g, src, sg, ix, iy, iz, st, srcs64 + f);
                } else {
                    u = UNIFORM ? fd3Uniform<T>(radius, h, src, sg, ix, iy, iz, st)
                                : fd3NonUniform<T>(radius, g, src, sg, ix, iy, iz, st);
                }
                uMin = u < uMin ? u : uMin;
            }
            // one-sided: reset what sweeps could not raise; two-sided: also what lies above
            // the update its neighbourhood gives
            const bool under = static_cast<double>(v) < static_cast<double>(uMin) - gateTol ||
                               (twoSided && static_cast<double>(v) > static_cast<double>(uMin) + gateTol);
            if (corner) {
                const T an = fp64 ? static_cast<T>(analyticT3<double>(ix, iy, iz, dx, dy, dz, cn.xo, cn.yo, cn.zo, cn.s))
                                  : analyticT3<T>(ix, iy, iz, static_cast<T>(dx), static_cast<T>(dy),
                                                  static_cast<T>(dz), static_cast<T>(cn.xo), static_cast<T>(cn.yo),
                                                  static_cast<T>(cn.zo), static_cast<T>(cn.s));
                v = under || !(v < an) ? an : v;
            } else if (under) {
                v = static_cast<T>(1.e10);
            }
            if (under) ++resets;
        }
        tt[static_cast<long long>(f) * fieldStride + (static_cast<long long>(iz) * ny + iy) * pitch + ix] = v;
    }
    if (resets) atomicAdd(nReset, resets);
}

// FP64 analytic-factor tables (eikx_options.near_fp64): one block per field fills the
// entries of its box of near-source nodes for all 8 sweep orderings (nearFactor, FP64).
__global__ void factorTableKernel(const SourceFp64 *srcs) {
    const SourceFp64 f = srcs[blockIdx.x];
    if (!f.table) return;
    NearFactor *table = const_cast<NearFactor *>(f.table);
    const int box = f.bnx * f.bny * f.bnz;
    auto clampi = [](int a, int lo, int hi) { return a < lo ? lo : (a > hi ? hi : a); };
    for (int i = threadIdx.x; i < 8 * box; i += blockDim.x) {
        const int e = i / box, r = i - e * box;
        const int ix = f.bx0 + r % f.bnx, iy = f.by0 + (r / f.bnx) % f.bny, iz = f.bz0 + r / (f.bnx * f.bny);
        const int fx = e & 1, fy = (e >> 1) & 1, fz = (e >> 2) & 1;
        SweepSigns sg;
        sg.ixShift = fx ? 1 : -1; sg.iyShift = fy ? 1 : -1; sg.izShift = fz ? 1 : -1;
        sg.signX = fx ? -1 : 1; sg.signY = fy ? -1 : 1; sg.signZ = fz ? -1 : 1;
        // the node's home cell in this ordering (the sweep's s0)
        const int cx = fx ? clampi(ix, 0, f.ncx - 1) : clampi(ix - 1, 0, f.ncx - 1);
        const int cy = fy ? clampi(iy, 0, f.ncy - 1) : clampi(iy - 1, 0, f.ncy - 1);
        const int cz = fz ? clampi(iz, 0, f.ncz - 1) : clampi(iz - 1, 0, f.ncz - 1);
        const float s0 = f.sp[(cz + 1) * f.spPlane + static_cast<long long>(cy + 1) * f.spPitch + cx + 1];
        table[i] = nearFactor(f, s0, sg, ix, iy, iz);
    }
}

// Pads of the pitched rows (x >= nx) stay HUGE in a warm start.
template <class T>
__global__ void fillPadKernel(T *tt, int nFields, long long fieldStride, int pitch, int nx, int rows) {
    const int padW = pitch - nx;
    const long long n = static_cast<long long>(nFields) * rows * padW;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long q = i / padW;
        const int x = nx + static_cast<int>(i % padW);
        const int f = static_cast<int>(q / rows);
        const long long row = q % rows;
        tt[f * fieldStride + row * pitch + x] = static_cast<T>(1.e10);
    }
}

// 2D (Solver2D::initializeTravelTimes, src/solver2d.cpp:61-105).
template <class T>
__global__ void init2Kernel(T *tt, int nFields, long long fieldStride, int pitch, int nx, int nz,
                            double dx, double dz, const Corner3 *corners, int fp64) {
    const long long perField = static_cast<long long>(pitch) * nz;
    const long long n = perField * nFields;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int f = static_cast<int>(i / perField);
        const long long r = i - f * perField;
        const int ix = static_cast<int>(r % pitch);
        const int iz = static_cast<int>(r / pitch);
        const Corner3 cn = corners[f];
        T v = static_cast<T>(1.e10);
        if (ix - cn.isx >= 0 && ix - cn.isx <= 1 && iz - cn.isz >= 0 && iz - cn.isz <= 1 && ix < nx) {
            if (fp64) {
                v = static_cast<T>(analyticT2<double>(ix, iz, dx, dz, cn.xo, cn.zo, cn.s));
            } else {
                v = analyticT2<T>(ix, iz, static_cast<T>(dx), static_cast<T>(dz), static_cast<T>(cn.xo),
                                  static_cast<T>(cn.zo), static_cast<T>(cn.s));
            }
        }
        tt[static_cast<long long>(f) * fieldStride + static_cast<long long>(iz) * pitch + ix] = v;
    }
}

// Edge-replicated slowness: padded cell p holds cell clamp(p - 1) on every axis, so a
// node i reads padded cells i and i + 1 without the clamps of
// gridToSurroundingSlownessIndices (solverUtilities3d.hpp:1300-1442).  Along x the
// copy is stored `shift` columns to the right, which aligns the cells a forward sweep
// streams with the 16-byte chunks of its travel-time rows.
template <class T, class U>
__global__ void pad3Kernel(T *sp, int spPitch, int shift, const U *s, int nx, int ny, int nz, T h) {
    const int ncx = nx - 1, ncy = ny - 1, ncz = nz - 1;
    const long long n = static_cast<long long>(spPitch) * (ny + 1) * (nz + 1);
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int px = static_cast<int>(i % spPitch);
        const long long r = i / spPitch;
        const int py = static_cast<int>(r % (ny + 1));
        const int pz = static_cast<int>(r / (ny + 1));
        const int cx = clampi(px - 1 - shift, 0, ncx - 1), cy = clampi(py - 1, 0, ncy - 1),
                  cz = clampi(pz - 1, 0, ncz - 1);
        const T v = static_cast<T>(s[(static_cast<long long>(cz) * ncy + cy) * ncx + cx]);
        sp[i] = h > 0 ? v * h : v;
    }
}


template <class T, class U>
__global__ void pad2Kernel(T *sp, int spPitch, int shift, const U *s, int nx, int nz) {
    const int ncx = nx - 1, ncz = nz - 1;
    const long long n = static_cast<long long>(spPitch) * (nz + 1);
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int px = static_cast<int>(i % spPitch);
        const int pz = static_cast<int>(i / spPitch);
        const int cx = clampi(px - 1 - shift, 0, ncx - 1), cz = clampi(pz - 1, 0, ncz - 1);
        sp[i] = static_cast<T>(s[static_cast<long long>(cz) * ncx + cx]);
    }
}

// Nodal velocity -> cell slowness = 8 / (sum of the 8 corner velocities), summed in pairs
// as interpolate3d (src/model3d.cpp:79-137); ordering 1 reads the transposed (XYZ) input.
template <class U>
__global__ void nodal3Kernel(double *slow, const U *v, int nx, int ny, int nz, int ordering) {
    const long long ncx = nx - 1, ncy = ny - 1, ncz = nz - 1;
    const long long n = ncx * ncy * ncz;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long ix = i % ncx, iy = (i / ncx) % ncy, iz = i / (ncx * ncy);
        long long i1, i3, i5;
        long long d1, d3, d5;  // strides of +x, +y, +z in the input
        if (ordering == 0) {
            d1 = 1; d3 = ncx + 1; d5 = (ncx + 1) * (ncy + 1);
            i1 = iz * d5 + iy * d3 + ix;
        } else {
            d1 = static_cast<long long>(ncz + 1) * (ncy + 1); d3 = ncz + 1; d5 = 1;
            // the reference's transposed indices: idx1 = ix*(ncz+1)*(ncy+1) + iy*(ncz+1) + iz,
            // idx2 = idx1 + 1, idx3 = idx1 + (ncz+1), idx5 = idx1 + (ncz+1)*(ncy+1)
            i1 = ix * d1 + iy * d3 + iz;
            d1 = 1; d5 = static_cast<long long>(ncz + 1) * (ncy + 1);
        }
        i3 = i1 + d3;
        i5 = i1 + d5;
        const U sum1 = v[i1] + v[i1 + d1];
        const U sum2 = v[i3] + v[i3 + d1];
        const U sum3 = v[i5] + v[i5 + d1];
        const U sum4 = v[i5 + d3] + v[i5 + d3 + d1];
        const U eight = 8;
        slow[i] = static_cast<double>(eight / (sum1 + sum2 + sum3 + sum4));
    }
}

template <class U>
__global__ void nodal2Kernel(double *slow, const U *v, int nx, int nz, int ordering) {
    const long long ncx = nx - 1, ncz = nz - 1;
    const long long n = ncx * ncz;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long ix = i % ncx, iz = i / ncx;
        long long i1, d1, d3;
        if (ordering == 0) { i1 = iz * (ncx + 1) + ix; d1 = 1; d3 = ncx + 1; }
        else { i1 = ix * (ncz + 1) + iz; d1 = 1; d3 = ncz + 1; }
        const U sum1 = v[i1] + v[i1 + d1];
        const U sum2 = v[i1 + d3] + v[i1 + d3 + d1];
        const U four = 4;
        slow[i] = static_cast<double>(four / (sum1 + sum2));
    }
}

// Cell values in natural or transposed order -> natural-order slowness (double master).
// `U` values are slowness already (the caller converts velocities on the host side).
template <class U>
__global__ void cells3Kernel(double *slow, const U *c, int nx, int ny, int nz, int ordering) {
    const long long ncx = nx - 1, ncy = ny - 1, ncz = nz - 1;
    const long long n = ncx * ncy * ncz;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long ix = i % ncx, iy = (i / ncx) % ncy, iz = i / (ncx * ncy);
        const long long src = ordering == 0 ? i : (ix * ncy + iy) * ncz + iz;
        slow[i] = static_cast<double>(c[src]);
    }
}

template <class U>
__global__ void cells2Kernel(double *slow, const U *c, int nx, int nz, int ordering) {
    const long long ncx = nx - 1, ncz = nz - 1;
    const long long n = ncx * ncz;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const long long ix = i % ncx, iz = i / ncx;
        const long long src = ordering == 0 ? i : ix * ncz + iz;
        slow[i] = static_cast<double>(c[src]);
    }
}

// Start of a solve: fresh residual slots and flags, and a new range of mailbox tags.  The
// base moves past every tag the previous solve used (epoch[1] holds how many), so words
// written by earlier solves can never match a tag of this one, whatever their sweep
// counts; the first base is 1, so zeroed words (tag 0) never match either.
__global__ void resetKernel(SolveState st, int nFields, int buf) {
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gthreads = gridDim.x * blockDim.x;
    const long long nres = static_cast<long long>(nFields) * st.residualStride;
    for (long long i = gtid; i < nres; i += gthreads) st.residual[i] = 0ull;
    for (int i = gtid; i < nFields; i += gthreads) {
        st.converged[i] = 0;
        st.sweepsRun[i] = 0;
    }
    if (gtid == 0) {
        *st.queue[buf] = 0u;
        *st.abortFlag = 0;
        st.epoch[0] += st.epoch[1] + 1u;
        st.epoch[1] = static_cast<unsigned>(st.epochStride);
    }
}

// After a refinement sweep: a field whose largest decrease in each of the last sweeps of the
// window (slots [firstSlot, firstSlot + nSlots)) fell below tol is frozen; later sweeps skip it.
__global__ void checkKernel(SolveState st, int nFields, int firstSlot, int nSlots, int sweepsDone,
                            double tol) {
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nFields; f += gridDim.x * blockDim.x) {
        if (st.converged[f]) continue;
        double m = 0;
        for (int k = 0; k < nSlots; ++k)
            m = fmax(m, __longlong_as_double(static_cast<long long>(
                            st.residual[static_cast<long long>(f) * st.residualStride + firstSlot + k])));
        st.sweepsRun[f] = sweepsDone;
        if (m < tol) st.converged[f] = 1;
    }
}

// The same test in a stream of sources through slots (eikx_options.max_in_flight): after
// sweep `sweepIndex` of the stream, slot f's field has run sweepIndex - slots[f].x + 1 sweeps
// of its own, the first 8 its initialisation pass when initSweeps is set.
__global__ void checkStreamKernel(SolveState st, const int2 *slots, int nSlots, int sweepIndex, int initSweeps,
                                  double tol) {
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nSlots; f += gridDim.x * blockDim.x) {
        const int start = slots[f].x;
        if (start < 0 || st.converged[f]) continue;
        const int r = sweepIndex - start - (initSweeps ? 8 : 0);   // refinement sweep just run
        if (r < 0) continue;
        const int lo = r > 7 ? r - 7 : 0;
        double m = 0;
        for (int k = lo; k <= r; ++k)
            m = fmax(m, __longlong_as_double(static_cast<long long>(
                            st.residual[static_cast<long long>(f) * st.residualStride + 8 + k])));
        st.sweepsRun[f] = r + 1;
        if (r >= 7 && m < tol) st.converged[f] = 1;
    }
}

// A slot takes a new source (stream mode): its field buffer slots[f].y := HUGE (16-byte
// stores), then the source-cell corners, its residual row, flag and sweep count cleared.
template <class T>
__global__ void refillFillKernel(uint4 *tt, long long fieldStride16, const int2 *slots, const int *list, int n) {
    const long long total = fieldStride16 * n;
    const T huge = static_cast<T>(1.e10);
    uint4 v;
    T *e = reinterpret_cast<T *>(&v);
#pragma unroll
    for (int k = 0; k < static_cast<int>(16 / sizeof(T)); ++k) e[k] = huge;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int f = list[i / fieldStride16];
        tt[static_cast<long long>(slots[f].y) * fieldStride16 + i % fieldStride16] = v;
    }
}
template <class T>
__global__ void refillSlotKernel(T *tt, SolveState st, long long fieldStride, int pitch, int nx, int ny, int nz,
                                 double dx, double dy, double dz, const Corner3 *corners, int fp64, const int2 *slots,
                                 const int *list, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 8 * n) return;
    const int f = list[i >> 3], k = i & 7;
    if (k == 0) {
        for (int r = 0; r < st.residualStride; ++r) st.residual[static_cast<long long>(f) * st.residualStride + r] = 0ull;
        st.converged[f] = 0;
        st.sweepsRun[f] = 0;
    }
    const Corner3 cn = corners[f];
    const int ix = cn.isx + (k & 1), iy = cn.isy + ((k >> 1) & 1), iz = cn.isz + ((k >> 2) & 1);
    if (ix >= nx || iy >= ny || iz >= nz) return;
    T v;
    if (fp64) {
        v = static_cast<T>(analyticT3<double>(ix, iy, iz, dx, dy, dz, cn.xo, cn.yo, cn.zo, cn.s));
    } else {
        v = analyticT3<T>(ix, iy, iz, static_cast<T>(dx), static_cast<T>(dy), static_cast<T>(dz),
                          static_cast<T>(cn.xo), static_cast<T>(cn.yo), static_cast<T>(cn.zo),
                          static_cast<T>(cn.s));
    }
    tt[static_cast<long long>(slots[f].y) * fieldStride + (static_cast<long long>(iz) * ny + iy) * pitch + ix] = v;
}

// Analytic linear-gradient / homogeneous travel times in FP64
// (src/analytic/linearGradient3d.cpp:12-116, linearGradient2d.cpp:12-124).
__global__ void analytic3Kernel(double *t, int nx, int ny, int nz, double dx, double dy, double dz,
                                double xs, double ys, double zs, double vTop, double vBottom) {
    const double gz = (vBottom - vTop) / ((nz - 1) * dz);
    const double absG2 = gz * gz;
    const double absG = sqrt(absG2);
    const double v0 = vTop + gz * zs;
    const double s0 = 1 / v0;
    const bool gradient = fabs(vTop - vBottom) > 1.e-14;
    const long long n = static_cast<long long>(nx) * ny * nz;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int ix = static_cast<int>(i % nx);
        const int iy = static_cast<int>((i / nx) % ny);
        const int iz = static_cast<int>(i / (static_cast<long long>(nx) * ny));
        if (gradient) {
            const double ddx = ix * dx - xs, ddy = iy * dy - ys, ddz = iz * dz - zs;
            const double dist2 = ddx * ddx + ddy * ddy + ddz * ddz;
            const double vel = v0 + 0 * ddx + 0 * ddy + gz * ddz;
            const double arg = 1 + (s0 * absG2 * dist2) / (2 * vel);
            t[i] = acosh(arg) / absG;
        } else {
            const double ddx = xs - ix * dx, ddy = ys - iy * dy, ddz = zs - iz * dz;
            t[i] = sqrt(ddx * ddx + ddy * ddy + ddz * ddz) * s0;
        }
    }
}

__global__ void analytic2Kernel(double *t, int nx, int nz, double dx, double dz, double xs, double zs,
                                double vTop, double vBottom) {
    const double gz = (vBottom - vTop) / ((nz - 1) * dz);
    const double absG2 = gz * gz;
    const double absG = sqrt(absG2);
    const double v0 = vTop + gz * zs;
    const double s0 = 1 / v0;
    const bool gradient = fabs(vTop - vBottom) > 1.e-14;
    const long long n = static_cast<long long>(nx) * nz;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int ix = static_cast<int>(i % nx);
        const int iz = static_cast<int>(i / nx);
        if (gradient) {
            const double ddx = ix * dx - xs, ddz = iz * dz - zs;
            const double dist2 = ddx * ddx + ddz * ddz;
            const double vel = v0 + 0 * ddx + gz * ddz;
            const double arg = 1 + (s0 * absG2 * dist2) / (2 * vel);
            t[i] = acosh(arg) / absG;
        } else {
            t[i] = hypot(xs - ix * dx, zs - iz * dz) * s0;
        }
    }
}

}  // namespace

template <class T>
cudaError_t launchInit3(T *tt, int nFields, long long fieldStride, int pitch, int nx, int ny, int nz,
                        double dx, double dy, double dz, const Corner3 *corners, int fp64, cudaStream_t s) {
    // the fields are contiguous (fieldStride = pitch * ny * nz) and pitch * sizeof(T) is a
    // multiple of 16 bytes, so the fill covers them in 16-byte stores
    const long long n16 = fieldStride * nFields * static_cast<long long>(sizeof(T)) / 16;
    fillHugeKernel<T><<<gridFor(n16), kThreads, 0, s>>>(reinterpret_cast<uint4 *>(tt), n16);
    init3CornerKernel<T><<<(8 * nFields + kThreads - 1) / kThreads, kThreads, 0, s>>>(
        tt, nFields, fieldStride, pitch, nx, ny, nz, dx, dy, dz, corners, fp64);
    return cudaGetLastError();
}
template <class T>
cudaError_t launchInit2(T *tt, int nFields, long long fieldStride, int pitch, int nx, int nz, double dx,
                        double dz, const Corner3 *corners, int fp64, cudaStream_t s) {
    const long long n = static_cast<long long>(pitch) * nz * nFields;
    init2Kernel<T><<<gridFor(n), kThreads, 0, s>>>(tt, nFields, fieldStride, pitch, nx, nz, dx, dz, corners, fp64);
    return cudaGetLastError();
}
template <class T, class U>
cudaError_t launchPadSlowness3(T *sp, int spPitch, int shift, const U *s, int nx, int ny, int nz, cudaStream_t st,
                               T h) {
    const long long n = static_cast<long long>(spPitch) * (ny + 1) * (nz + 1);
    pad3Kernel<T, U><<<gridFor(n), kThreads, 0, st>>>(sp, spPitch, shift, s, nx, ny, nz, h);
    return cudaGetLastError();
}
template <class T, class U>
cudaError_t launchPadSlowness2(T *sp, int spPitch, int shift, const U *s, int nx, int nz, cudaStream_t st) {
    const long long n = static_cast<long long>(spPitch) * (nz + 1);
    pad2Kernel<T, U><<<gridFor(n), kThreads, 0, st>>>(sp, spPitch, shift, s, nx, nz);
    return cudaGetLastError();
}
template <class U>
cudaError_t launchNodalToCell3(double *slow, const U *v, int nx, int ny, int nz, int ordering, cudaStream_t s) {
    const long long n = static_cast<long long>(nx - 1) * (ny - 1) * (nz - 1);
    nodal3Kernel<U><<<gridFor(n), kThreads, 0, s>>>(slow, v, nx, ny, nz, ordering);
    return cudaGetLastError();
}
template <class U>
cudaError_t launchNodalToCell2(double *slow, const U *v, int nx, int nz, int ordering, cudaStream_t s) {
    const long long n = static_cast<long long>(nx - 1) * (nz - 1);
    nodal2Kernel<U><<<gridFor(n), kThreads, 0, s>>>(slow, v, nx, nz, ordering);
    return cudaGetLastError();
}
template <class U>
cudaError_t launchCellsToNatural3(double *slow, const U *c, int nx, int ny, int nz, int ordering, cudaStream_t s) {
    const long long n = static_cast<long long>(nx - 1) * (ny - 1) * (nz - 1);
    cells3Kernel<U><<<gridFor(n), kThreads, 0, s>>>(slow, c, nx, ny, nz, ordering);
    return cudaGetLastError();
}
template <class U>
cudaError_t launchCellsToNatural2(double *slow, const U *c, int nx, int nz, int ordering, cudaStream_t s) {
    const long long n = static_cast<long long>(nx - 1) * (nz - 1);
    cells2Kernel<U><<<gridFor(n), kThreads, 0, s>>>(slow, c, nx, nz, ordering);
    return cudaGetLastError();
}
cudaError_t launchResetState(const SolveState &st, int nFields, int buf, cudaStream_t s) {
    resetKernel<<<gridFor(static_cast<long long>(nFields) * st.residualStride), kThreads, 0, s>>>(st, nFields, buf);
    return cudaGetLastError();
}
template <class T>
cudaError_t launchWarmInit3(T *tt, const T *init, int nFields, long long fieldStride, int pitch, int nx, int ny, int nz,
                            double dx, double dy, double dz, const Corner3 *corners, const SourceT<T> *srcs,
                            const double *slow, int radius, bool uniform, T h, const Spacing3<T> &g, double gateTol,
                            int twoSided, int fp64, const SourceFp64 *srcs64, unsigned long long *nReset,
                            cudaStream_t s) {
    const long long n = static_cast<long long>(nx) * ny * nz * nFields;
    if (uniform)
        warmInit3Kernel<T, true><<<gridFor(n), kThreads, 0, s>>>(tt, init, nFields, fieldStride, pitch, nx, ny, nz, dx,
                                                                 dy, dz, corners, srcs, slow, radius, h, g, gateTol,
                                                                 twoSided, fp64, srcs64, nReset);
    else
        warmInit3Kernel<T, false><<<gridFor(n), kThreads, 0, s>>>(tt, init, nFields, fieldStride, pitch, nx, ny, nz, dx,
                                                                  dy, dz, corners, srcs, slow, radius, h, g, gateTol,
                                                                  twoSided, fp64, srcs64, nReset);
    if (pitch > nx) {
        const long long np = static_cast<long long>(nFields) * ny * nz * (pitch - nx);
        fillPadKernel<T><<<gridFor(np), kThreads, 0, s>>>(tt, nFields, fieldStride, pitch, nx, ny * nz);
    }
    return cudaGetLastError();
}
template cudaError_t launchWarmInit3<float>(float *, const float *, int, long long, int, int, int, int, double, double,
                                            double, const Corner3 *, const SourceT<float> *, const double *, int, bool,
                                            float, const Spacing3<float> &, double, int, int, const SourceFp64 *,
                                            unsigned long long *, cudaStream_t);
template cudaError_t launchWarmInit3<double>(double *, const double *, int, long long, int, int, int, int, double,
                                             double, double, const Corner3 *, const SourceT<double> *, const double *,
                                             int, bool, double, const Spacing3<double> &, double, int, int,
                                             const SourceFp64 *, unsigned long long *, cudaStream_t);

cudaError_t launchFactorTables(const SourceFp64 *srcs, int nFields, cudaStream_t s) {
    factorTableKernel<<<nFields, 256, 0, s>>>(srcs);
    return cudaGetLastError();
}

cudaError_t launchCheckPositive(const double *s, long long n, int *flag, cudaStream_t st) {
    positiveKernel<double><<<gridFor(n), kThreads, 0, st>>>(s, n, flag);
    return cudaGetLastError();
}
cudaError_t launchCheckPositive(const float *s, long long n, int *flag, cudaStream_t st) {
    positiveKernel<float><<<gridFor(n), kThreads, 0, st>>>(s, n, flag);
    return cudaGetLastError();
}

cudaError_t launchCheckConvergence(const SolveState &st, int nFields, int firstSlot, int nSlots, int sweepsDone,
                                   double tol, cudaStream_t s) {
    checkKernel<<<gridFor(nFields, 128), 128, 0, s>>>(st, nFields, firstSlot, nSlots, sweepsDone, tol);
    return cudaGetLastError();
}
cudaError_t launchCheckStream(const SolveState &st, const int2 *slots, int nSlots, int sweepIndex, int initSweeps,
                              double tol, cudaStream_t s) {
    checkStreamKernel<<<gridFor(nSlots, 128), 128, 0, s>>>(st, slots, nSlots, sweepIndex, initSweeps, tol);
    return cudaGetLastError();
}
template <class T>
cudaError_t launchRefillSlots(T *tt, long long fieldStride, int pitch, int nx, int ny, int nz, double dx, double dy,
                              double dz, const SolveState &st, const int2 *slots, const int *list, int n,
                              const Corner3 *corners, int fp64, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    // fieldStride * sizeof(T) is a multiple of 16 bytes (pitch * sizeof(T) is)
    const long long f16 = fieldStride * static_cast<long long>(sizeof(T)) / 16;
    refillFillKernel<T><<<gridFor(f16 * n), kThreads, 0, s>>>(reinterpret_cast<uint4 *>(tt), f16, slots, list, n);
    refillSlotKernel<T><<<(8 * n + kThreads - 1) / kThreads, kThreads, 0, s>>>(
        tt, st, fieldStride, pitch, nx, ny, nz, dx, dy, dz, corners, fp64, slots, list, n);
    return cudaGetLastError();
}
template cudaError_t launchRefillSlots<float>(float *, long long, int, int, int, int, double, double, double,
                                              const SolveState &, const int2 *, const int *, int, const Corner3 *,
                                              int, cudaStream_t);
template cudaError_t launchRefillSlots<double>(double *, long long, int, int, int, int, double, double, double,
                                               const SolveState &, const int2 *, const int *, int, const Corner3 *,
                                               int, cudaStream_t);
cudaError_t launchAnalytic3(double *t, int nx, int ny, int nz, double dx, double dy, double dz, double xs,
                            double ys, double zs, double vTop, double vBottom, cudaStream_t s) {
    const long long n = static_cast<long long>(nx) * ny * nz;
    analytic3Kernel<<<gridFor(n), kThreads, 0, s>>>(t, nx, ny, nz, dx, dy, dz, xs, ys, zs, vTop, vBottom);
    return cudaGetLastError();
}
cudaError_t launchAnalytic2(double *t, int nx, int nz, double dx, double dz, double xs, double zs, double vTop,
                            double vBottom, cudaStream_t s) {
    const long long n = static_cast<long long>(nx) * nz;
    analytic2Kernel<<<gridFor(n), kThreads, 0, s>>>(t, nx, nz, dx, dz, xs, zs, vTop, vBottom);
    return cudaGetLastError();
}

template cudaError_t launchInit3<float>(float *, int, long long, int, int, int, int, double, double, double,
                                        const Corner3 *, int, cudaStream_t);
template cudaError_t launchInit3<double>(double *, int, long long, int, int, int, int, double, double, double,
                                         const Corner3 *, int, cudaStream_t);
template cudaError_t launchInit2<float>(float *, int, long long, int, int, int, double, double, const Corner3 *,
                                        int, cudaStream_t);
template cudaError_t launchInit2<double>(double *, int, long long, int, int, int, double, double,
                                         const Corner3 *, int, cudaStream_t);
template cudaError_t launchPadSlowness3<float, double>(float *, int, int, const double *, int, int, int, cudaStream_t,
                                                       float);
template cudaError_t launchPadSlowness3<double, double>(double *, int, int, const double *, int, int, int,
                                                        cudaStream_t, double);
template cudaError_t launchPadSlowness3<float, float>(float *, int, int, const float *, int, int, int, cudaStream_t,
                                                      float);
template cudaError_t launchPadSlowness2<float, double>(float *, int, int, const double *, int, int, cudaStream_t);
template cudaError_t launchPadSlowness2<double, double>(double *, int, int, const double *, int, int, cudaStream_t);
template cudaError_t launchNodalToCell3<float>(double *, const float *, int, int, int, int, cudaStream_t);
template cudaError_t launchNodalToCell3<double>(double *, const double *, int, int, int, int, cudaStream_t);
template cudaError_t launchNodalToCell2<float>(double *, const float *, int, int, int, cudaStream_t);
template cudaError_t launchNodalToCell2<double>(double *, const double *, int, int, int, cudaStream_t);
template cudaError_t launchCellsToNatural3<float>(double *, const float *, int, int, int, int, cudaStream_t);
template cudaError_t launchCellsToNatural3<double>(double *, const double *, int, int, int, int, cudaStream_t);
template cudaError_t launchCellsToNatural2<float>(double *, const float *, int, int, int, cudaStream_t);
template cudaError_t launchCellsToNatural2<double>(double *, const double *, int, int, int, cudaStream_t);

}  // namespace eikx
