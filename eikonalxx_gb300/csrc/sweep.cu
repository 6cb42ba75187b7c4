// Level-set fast-sweeping kernels (3D and 2D) for sm_103a.
//
// One launch performs one sweep (one of the 8 / 4 orderings) over every field of a
// batch.  The warp-block wavefront is described in wavefront.cuh; the per-node update
// is the reference's local solver (local_solver.cuh).  A node is written back only
// when its time decreases, as Solver3DSweep::updateFSM (include/private/solver3d.hpp:
// 236-240) and Solver2DSweep::updateFSM (include/private/solver2d.hpp:264-271) do; the
// largest decrease of the sweep is reduced per warp with shuffles and per field with
// a 64-bit atomic max on the FP64 bit pattern (the convergence residual).
#include "sweep.h"
#include "wavefront.cuh"

namespace eikx {

namespace {

constexpr int HY3 = LY3 + 1, HZ3 = LZ3 + 1;          // ring plane incl. halo row/column
constexpr int kPlane3 = HY3 * HZ3;
constexpr int kPlane2 = LZ2 + 1;
constexpr int kThreads = 32 * kWarpsPerBlock;

template <class T> __device__ __forceinline__ T hugeT() { return static_cast<T>(1.e10); }

// Zero the other progress buffer and queue head for the next sweep.  The launch
// boundary orders this before the next sweep reads them.
__device__ __forceinline__ void clearNext(const SolveState &st, int buf) {
    const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gthreads = gridDim.x * blockDim.x;
    unsigned *nxt = st.progress[buf ^ 1];
    for (int i = gtid; i < st.nProgress; i += gthreads) nxt[i] = 0u;
    if (gtid == 0) *st.queue[buf ^ 1] = 0u;
}

template <class T, bool UNIFORM>
__global__ void __launch_bounds__(kThreads) sweep3Kernel(const Sweep3Args<T> a) {
    extern __shared__ __align__(16) unsigned char smemRaw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ly = lane % LY3, lz = lane / LY3;
    T *tring = reinterpret_cast<T *>(smemRaw) + warp * (2 * kRing * kPlane3);
    T *sring = tring + kRing * kPlane3;
    const SolveState &st = a.st;
    clearNext(st, a.buf);
    if (ldVolatile(st.abortFlag)) return;

    const int fx = a.sweep & 1, fy = (a.sweep >> 1) & 1, fz = (a.sweep >> 2) & 1;
    SweepSigns sg;
    sg.ixShift = fx ? 1 : -1; sg.iyShift = fy ? 1 : -1; sg.izShift = fz ? 1 : -1;
    sg.signX = fx ? -1 : 1; sg.signY = fy ? -1 : 1; sg.signZ = fz ? -1 : 1;
    const int Px = a.pitch;
    const int nSteps = Px + LY3 + LZ3 - 2;
    const int spMaxX = a.spPitch - 1;
    const int sColOff = fx ? 0 : 1;   // own slowness column: the "offset" cell side
    const int tilesPerField = a.tilesY * a.tilesZ;
    unsigned *progress = st.progress[a.buf];
    const T huge = hugeT<T>();

    // helper lanes stand in for the virtual upwind lanes of the halo row/column
    const bool helper = lane < HZ3 + LY3;
    const int vly = lane < HZ3 ? -1 : lane - HZ3;
    const int vlz = lane < HZ3 ? lane - 1 : -1;
    const int vslot = (vlz + 1) * HY3 + (vly + 1);
    const int myslot = (lz + 1) * HY3 + (ly + 1);

    while (true) {
        unsigned q = 0;
        if (lane == 0) q = atomicAdd(st.queue[a.buf], 1u);
        q = __shfl_sync(kFull, q, 0);
        if (q >= static_cast<unsigned>(st.totalItems)) break;
        const int4 item = st.order[q];
        const int f = item.x, b = item.y, c = item.z;
        if (st.converged[f]) continue;
        const SourceT<T> src = a.srcs[f];
        const int y0 = b * LY3, z0 = c * LZ3;
        const int yp = y0 + ly, zp = z0 + lz;
        const bool laneValid = yp < a.ny && zp < a.nz;
        const int ya = laneValid ? reflect(yp, a.ny, fy) : 0;
        const int za = laneValid ? reflect(zp, a.nz, fz) : 0;
        int xlo, xhi, ylo, yhi, zlo, zhi;
        axisBounds(a.nx, fx, a.init, src.isx, xlo, xhi);
        axisBounds(a.ny, fy, a.init, src.isy, ylo, yhi);
        axisBounds(a.nz, fz, a.init, src.isz, zlo, zhi);
        const bool yzUpd = laneValid && ya >= ylo && ya <= yhi && za >= zlo && za <= zhi;
        T *field = a.tt + static_cast<long long>(f) * a.fieldStride;
        T *row = field + (static_cast<long long>(za) * a.ny + ya) * a.pitch;
        const T *srow = a.sp + static_cast<long long>(za + (fz ? 0 : 1)) * a.spPlane +
                        static_cast<long long>(ya + (fy ? 0 : 1)) * a.spPitch;
        // virtual lane rows
        const int vyp = y0 + vly, vzp = z0 + vlz;
        const bool vValid = helper && vyp >= 0 && vzp >= 0 && vyp < a.ny && vzp < a.nz;
        const int vya = vValid ? reflect(vyp, a.ny, fy) : 0;
        const int vza = vValid ? reflect(vzp, a.nz, fz) : 0;
        const T *vrow = field + (static_cast<long long>(vza) * a.ny + vya) * a.pitch;
        const T *vsrow = a.sp + static_cast<long long>(vza + (fz ? 0 : 1)) * a.spPlane +
                         static_cast<long long>(vya + (fy ? 0 : 1)) * a.spPitch;
        const unsigned *upY = b > 0 ? progress + f * tilesPerField + c * a.tilesY + (b - 1) : nullptr;
        const unsigned *upZ = c > 0 ? progress + f * tilesPerField + (c - 1) * a.tilesY + b : nullptr;
        unsigned *mine = progress + f * tilesPerField + c * a.tilesY + b;
        unsigned knownY = 0, knownZ = 0;
        bool ok = true;

        // Fill the halo entries of ring slot `sv` (values the virtual lanes produce at step sv).
        auto prefetch = [&](int sv) {
            bool good = true;
            if (lane == 0) {
                const int needY = max(0, min(sv + LY3 + 1, nSteps));
                const int needZ = max(0, min(sv + LZ3 + 1, nSteps));
                if (upY) good = waitAtLeast(upY, needY, knownY, st.abortFlag, st.spinLimit);
                if (good && upZ) good = waitAtLeast(upZ, needZ, knownZ, st.abortFlag, st.spinLimit);
            }
            good = __shfl_sync(kFull, good ? 1 : 0, 0) != 0;
            if (good && helper) {
                const int xv = sv - vly - vlz;
                T tv = huge, svv = huge;
                if (vValid && xv >= 0 && xv < Px) {
                    const int xa = reflect(xv, Px, fx);
                    tv = ldL2(vrow + xa);
                    svv = vsrow[min(xa + sColOff, spMaxX)];
                }
                const int slot = (sv & (kRing - 1)) * kPlane3 + vslot;
                tring[slot] = tv;
                sring[slot] = svv;
            }
            return good;
        };

        for (int sv = -2; sv < kPref && ok; ++sv) ok = prefetch(sv);
        T res = 0;
        for (int s = 0; s < nSteps && ok; ++s) {
            ok = prefetch(s + kPref);
            if (!ok) break;
            const int xp = s - ly - lz;
            const bool active = laneValid && xp >= 0 && xp < Px;
            const int xa = reflect(xp, Px, fx);
            T t0 = huge, sOwn = huge;
            if (active) {
                t0 = row[xa];
                sOwn = srow[min(xa + sColOff, spMaxX)];
            }
            const int cur = (s & (kRing - 1)) * kPlane3;
            const int p1 = ((s - 1) & (kRing - 1)) * kPlane3;
            const int p2 = ((s - 2) & (kRing - 1)) * kPlane3;
            const int p3 = ((s - 3) & (kRing - 1)) * kPlane3;
            sring[cur + myslot] = sOwn;
            __syncwarp();
            Stencil3<T> n;
            n.t1 = tring[p1 + myslot];
            n.t3 = tring[p1 + myslot - 1];
            n.t2 = tring[p2 + myslot - 1];
            n.t4 = tring[p1 + myslot - HY3];
            n.t5 = tring[p2 + myslot - HY3];
            n.t7 = tring[p2 + myslot - HY3 - 1];
            n.t6 = tring[p3 + myslot - HY3 - 1];
            n.s0 = sring[p3 + myslot - HY3 - 1];
            n.s1 = sring[p2 + myslot - HY3 - 1];
            n.s2 = sring[p1 + myslot - HY3];
            n.s3 = sring[p2 + myslot - HY3];
            n.s4 = sring[p2 + myslot - 1];
            n.s5 = sring[p1 + myslot - 1];
            n.s7 = sring[p1 + myslot];
            T v = t0;
            if (active && yzUpd && xa >= xlo && xa <= xhi) {
                const T tu = UNIFORM ? fd3Uniform<T>(a.radius, a.h, src, sg, xa, ya, za, n)
                                     : fd3NonUniform<T>(a.radius, a.sp3, src, sg, xa, ya, za, n);
                if (tu < t0) {
                    v = tu;
                    row[xa] = tu;
                    res = dmax(res, t0 - tu);
                }
            }
            tring[cur + myslot] = v;
            if (((s + 1) % kPub) == 0 || s == nSteps - 1) {
                fenceAcqRel();
                __syncwarp();
                if (lane == 0) stRelease(mine, static_cast<unsigned>(s + 1));
            }
        }
        if (!ok) break;
        const double r = warpMax(static_cast<double>(res));
        if (lane == 0 && r > 0)
            atomicMax(st.residual + static_cast<long long>(f) * st.residualStride + a.residualSlot,
                      static_cast<unsigned long long>(__double_as_longlong(r)));
    }
}

template <class T, bool UNIFORM>
__global__ void __launch_bounds__(kThreads) sweep2Kernel(const Sweep2Args<T> a) {
    extern __shared__ __align__(16) unsigned char smemRaw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int lz = lane;
    T *tring = reinterpret_cast<T *>(smemRaw) + warp * (2 * kRing * kPlane2);
    T *sring = tring + kRing * kPlane2;
    const SolveState &st = a.st;
    clearNext(st, a.buf);
    if (ldVolatile(st.abortFlag)) return;

    const int fx = a.sweep & 1, fz = (a.sweep >> 1) & 1;
    SweepSigns sg;
    sg.ixShift = fx ? 1 : -1; sg.iyShift = 0; sg.izShift = fz ? 1 : -1;
    sg.signX = fx ? -1 : 1; sg.signY = 1; sg.signZ = fz ? -1 : 1;
    const int Px = a.pitch;
    const int nSteps = Px + LZ2 - 1;
    const int spMaxX = a.spPitch - 1;
    const int sColOff = fx ? 0 : 1;
    unsigned *progress = st.progress[a.buf];
    const T huge = hugeT<T>();
    const int myslot = lz + 1;

    while (true) {
        unsigned q = 0;
        if (lane == 0) q = atomicAdd(st.queue[a.buf], 1u);
        q = __shfl_sync(kFull, q, 0);
        if (q >= static_cast<unsigned>(st.totalItems)) break;
        const int4 item = st.order[q];
        const int f = item.x, c = item.z;
        if (st.converged[f]) continue;
        const SourceT<T> src = a.srcs[f];
        const int z0 = c * LZ2;
        const int zp = z0 + lz;
        const bool laneValid = zp < a.nz;
        const int za = laneValid ? reflect(zp, a.nz, fz) : 0;
        int xlo, xhi, zlo, zhi;
        axisBounds(a.nx, fx, a.init, src.isx, xlo, xhi);
        axisBounds(a.nz, fz, a.init, src.isz, zlo, zhi);
        const bool zUpd = laneValid && za >= zlo && za <= zhi;
        T *field = a.tt + static_cast<long long>(f) * a.fieldStride;
        T *row = field + static_cast<long long>(za) * a.pitch;
        const T *srow = a.sp + static_cast<long long>(za + (fz ? 0 : 1)) * a.spPitch;
        // lane 0 also stands in for the virtual lane z' = z0 - 1
        const bool vValid = (lane == 0) && c > 0;
        const int vza = vValid ? reflect(z0 - 1, a.nz, fz) : 0;
        const T *vrow = field + static_cast<long long>(vza) * a.pitch;
        const T *vsrow = a.sp + static_cast<long long>(vza + (fz ? 0 : 1)) * a.spPitch;
        const unsigned *up = c > 0 ? progress + f * a.tilesZ + (c - 1) : nullptr;
        unsigned *mine = progress + f * a.tilesZ + c;
        unsigned known = 0;
        bool ok = true;

        auto prefetch = [&](int sv) {
            bool good = true;
            if (lane == 0 && up) {
                const int need = max(0, min(sv + LZ2 + 1, nSteps));
                good = waitAtLeast(up, need, known, st.abortFlag, st.spinLimit);
            }
            good = __shfl_sync(kFull, good ? 1 : 0, 0) != 0;
            if (good && lane == 0) {
                const int xv = sv + 1;
                T tv = huge, svv = huge;
                if (vValid && xv >= 0 && xv < Px) {
                    const int xa = reflect(xv, Px, fx);
                    tv = ldL2(vrow + xa);
                    svv = vsrow[min(xa + sColOff, spMaxX)];
                }
                const int slot = (sv & (kRing - 1)) * kPlane2;
                tring[slot] = tv;
                sring[slot] = svv;
            }
            return good;
        };

        for (int sv = -1; sv < kPref && ok; ++sv) ok = prefetch(sv);
        T res = 0;
        for (int s = 0; s < nSteps && ok; ++s) {
            ok = prefetch(s + kPref);
            if (!ok) break;
            const int xp = s - lz;
            const bool active = laneValid && xp >= 0 && xp < Px;
            const int xa = reflect(xp, Px, fx);
            T t0 = huge, sOwn = huge;
            if (active) {
                t0 = row[xa];
                sOwn = srow[min(xa + sColOff, spMaxX)];
            }
            const int cur = (s & (kRing - 1)) * kPlane2;
            const int p1 = ((s - 1) & (kRing - 1)) * kPlane2;
            const int p2 = ((s - 2) & (kRing - 1)) * kPlane2;
            sring[cur + myslot] = sOwn;
            __syncwarp();
            const T t1 = tring[p1 + myslot];
            const T t3 = tring[p1 + myslot - 1];
            const T t2 = tring[p2 + myslot - 1];
            const T s0 = sring[p2 + myslot - 1];
            const T s1 = sring[p1 + myslot - 1];
            const T s3 = sring[p1 + myslot];
            T v = t0;
            if (active && zUpd && xa >= xlo && xa <= xhi) {
                const T tu = UNIFORM ? fd2Uniform<T>(a.radius, a.h, src, sg, xa, za, s0, s1, s3, t1, t2, t3)
                                     : fd2NonUniform<T>(a.radius, a.sp2, src, sg, xa, za, s0, s1, s3, t1, t2, t3);
                if (tu < t0) {
                    v = tu;
                    row[xa] = tu;
                    res = dmax(res, t0 - tu);
                }
            }
            tring[cur + myslot] = v;
            if (((s + 1) % kPub) == 0 || s == nSteps - 1) {
                fenceAcqRel();
                __syncwarp();
                if (lane == 0) stRelease(mine, static_cast<unsigned>(s + 1));
            }
        }
        if (!ok) break;
        const double r = warpMax(static_cast<double>(res));
        if (lane == 0 && r > 0)
            atomicMax(st.residual + static_cast<long long>(f) * st.residualStride + a.residualSlot,
                      static_cast<unsigned long long>(__double_as_longlong(r)));
    }
}

}  // namespace

size_t sweep3SmemBytes(size_t elem) { return elem * 2 * kRing * kPlane3 * kWarpsPerBlock; }
size_t sweep2SmemBytes(size_t elem) { return elem * 2 * kRing * kPlane2 * kWarpsPerBlock; }

template <class T>
cudaError_t launchSweep3(const Sweep3Args<T> &a, bool uniform, int blocks, cudaStream_t s) {
    const size_t smem = sweep3SmemBytes(sizeof(T));
    if (uniform) sweep3Kernel<T, true><<<blocks, kThreads, smem, s>>>(a);
    else sweep3Kernel<T, false><<<blocks, kThreads, smem, s>>>(a);
    return cudaGetLastError();
}

template <class T>
cudaError_t launchSweep2(const Sweep2Args<T> &a, bool uniform, int blocks, cudaStream_t s) {
    const size_t smem = sweep2SmemBytes(sizeof(T));
    if (uniform) sweep2Kernel<T, true><<<blocks, kThreads, smem, s>>>(a);
    else sweep2Kernel<T, false><<<blocks, kThreads, smem, s>>>(a);
    return cudaGetLastError();
}

template <class T> int sweep3BlocksPerSM(bool uniform) {
    int n = 0;
    const size_t smem = sweep3SmemBytes(sizeof(T));
    if (uniform) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep3Kernel<T, true>, kThreads, smem);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep3Kernel<T, false>, kThreads, smem);
    return n > 0 ? n : 1;
}
template <class T> int sweep2BlocksPerSM(bool uniform) {
    int n = 0;
    const size_t smem = sweep2SmemBytes(sizeof(T));
    if (uniform) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep2Kernel<T, true>, kThreads, smem);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep2Kernel<T, false>, kThreads, smem);
    return n > 0 ? n : 1;
}

template cudaError_t launchSweep3<float>(const Sweep3Args<float> &, bool, int, cudaStream_t);
template cudaError_t launchSweep3<double>(const Sweep3Args<double> &, bool, int, cudaStream_t);
template cudaError_t launchSweep2<float>(const Sweep2Args<float> &, bool, int, cudaStream_t);
template cudaError_t launchSweep2<double>(const Sweep2Args<double> &, bool, int, cudaStream_t);
template int sweep3BlocksPerSM<float>(bool);
template int sweep3BlocksPerSM<double>(bool);
template int sweep2BlocksPerSM<float>(bool);
template int sweep2BlocksPerSM<double>(bool);

}  // namespace eikx
