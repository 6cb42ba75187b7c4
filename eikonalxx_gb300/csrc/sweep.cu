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

// Zero the queue head the next sweep uses; the launch boundary orders it before use.
__device__ __forceinline__ void clearNext(const SolveState &st, int buf) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *st.queue[buf ^ 1] = 0u;
}

// Own-row stream: the travel times and slowness of one lane's x'-pencil, consumed one
// element per step in walk order, fetched in 16-byte chunks one chunk ahead.
//   T row     forward (+x sweep): chunk k at row + k*V;   reverse: row + Px - (k+1)*V
//   slowness  forward: shifted copy, chunk k at srow + (k+1)*V; reverse: srow + Px - (k+1)*V
template <class T> struct RowStream {
    static constexpr int V = Chunk<T>::kN;
    Chunk<T> tCur, tNxt, sCur, sNxt;
    const T *row, *srow;
    int Px, rev, nChunks;
    __device__ __forceinline__ const T *tAddr(int k) const { return rev ? row + Px - (k + 1) * V : row + k * V; }
    __device__ __forceinline__ const T *sAddr(int k) const { return rev ? srow + Px - (k + 1) * V : srow + (k + 1) * V; }
    __device__ __forceinline__ void start() {
        tCur.load(tAddr(0));
        sCur.load(sAddr(0));
        if (nChunks > 1) {
            tNxt.load(tAddr(1));
            sNxt.load(sAddr(1));
        }
    }
    // values of walk position xp (called for xp = 0, 1, 2, ... in order)
    __device__ __forceinline__ void take(int xp, T &t, T &s) {
        const int e = xp & (V - 1);
        if (e == 0 && xp > 0) {
            tCur = tNxt;
            sCur = sNxt;
            const int k = (xp / V) + 1;
            if (k < nChunks) {
                tNxt.load(tAddr(k));
                sNxt.load(sAddr(k));
            }
        }
        const int i = rev ? V - 1 - e : e;
        t = tCur.at(i);
        s = sCur.at(i);
    }
};

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
    constexpr int W = Mail<T>::kWords;
    const unsigned tag = *st.epoch + static_cast<unsigned>(a.sweepIndex);

    const int fx = a.sweep & 1, fy = (a.sweep >> 1) & 1, fz = (a.sweep >> 2) & 1;
    SweepSigns sg;
    sg.ixShift = fx ? 1 : -1; sg.iyShift = fy ? 1 : -1; sg.izShift = fz ? 1 : -1;
    sg.signX = fx ? -1 : 1; sg.signY = fy ? -1 : 1; sg.signZ = fz ? -1 : 1;
    const int Px = a.pitch;
    const int nSteps = Px + LY3 + LZ3 - 2;
    const T *sp = fx ? a.spNeg : a.spPos;
    const T huge = hugeT<T>();
    const long long faceWords = static_cast<long long>(LY3 + LZ3) * Px * W;

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
        RowStream<T> rs;
        rs.row = row;
        rs.srow = sp + static_cast<long long>(za + (fz ? 0 : 1)) * a.spPlane +
                  static_cast<long long>(ya + (fy ? 0 : 1)) * a.spPitch;
        rs.Px = Px;
        rs.rev = fx;
        rs.nChunks = Px / RowStream<T>::V;
        if (laneValid) rs.start();

        // mailbox: this block's faces, and the upstream face row a helper lane reads
        const long long tileId = (static_cast<long long>(f) * a.tilesZ + c) * a.tilesY + b;
        unsigned long long *box = st.mbox + tileId * faceWords;
        unsigned long long *yFace = box + static_cast<long long>(lz) * Px * W;          // ly == LY-1
        unsigned long long *zFace = box + static_cast<long long>(LZ3 + ly) * Px * W;    // lz == LZ-1
        const int vyp = y0 + vly, vzp = z0 + vlz;
        const bool vValid = helper && vyp >= 0 && vzp >= 0 && vyp < a.ny && vzp < a.nz;
        const unsigned long long *vbox = st.mbox;
        const T *vsrow = sp;
        if (vValid) {
            const int vya = reflect(vyp, a.ny, fy), vza = reflect(vzp, a.nz, fz);
            if (vly < 0) {
                const long long up = vlz >= 0 ? tileId - 1 : tileId - a.tilesY - 1;
                vbox = st.mbox + up * faceWords + static_cast<long long>(vlz >= 0 ? vlz : LZ3 - 1) * Px * W;
            } else {
                vbox = st.mbox + (tileId - a.tilesY) * faceWords + static_cast<long long>(LZ3 + vly) * Px * W;
            }
            vsrow = sp + static_cast<long long>(vza + (fz ? 0 : 1)) * a.spPlane +
                    static_cast<long long>(vya + (fy ? 0 : 1)) * a.spPitch;
        }

        // Halo pipeline.  The values the virtual lanes produce at step sv go into ring slot
        // sv; the reads for step sv are issued at step sv - kPref into register slot
        // sv % kPref and checked (and stored into the ring) at step sv.
        auto haloT = [&](int sv) { return sv - vly - vlz; };
        auto haloValid = [&](int xv) { return vValid && xv >= 0 && xv < Px; };
        auto haloStore = [&](int sv, T tv, T svv) {
            const int slot = (sv & (kRing - 1)) * kPlane3 + vslot;
            tring[slot] = tv;
            sring[slot] = svv;
        };
        auto fillNow = [&](int sv) -> bool {
            bool good = true;
            if (helper) {
                const int xv = haloT(sv);
                T tv = huge, svv = huge;
                if (haloValid(xv)) {
                    good = Mail<T>::get(vbox + static_cast<long long>(xv) * W, tag, tv, st.abortFlag, st.spinLimit);
                    svv = vsrow[fx ? Px - 1 - xv : xv + RowStream<T>::V];
                }
                haloStore(sv, tv, svv);
            }
            return __all_sync(kFull, good);
        };
        MailSlot<T> mslot[kPref];
        T sslot[kPref];
        auto issue = [&](int j, int sv) {
            const int xv = haloT(sv);
            if (helper && haloValid(xv)) {
                mslot[j].issue(vbox + static_cast<long long>(xv) * W);
                sslot[j] = vsrow[fx ? Px - 1 - xv : xv + RowStream<T>::V];
            }
        };
        auto consume = [&](int j, int sv) -> bool {
            bool good = true;
            if (helper) {
                const int xv = haloT(sv);
                T tv = huge, svv = huge;
                if (haloValid(xv)) {
                    good = mslot[j].take(vbox + static_cast<long long>(xv) * W, tag, tv, st.abortFlag, st.spinLimit);
                    svv = sslot[j];
                }
                haloStore(sv, tv, svv);
            }
            return __all_sync(kFull, good);
        };

        bool ok = fillNow(-2) && fillNow(-1);
#pragma unroll
        for (int j = 0; j < kPref; ++j) issue(j, j);
        T res = 0;
        for (int s0 = 0; s0 < nSteps && ok; s0 += kPref) {
#pragma unroll
            for (int j = 0; j < kPref; ++j) {
                const int s = s0 + j;
                if (!ok || s >= nSteps) continue;
                ok = consume(j, s);
                if (!ok) continue;
                issue(j, s + kPref);
                const int xp = s - ly - lz;
                const bool active = laneValid && xp >= 0 && xp < Px;
                const int xa = reflect(xp, Px, fx);
                T t0 = huge, sOwn = huge;
                if (active) rs.take(xp, t0, sOwn);
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
                if (active) {
                    if (ly == LY3 - 1) Mail<T>::put(yFace + static_cast<long long>(xp) * W, tag, v);
                    if (lz == LZ3 - 1) Mail<T>::put(zFace + static_cast<long long>(xp) * W, tag, v);
                }
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
    constexpr int W = Mail<T>::kWords;
    const unsigned tag = *st.epoch + static_cast<unsigned>(a.sweepIndex);

    const int fx = a.sweep & 1, fz = (a.sweep >> 1) & 1;
    SweepSigns sg;
    sg.ixShift = fx ? 1 : -1; sg.iyShift = 0; sg.izShift = fz ? 1 : -1;
    sg.signX = fx ? -1 : 1; sg.signY = 1; sg.signZ = fz ? -1 : 1;
    const int Px = a.pitch;
    const int nSteps = Px + LZ2 - 1;
    const T *sp = fx ? a.spNeg : a.spPos;
    const T huge = hugeT<T>();
    const int myslot = lz + 1;
    const long long faceWords = static_cast<long long>(Px) * W;

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
        RowStream<T> rs;
        rs.row = row;
        rs.srow = sp + static_cast<long long>(za + (fz ? 0 : 1)) * a.spPitch;
        rs.Px = Px;
        rs.rev = fx;
        rs.nChunks = Px / RowStream<T>::V;
        if (laneValid) rs.start();
        const long long tileId = static_cast<long long>(f) * a.tilesZ + c;
        unsigned long long *face = st.mbox + tileId * faceWords;   // written by lane LZ2-1
        // lane 0 also stands in for the virtual lane z' = z0 - 1 (row LZ2-1 of block c-1)
        const bool vValid = (lane == 0) && c > 0;
        const unsigned long long *vbox = st.mbox + (tileId - (c > 0 ? 1 : 0)) * faceWords;
        const int vza = vValid ? reflect(z0 - 1, a.nz, fz) : 0;
        const T *vsrow = sp + static_cast<long long>(vza + (fz ? 0 : 1)) * a.spPitch;

        // Halo pipeline as in the 3D kernel: lane 0 stands in for the virtual lane, whose
        // value at step sv is node x' = sv + 1 of the upstream block's last row.
        auto haloValid = [&](int xv) { return vValid && xv >= 0 && xv < Px; };
        auto haloStore = [&](int sv, T tv, T svv) {
            const int slot = (sv & (kRing - 1)) * kPlane2;
            tring[slot] = tv;
            sring[slot] = svv;
        };
        auto fillNow = [&](int sv) -> bool {
            bool good = true;
            if (lane == 0) {
                const int xv = sv + 1;
                T tv = huge, svv = huge;
                if (haloValid(xv)) {
                    good = Mail<T>::get(vbox + static_cast<long long>(xv) * W, tag, tv, st.abortFlag, st.spinLimit);
                    svv = vsrow[fx ? Px - 1 - xv : xv + RowStream<T>::V];
                }
                haloStore(sv, tv, svv);
            }
            return __all_sync(kFull, good);
        };
        MailSlot<T> mslot[kPref];
        T sslot[kPref];
        auto issue = [&](int j, int sv) {
            const int xv = sv + 1;
            if (lane == 0 && haloValid(xv)) {
                mslot[j].issue(vbox + static_cast<long long>(xv) * W);
                sslot[j] = vsrow[fx ? Px - 1 - xv : xv + RowStream<T>::V];
            }
        };
        auto consume = [&](int j, int sv) -> bool {
            bool good = true;
            if (lane == 0) {
                const int xv = sv + 1;
                T tv = huge, svv = huge;
                if (haloValid(xv)) {
                    good = mslot[j].take(vbox + static_cast<long long>(xv) * W, tag, tv, st.abortFlag, st.spinLimit);
                    svv = sslot[j];
                }
                haloStore(sv, tv, svv);
            }
            return __all_sync(kFull, good);
        };

        bool ok = fillNow(-1);
#pragma unroll
        for (int j = 0; j < kPref; ++j) issue(j, j);
        T res = 0;
        for (int s0 = 0; s0 < nSteps && ok; s0 += kPref) {
#pragma unroll
            for (int j = 0; j < kPref; ++j) {
                const int s = s0 + j;
                if (!ok || s >= nSteps) continue;
                ok = consume(j, s);
                if (!ok) continue;
                issue(j, s + kPref);
                const int xp = s - lz;
                const bool active = laneValid && xp >= 0 && xp < Px;
                const int xa = reflect(xp, Px, fx);
                T t0 = huge, sOwn = huge;
                if (active) rs.take(xp, t0, sOwn);
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
                if (active && lz == LZ2 - 1) Mail<T>::put(face + static_cast<long long>(xp) * W, tag, v);
            }
        }
        if (!ok) break;
        const double r = warpMax(static_cast<double>(res));
        if (lane == 0 && r > 0)
            atomicMax(st.residual + static_cast<long long>(f) * st.residualStride + a.residualSlot,
                      static_cast<unsigned long long>(__double_as_longlong(r)));
    }
}

// One CTA per field for 2D grids of up to 512 rows (sweep2BlockKernel): thread z' owns
// row z' and updates x' = s - z' at step s; the only upwind value from another thread is
// the row above's result of the step before, passed through shared memory with one
// __syncthreads() per step.  No mailbox, no inter-CTA waits: fields are independent
// CTAs, and a single field's sweep is a chain of barrier-separated steps instead of
// L2 round trips between warp blocks.
template <class T, bool UNIFORM>
__global__ void __launch_bounds__(512) sweep2BlockKernel(const Sweep2Args<T> a) {
    extern __shared__ __align__(16) unsigned char smemRaw[];
    const int nzp = blockDim.x;                         // rows rounded up to a warp multiple
    T *tUp = reinterpret_cast<T *>(smemRaw);            // [2][nzp + 1]: value of row z'-1 at step s-1
    T *sUp = tUp + 2 * (nzp + 1);                       // [2][nzp + 1]: its cell slowness
    const SolveState &st = a.st;
    const int f = blockIdx.x;
    if (st.converged[f]) return;
    const int lz = threadIdx.x;
    const int fx = a.sweep & 1, fz = (a.sweep >> 1) & 1;
    SweepSigns sg;
    sg.ixShift = fx ? 1 : -1; sg.iyShift = 0; sg.izShift = fz ? 1 : -1;
    sg.signX = fx ? -1 : 1; sg.signY = 1; sg.signZ = fz ? -1 : 1;
    const int Px = a.pitch;
    const int nSteps = Px + a.nz - 1;
    const T *sp = fx ? a.spNeg : a.spPos;
    const T huge = hugeT<T>();
    const SourceT<T> src = a.srcs[f];
    const bool laneValid = lz < a.nz;
    const int za = laneValid ? reflect(lz, a.nz, fz) : 0;
    int xlo, xhi, zlo, zhi;
    axisBounds(a.nx, fx, a.init, src.isx, xlo, xhi);
    axisBounds(a.nz, fz, a.init, src.isz, zlo, zhi);
    const bool zUpd = laneValid && za >= zlo && za <= zhi;
    T *row = a.tt + static_cast<long long>(f) * a.fieldStride + static_cast<long long>(za) * a.pitch;
    RowStream<T> rs;
    rs.row = row;
    rs.srow = sp + static_cast<long long>(za + (fz ? 0 : 1)) * a.spPitch;
    rs.Px = Px;
    rs.rev = fx;
    rs.nChunks = Px / RowStream<T>::V;
    if (laneValid) rs.start();
    // both buffers start as "nothing upwind": slot 0 is the virtual row above row 0 and
    // stays HUGE; the other slots hold HUGE until their row publishes (inactive rows
    // publish HUGE too, as the lanes of the warp-block kernel do)
    for (int i = lz; i < 2 * (nzp + 1); i += nzp) {
        tUp[i] = huge;
        sUp[i] = huge;
    }
    T t1 = huge, t2 = huge, s3 = huge, s0 = huge;      // own previous value / slowness, carries
    T res = 0;
    __syncthreads();
    for (int s = 0; s < nSteps; ++s) {
        const int cur = (s & 1) * (nzp + 1), prv = ((s - 1) & 1) * (nzp + 1);
        const int xp = s - lz;
        const bool active = laneValid && xp >= 0 && xp < Px;
        T t0 = huge, sOwn = huge;
        if (active) rs.take(xp, t0, sOwn);
        const T t3 = tUp[prv + lz];                     // row above, same x', previous step
        const T s1 = sUp[prv + lz];
        T v = t0;
        if (active) {
            const int xa = reflect(xp, Px, fx);
            if (zUpd && xa >= xlo && xa <= xhi) {
                const T tu = UNIFORM ? fd2Uniform<T>(a.radius, a.h, src, sg, xa, za, s0, s1, s3, t1, t2, t3)
                                     : fd2NonUniform<T>(a.radius, a.sp2, src, sg, xa, za, s0, s1, s3, t1, t2, t3);
                if (tu < t0) {
                    v = tu;
                    row[xa] = tu;
                    res = dmax(res, t0 - tu);
                }
            }
        }
        // publish for row z'+1 (slot lz + 1 of the current buffer)
        tUp[cur + lz + 1] = v;
        sUp[cur + lz + 1] = sOwn;
        // carries: t2 = row above at x'-1, s0 = its cell; t1 / s3 = own x'-1
        t2 = t3;
        s0 = s1;
        t1 = v;
        s3 = sOwn;
        __syncthreads();
    }
    double r = warpMax(static_cast<double>(res));
    __shared__ double blockMax[32];
    if ((lz & 31) == 0) blockMax[lz >> 5] = r;
    __syncthreads();
    if (lz < 32) {
        r = lz < (nzp >> 5) ? blockMax[lz] : 0.0;
        r = warpMax(r);
        if (lz == 0 && r > 0)
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

template <class T>
cudaError_t launchSweep2Block(const Sweep2Args<T> &a, bool uniform, int nFields, cudaStream_t s) {
    const int nzp = (a.nz + 31) / 32 * 32;
    const size_t smem = 4 * (nzp + 1) * sizeof(T);
    if (uniform) sweep2BlockKernel<T, true><<<nFields, nzp, smem, s>>>(a);
    else sweep2BlockKernel<T, false><<<nFields, nzp, smem, s>>>(a);
    return cudaGetLastError();
}
template cudaError_t launchSweep2Block<float>(const Sweep2Args<float> &, bool, int, cudaStream_t);
template cudaError_t launchSweep2Block<double>(const Sweep2Args<double> &, bool, int, cudaStream_t);

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
