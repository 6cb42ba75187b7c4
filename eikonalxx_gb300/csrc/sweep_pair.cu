// Paired level-set sweep kernel: two fields (two sources on one model) per lane.
//
// Same wavefront as sweep3Kernel (sweep.cu / wavefront.cuh) -- 8x4 x'-pencils per warp,
// one level per step, halo faces through tagged mailbox words -- but every lane updates
// the same node of two fields.  What depends only on the node and the model is done once
// for both: the slowness stream and ring, the slowness-only terms of the local solver,
// ring addressing, the warp synchronisation and the halo bookkeeping.  Travel times
// travel as pairs (64-bit shared-memory words, two tagged 64-bit mailbox words per node)
// and their arithmetic runs on the packed FP32 pipe (pair_solver.cuh).  Each field's
// result is bit-identical to the single-field kernel's.
#include "pair_solver.cuh"
#include "sweep.h"
#include "wavefront.cuh"

namespace eikx {

namespace {

constexpr int HY = LY3 + 1, HZ = LZ3 + 1;
constexpr int kPlane = HY * HZ;
constexpr int kThreads = 32 * kWarpsPerBlock;
constexpr int V = 4;   // floats per 16-byte chunk

// Mailbox slot of a node: two tagged words (field 0, field 1).
__device__ __forceinline__ void putPair(unsigned long long *w, unsigned tag, F2 v) {
    const unsigned long long t = static_cast<unsigned long long>(tag) << 32;
    const unsigned long long a = t | __float_as_uint(lo(v)), b = t | __float_as_uint(hi(v));
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(w), "l"(a), "l"(b));
}
__device__ __forceinline__ void loadPair(const unsigned long long *w, unsigned long long &a, unsigned long long &b) {
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(w));
}
// Value of a pair slot loaded earlier, re-read (bounded spin) until both words carry `tag`.
__device__ __forceinline__ bool takePair(const unsigned long long *w, unsigned tag, unsigned long long a,
                                         unsigned long long b, F2 &v, int *abortFlag,
                                         unsigned long long spinLimit) {
    unsigned long long it = 0;
    while (static_cast<unsigned>(a >> 32) != tag || static_cast<unsigned>(b >> 32) != tag) {
        if ((++it & 31ull) == 0) {
            if (ldVolatile(abortFlag)) return false;
            if (it > spinLimit) {
                atomicExch(abortFlag, 1);
                return false;
            }
        }
        __nanosleep(32);
        loadPair(w, a, b);
    }
    v = f2(__uint_as_float(static_cast<unsigned>(a)), __uint_as_float(static_cast<unsigned>(b)));
    return true;
}

__global__ void __launch_bounds__(kThreads, 3) sweep3PairKernel(const Sweep3Args<float> a) {
    extern __shared__ __align__(16) unsigned char smemRaw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ly = lane % LY3, lz = lane / LY3;
    F2 *tring = reinterpret_cast<F2 *>(smemRaw) + warp * (kRing * kPlane);
    float *sring = reinterpret_cast<float *>(smemRaw + sizeof(F2) * kWarpsPerBlock * kRing * kPlane) +
                   warp * (kRing * kPlane);
    const SolveState &st = a.st;
    if (blockIdx.x == 0 && threadIdx.x == 0) *st.queue[a.buf ^ 1] = 0u;
    if (ldVolatile(st.abortFlag)) return;
    const unsigned tag = *st.epoch + static_cast<unsigned>(a.sweepIndex);

    const int fx = a.sweep & 1, fy = (a.sweep >> 1) & 1, fz = (a.sweep >> 2) & 1;
    SweepSigns sg;
    sg.ixShift = fx ? 1 : -1; sg.iyShift = fy ? 1 : -1; sg.izShift = fz ? 1 : -1;
    sg.signX = fx ? -1 : 1; sg.signY = fy ? -1 : 1; sg.signZ = fz ? -1 : 1;
    const int Px = a.pitch;
    const int nChunks = Px / V;
    const int nSteps = Px + LY3 + LZ3 - 2;
    const float *sp = fx ? a.spNeg : a.spPos;
    const float huge = 1.e10f;
    const long long faceWords = static_cast<long long>(LY3 + LZ3) * Px * 2;

    const bool helper = lane < HZ + LY3;
    const int vly = lane < HZ ? -1 : lane - HZ;
    const int vlz = lane < HZ ? lane - 1 : -1;
    const int vslot = (vlz + 1) * HY + (vly + 1);
    const int myslot = (lz + 1) * HY + (ly + 1);

    while (true) {
        unsigned q = 0;
        if (lane == 0) q = atomicAdd(st.queue[a.buf], 1u);
        q = __shfl_sync(kFull, q, 0);
        if (q >= static_cast<unsigned>(st.totalItems)) break;
        const int4 item = st.order[q];
        const int p = item.x, b = item.y, c = item.z;
        const int2 fp = a.pairs[p];
        const int f0 = fp.x, f1 = fp.y;
        const bool conv0 = st.converged[f0] != 0, conv1 = st.converged[f1] != 0;
        if (conv0 && conv1) continue;
        const SourceT<float> src0 = a.srcs[f0], src1 = a.srcs[f1];
        const int y0 = b * LY3, z0 = c * LZ3;
        const int yp = y0 + ly, zp = z0 + lz;
        const bool laneValid = yp < a.ny && zp < a.nz;
        const int ya = laneValid ? reflect(yp, a.ny, fy) : 0;
        const int za = laneValid ? reflect(zp, a.nz, fz) : 0;
        // update ranges of the two fields (they differ only in the initialisation pass)
        int xlo0, xhi0, ylo0, yhi0, zlo0, zhi0, xlo1, xhi1, ylo1, yhi1, zlo1, zhi1;
        axisBounds(a.nx, fx, a.init, src0.isx, xlo0, xhi0);
        axisBounds(a.ny, fy, a.init, src0.isy, ylo0, yhi0);
        axisBounds(a.nz, fz, a.init, src0.isz, zlo0, zhi0);
        axisBounds(a.nx, fx, a.init, src1.isx, xlo1, xhi1);
        axisBounds(a.ny, fy, a.init, src1.isy, ylo1, yhi1);
        axisBounds(a.nz, fz, a.init, src1.isz, zlo1, zhi1);
        const bool yz0 = !conv0 && laneValid && ya >= ylo0 && ya <= yhi0 && za >= zlo0 && za <= zhi0;
        const bool yz1 = !conv1 && laneValid && ya >= ylo1 && ya <= yhi1 && za >= zlo1 && za <= zhi1;
        const long long rowOff = (static_cast<long long>(za) * a.ny + ya) * a.pitch;
        float *row0 = a.tt + static_cast<long long>(f0) * a.fieldStride + rowOff;
        float *row1 = a.tt + static_cast<long long>(f1) * a.fieldStride + rowOff;
        const float *srow = sp + static_cast<long long>(za + (fz ? 0 : 1)) * a.spPlane +
                            static_cast<long long>(ya + (fy ? 0 : 1)) * a.spPitch;
        auto tAddr = [&](const float *r, int k) { return fx ? r + Px - (k + 1) * V : r + k * V; };
        auto sAddr = [&](int k) { return fx ? srow + Px - (k + 1) * V : srow + (k + 1) * V; };
        Chunk<float> c0, n0, c1, n1, cs, ns;
        if (laneValid) {
            c0.load(tAddr(row0, 0)); c1.load(tAddr(row1, 0)); cs.load(sAddr(0));
            if (nChunks > 1) { n0.load(tAddr(row0, 1)); n1.load(tAddr(row1, 1)); ns.load(sAddr(1)); }
        }

        const long long tileId = (static_cast<long long>(p) * a.tilesZ + c) * a.tilesY + b;
        unsigned long long *box = st.mbox + tileId * faceWords;
        unsigned long long *yFace = box + static_cast<long long>(lz) * Px * 2;
        unsigned long long *zFace = box + static_cast<long long>(LZ3 + ly) * Px * 2;
        const int vyp = y0 + vly, vzp = z0 + vlz;
        const bool vValid = helper && vyp >= 0 && vzp >= 0 && vyp < a.ny && vzp < a.nz;
        const unsigned long long *vbox = st.mbox;
        const float *vsrow = sp;
        if (vValid) {
            const int vya = reflect(vyp, a.ny, fy), vza = reflect(vzp, a.nz, fz);
            if (vly < 0) {
                const long long up = vlz >= 0 ? tileId - 1 : tileId - a.tilesY - 1;
                vbox = st.mbox + up * faceWords + static_cast<long long>(vlz >= 0 ? vlz : LZ3 - 1) * Px * 2;
            } else {
                vbox = st.mbox + (tileId - a.tilesY) * faceWords + static_cast<long long>(LZ3 + vly) * Px * 2;
            }
            vsrow = sp + static_cast<long long>(vza + (fz ? 0 : 1)) * a.spPlane +
                    static_cast<long long>(vya + (fy ? 0 : 1)) * a.spPitch;
        }
        auto haloValid = [&](int xv) { return vValid && xv >= 0 && xv < Px; };
        auto haloStore = [&](int sv, F2 tv, float svv) {
            const int slot = (sv & (kRing - 1)) * kPlane + vslot;
            tring[slot] = tv;
            sring[slot] = svv;
        };
        auto fillNow = [&](int sv) -> bool {
            bool good = true;
            if (helper) {
                const int xv = sv - vly - vlz;
                F2 tv = f2(huge);
                float svv = huge;
                if (haloValid(xv)) {
                    unsigned long long wa, wb;
                    loadPair(vbox + static_cast<long long>(xv) * 2, wa, wb);
                    good = takePair(vbox + static_cast<long long>(xv) * 2, tag, wa, wb, tv, st.abortFlag, st.spinLimit);
                    svv = vsrow[fx ? Px - 1 - xv : xv + V];
                }
                haloStore(sv, tv, svv);
            }
            return __all_sync(kFull, good);
        };
        unsigned long long wA[kPref], wB[kPref];
        float hs[kPref];
        auto issue = [&](int j, int sv) {
            const int xv = sv - vly - vlz;
            if (helper && haloValid(xv)) {
                loadPair(vbox + static_cast<long long>(xv) * 2, wA[j], wB[j]);
                hs[j] = vsrow[fx ? Px - 1 - xv : xv + V];
            }
        };
        auto consume = [&](int j, int sv) -> bool {
            bool good = true;
            if (helper) {
                const int xv = sv - vly - vlz;
                F2 tv = f2(huge);
                float svv = huge;
                if (haloValid(xv)) {
                    good = takePair(vbox + static_cast<long long>(xv) * 2, tag, wA[j], wB[j], tv, st.abortFlag,
                                    st.spinLimit);
                    svv = hs[j];
                }
                haloStore(sv, tv, svv);
            }
            return __all_sync(kFull, good);
        };

        bool ok = fillNow(-2) && fillNow(-1);
#pragma unroll
        for (int j = 0; j < kPref; ++j) issue(j, j);
        float res0 = 0, res1 = 0;
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
                float t0a = huge, t0b = huge, sOwn = huge;
                if (active) {
                    const int e = xp & (V - 1);
                    if (e == 0 && xp > 0) {
                        c0 = n0; c1 = n1; cs = ns;
                        const int k = xp / V + 1;
                        if (k < nChunks) { n0.load(tAddr(row0, k)); n1.load(tAddr(row1, k)); ns.load(sAddr(k)); }
                    }
                    const int i = fx ? V - 1 - e : e;
                    t0a = c0.at(i); t0b = c1.at(i); sOwn = cs.at(i);
                }
                const int cur = (s & (kRing - 1)) * kPlane;
                const int p1 = ((s - 1) & (kRing - 1)) * kPlane;
                const int p2 = ((s - 2) & (kRing - 1)) * kPlane;
                const int p3 = ((s - 3) & (kRing - 1)) * kPlane;
                sring[cur + myslot] = sOwn;
                __syncwarp();
                Stencil3Pair n;
                n.t1 = tring[p1 + myslot];
                n.t3 = tring[p1 + myslot - 1];
                n.t2 = tring[p2 + myslot - 1];
                n.t4 = tring[p1 + myslot - HY];
                n.t5 = tring[p2 + myslot - HY];
                n.t7 = tring[p2 + myslot - HY - 1];
                n.t6 = tring[p3 + myslot - HY - 1];
                n.s0 = sring[p3 + myslot - HY - 1];
                n.s1 = sring[p2 + myslot - HY - 1];
                n.s2 = sring[p1 + myslot - HY];
                n.s3 = sring[p2 + myslot - HY];
                n.s4 = sring[p2 + myslot - 1];
                n.s5 = sring[p1 + myslot - 1];
                n.s7 = sring[p1 + myslot];
                float va = t0a, vb = t0b;
                const bool u0 = active && yz0 && xa >= xlo0 && xa <= xhi0;
                const bool u1 = active && yz1 && xa >= xlo1 && xa <= xhi1;
                if (u0 || u1) {
                    const bool far0 = abs(src0.isx - xa) > a.radius || abs(src0.isy - ya) > a.radius ||
                                      abs(src0.isz - za) > a.radius;
                    const bool far1 = abs(src1.isx - xa) > a.radius || abs(src1.isy - ya) > a.radius ||
                                      abs(src1.isz - za) > a.radius;
                    F2 tu = fd3CartesianPair(a.h, n);
                    float tua = lo(tu), tub = hi(tu);
                    if (!far0) tua = fd3Uniform<float>(a.radius, a.h, src0, sg, xa, ya, za, fieldStencil(n, 0));
                    if (!far1) tub = fd3Uniform<float>(a.radius, a.h, src1, sg, xa, ya, za, fieldStencil(n, 1));
                    if (u0 && tua < t0a) {
                        va = tua;
                        row0[xa] = tua;
                        res0 = fmaxf(res0, t0a - tua);
                    }
                    if (u1 && tub < t0b) {
                        vb = tub;
                        row1[xa] = tub;
                        res1 = fmaxf(res1, t0b - tub);
                    }
                }
                const F2 v = f2(va, vb);
                tring[cur + myslot] = v;
                if (active) {
                    if (ly == LY3 - 1) putPair(yFace + static_cast<long long>(xp) * 2, tag, v);
                    if (lz == LZ3 - 1) putPair(zFace + static_cast<long long>(xp) * 2, tag, v);
                }
            }
        }
        if (!ok) break;
        const double r0 = warpMax(static_cast<double>(res0)), r1 = warpMax(static_cast<double>(res1));
        if (lane == 0) {
            if (r0 > 0)
                atomicMax(st.residual + static_cast<long long>(f0) * st.residualStride + a.residualSlot,
                          static_cast<unsigned long long>(__double_as_longlong(r0)));
            if (r1 > 0 && f1 != f0)
                atomicMax(st.residual + static_cast<long long>(f1) * st.residualStride + a.residualSlot,
                          static_cast<unsigned long long>(__double_as_longlong(r1)));
        }
    }
}

}  // namespace

size_t sweep3PairSmemBytes() { return (sizeof(F2) + sizeof(float)) * kRing * kPlane * kWarpsPerBlock; }

cudaError_t launchSweep3Pair(const Sweep3Args<float> &a, int blocks, cudaStream_t s) {
    sweep3PairKernel<<<blocks, kThreads, sweep3PairSmemBytes(), s>>>(a);
    return cudaGetLastError();
}

int sweep3PairBlocksPerSM() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sweep3PairKernel, kThreads, sweep3PairSmemBytes());
    return n > 0 ? n : 1;
}

}  // namespace eikx
