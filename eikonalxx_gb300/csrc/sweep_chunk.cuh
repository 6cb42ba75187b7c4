// Chunk-step 3D level-set sweep kernel for sm_103a.
//
// The same warp-block wavefront as sweep3Kernel (wavefront.cuh), with the unit of a
// step widened from one node to one 16-byte chunk of V = 16 / sizeof(T) consecutive
// x'-nodes (4 in FP32, 2 in FP64).  At step s lane (ly, lz) updates chunk
// k = s - ly - lz of its pencil, its V nodes in walk order: node e of the chunk reads
// node e-1 just updated, so the chunk reproduces the serial x-loop of the reference
// (include/private/solver3d.hpp:186-243) node for node, and every value it reads from
// another lane lies on an earlier level.
//
// What a step costs is paid once per chunk instead of once per node:
//   * the y'-, z'- and yz'-upwind lanes' chunks (travel times and cell slowness) come
//     from the per-warp ring as six 16-byte shared-memory loads; their x'-1 values are
//     the last elements of the chunks the lane read the step before (register carries);
//   * the own pencil streams as one 16-byte load of travel times and one of slowness per
//     step (fetched a step ahead), and a chunk is stored back with one 16-byte store
//     when any of its nodes decreased;
//   * halo values cross warp blocks as 32-byte mailbox chunks (four tagged 64-bit words:
//     one per FP32 value, two per FP64 value), read with two 16-byte relaxed loads that
//     are issued a step before they are needed.
// Near-source nodes (factored branch) are evaluated by an out-of-line call, so the V
// inlined copies of the update are the Cartesian operators only.
//
// The warp-block shape LY x LZ (pencils per warp, LY * LZ = 32) is a template parameter;
// each shape is instantiated in its own translation unit (sweep_chunk_<LY>x<LZ>.cu).
#pragma once
#include "sweep.h"
#include "wavefront.cuh"

namespace eikx {

namespace chunk {

constexpr int kRingC = 4;                           // ring depth in steps (reads go back 2)
constexpr int kThreadsC = 32 * kWarpsPerBlock;
// Own-pencil prefetch: a lane's travel-time and slowness chunks of step s are copied into
// shared-memory slot s % kPre, kAhead steps before they are used (cp.async, no registers).
constexpr int kPre = 4, kAhead = 3;
static_assert(kAhead < kPre && (kPre & (kPre - 1)) == 0, "a slot is refilled only after its step");

template <class T> struct alignas(16) Vec {
    static constexpr int N = 16 / sizeof(T);
    T v[N];
};
template <class T> __device__ __forceinline__ Vec<T> ldVec(const T *p) {
    Vec<T> r;
    *reinterpret_cast<uint4 *>(r.v) = *reinterpret_cast<const uint4 *>(p);
    return r;
}
template <class T> __device__ __forceinline__ void stVec(T *p, const Vec<T> &a) {
    *reinterpret_cast<uint4 *>(p) = *reinterpret_cast<const uint4 *>(a.v);
}
template <class T> __device__ __forceinline__ Vec<T> splat(T x) {
    Vec<T> r;
#pragma unroll
    for (int e = 0; e < Vec<T>::N; ++e) r.v[e] = x;
    return r;
}
template <class T> __device__ __forceinline__ Vec<T> reversed(const Vec<T> &a) {
    Vec<T> r;
#pragma unroll
    for (int e = 0; e < Vec<T>::N; ++e) r.v[e] = a.v[Vec<T>::N - 1 - e];
    return r;
}

__device__ __forceinline__ void ldRelaxed2(const unsigned long long *p, unsigned long long &a,
                                           unsigned long long &b) {
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(p));
}
__device__ __forceinline__ void stRelaxed2(unsigned long long *p, unsigned long long a, unsigned long long b) {
    asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(a), "l"(b));
}
// 16-byte asynchronous copy global -> shared (L2 only), its commit and its wait.
__device__ __forceinline__ void cpAsync16(void *smem, const void *gmem) {
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cpAsyncWait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// One chunk in the mailbox: four tagged words.  Each 64-bit word is written and read
// single-copy atomically and carries the tag of the sweep that wrote it, so a reader
// knows word by word whether the value is this sweep's.
template <class T> struct MailChunk {
    unsigned long long w[4];
    __device__ __forceinline__ void issue(const unsigned long long *p) {
        ldRelaxed2(p, w[0], w[1]);
        ldRelaxed2(p + 2, w[2], w[3]);
    }
    __device__ __forceinline__ bool ready(unsigned tag) const {
        return static_cast<unsigned>(w[0] >> 32) == tag && static_cast<unsigned>(w[1] >> 32) == tag &&
               static_cast<unsigned>(w[2] >> 32) == tag && static_cast<unsigned>(w[3] >> 32) == tag;
    }
    __device__ __forceinline__ Vec<T> value() const {
        Vec<T> r;
        if constexpr (sizeof(T) == 4) {
#pragma unroll
            for (int e = 0; e < 4; ++e) r.v[e] = __uint_as_float(static_cast<unsigned>(w[e]));
        } else {
#pragma unroll
            for (int e = 0; e < 2; ++e)
                r.v[e] = __longlong_as_double(
                    static_cast<long long>((w[2 * e + 1] << 32) | (w[2 * e] & 0xffffffffull)));
        }
        return r;
    }
    // Wait (bounded) until all four words carry `tag`, re-reading them.
    __device__ __forceinline__ bool take(const unsigned long long *p, unsigned tag, int *abortFlag,
                                         unsigned long long spinLimit) {
        unsigned long long it = 0;
        while (!ready(tag)) {
            if ((++it & 31ull) == 0) {
                if (ldVolatile(abortFlag)) return false;
                if (it > spinLimit) {
                    atomicExch(abortFlag, 1);
                    return false;
                }
            }
            __nanosleep(32);
            issue(p);
        }
        return true;
    }
};
// The four tagged words a chunk of values would carry in the mailbox.
template <class T>
__device__ __forceinline__ void tagWords(unsigned tag, const Vec<T> &v, unsigned long long (&w)[4]) {
    const unsigned long long t = static_cast<unsigned long long>(tag) << 32;
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int e = 0; e < 4; ++e) w[e] = t | __float_as_uint(v.v[e]);
    } else {
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v.v[e]));
            w[2 * e] = t | (b & 0xffffffffull);
            w[2 * e + 1] = t | (b >> 32);
        }
    }
}
template <class T>
__device__ __forceinline__ void putChunk(unsigned long long *p, unsigned tag, const Vec<T> &v) {
    const unsigned long long t = static_cast<unsigned long long>(tag) << 32;
    unsigned long long w[4];
    if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int e = 0; e < 4; ++e) w[e] = t | __float_as_uint(v.v[e]);
    } else {
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v.v[e]));
            w[2 * e] = t | (b & 0xffffffffull);
            w[2 * e + 1] = t | (b >> 32);
        }
    }
    stRelaxed2(p, w[0], w[1]);
    stRelaxed2(p + 2, w[2], w[3]);
}

// The raw slowness of a node's stencil cells (the reference's cell indices, clamped to the
// grid: Solver3DSweep::updateFSM in include/private/solver3d.hpp), from the model's
// natural-order cells, for launches whose stencils carry the scaled slowness.
template <class T>
__device__ __forceinline__ void rawStencilCells(Stencil3<T> &n, const void *cells, int cells64, int nx, int ny, int nz,
                                                const SweepSigns &sg, int ix, int iy, int iz) {
    const int ncx = nx - 1, ncy = ny - 1, ncz = nz - 1;
    auto cl = [](int v, int hi) { return v < 0 ? 0 : (v > hi ? hi : v); };
    const bool fx = sg.ixShift > 0, fy = sg.iyShift > 0, fz = sg.izShift > 0;
    const int cxu = cl(fx ? ix : ix - 1, ncx - 1), cxo = cl(fx ? cxu - 1 : cxu + 1, ncx - 1);
    const int cyu = cl(fy ? iy : iy - 1, ncy - 1), cyo = cl(fy ? cyu - 1 : cyu + 1, ncy - 1);
    const int czu = cl(fz ? iz : iz - 1, ncz - 1), czo = cl(fz ? czu - 1 : czu + 1, ncz - 1);
    auto S = [&](int cx, int cy, int cz) -> T {
        const long long i = (static_cast<long long>(cz) * ncy + cy) * ncx + cx;
        return cells64 ? static_cast<T>(static_cast<const double *>(cells)[i])
                       : static_cast<T>(static_cast<const float *>(cells)[i]);
    };
    n.s0 = S(cxu, cyu, czu); n.s1 = S(cxo, cyu, czu); n.s2 = S(cxo, cyo, czu); n.s3 = S(cxu, cyo, czu);
    n.s4 = S(cxu, cyu, czo); n.s5 = S(cxo, cyu, czo); n.s7 = S(cxu, cyo, czo);
}

// Factored (near-source) updates, out of line: taken by a few hundred nodes per field,
// so the V inlined copies of the update hold only the Cartesian operators.
template <class T>
__device__ __noinline__ T nearUniform(T h, const SourceT<T> src, const SweepSigns sg, int ix, int iy, int iz,
                                      const Stencil3<T> n) {
    return fd3UniformNear(h, src, sg, ix, iy, iz, n);
}
template <class T>
__device__ __noinline__ T nearUniformRaw(T h, const SourceT<T> src, const SweepSigns sg, int ix, int iy, int iz,
                                         Stencil3<T> n, const void *cells, int cells64, int nx, int ny, int nz) {
    rawStencilCells(n, cells, cells64, nx, ny, nz, sg, ix, iy, iz);
    return fd3UniformNear(h, src, sg, ix, iy, iz, n);
}
template <class T>
__device__ __noinline__ T nearNonUniform(const Spacing3<T> g, const SourceT<T> src, const SweepSigns sg, int ix,
                                         int iy, int iz, const Stencil3<T> n) {
    return fd3NonUniformNear(g, src, sg, ix, iy, iz, n);
}
// The factored branch with the analytic factor in FP64 (eikx_options.near_fp64, FP32).
template <class T>
__device__ __noinline__ T nearUniform64(T h, const SourceT<T> src, const SourceFp64 *f, const SweepSigns sg, int ix,
                                        int iy, int iz, const Stencil3<T> n) {
    const SourceFp64 d = *f;
    return fd3UniformNear<T, true>(h, src, sg, ix, iy, iz, n, &d);
}
template <class T>
__device__ __noinline__ T nearNonUniform64(const Spacing3<T> g, const SourceT<T> src, const SourceFp64 *f,
                                           const SweepSigns sg, int ix, int iy, int iz, const Stencil3<T> n) {
    const SourceFp64 d = *f;
    return fd3NonUniformNear<T, true>(g, src, sg, ix, iy, iz, n, &d);
}

__device__ __forceinline__ void clearNextQueue(const SolveState &st, int buf) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *st.queue[buf ^ 1] = 0u;
}

// INITMODE 1: the source-limited initialisation pass (a.init = 1), compiled apart so that
// the refinement sweeps (INITMODE 0) carry none of its block skipping.  INITMODE 2: a stream
// of sources through slots (a.slots, eikx_options.max_in_flight): each slot's field is in
// its initialisation pass or in refinement according to the sweep at which it started, so
// the mode, the residual slot and the field buffer are read per work item.  NEAR64: the
// factored branch with its analytic factor in FP64 (eikx_options.near_fp64, FP32 sweeps),
// compiled into its own kernels (sweep3ChunkNear64Kernel) so that the others carry none of it.
template <class T, bool UNIFORM, bool REV, bool BATCH, int LY, int LZ, int INITMODE, bool NEAR64>
__device__ __forceinline__ void sweep3ChunkBody(const Sweep3Args<T> &a) {
    static_assert(LY * LZ == 32 && LZ + 1 + LY <= 32, "a warp holds 32 pencils and its halo helpers");
    constexpr int HY = LY + 1, HZ = LZ + 1;          // ring plane incl. halo row/column
    constexpr int kPlane = HY * HZ;
    constexpr int V = Vec<T>::N;
    constexpr int W = sizeof(T) / 4;                // mailbox words per value
    extern __shared__ __align__(16) unsigned char smemRaw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ly = lane % LY, lz = lane / LY;
    Vec<T> *tring = reinterpret_cast<Vec<T> *>(smemRaw) + warp * (2 * kRingC * kPlane);
    Vec<T> *sring = tring + kRingC * kPlane;
    // prefetch slots after all rings: [warp][slot][T | S][lane]
    Vec<T> *pre = reinterpret_cast<Vec<T> *>(smemRaw) + kWarpsPerBlock * (2 * kRingC * kPlane) +
                  warp * (kPre * 64) + lane;
    const SolveState &st = a.st;
    clearNextQueue(st, a.buf);
    if (ldVolatile(st.abortFlag)) return;
    const unsigned tag = *st.epoch + static_cast<unsigned>(a.sweepIndex);

    const int fy = (a.sweep >> 1) & 1, fz = (a.sweep >> 2) & 1;
    SweepSigns sg;
    sg.ixShift = REV ? 1 : -1; sg.iyShift = fy ? 1 : -1; sg.izShift = fz ? 1 : -1;
    sg.signX = REV ? -1 : 1; sg.signY = fy ? -1 : 1; sg.signZ = fz ? -1 : 1;
    const T huge = static_cast<T>(1.e10);
    // FP64 sweeps of one model on a uniform grid read the slowness copies multiplied by h
    // (a.hsPos, a.hsNeg): with h > 0 round-to-nearest multiplication is monotone, so
    // h * min(s, ...) equals min(h * s, ...) bit for bit, and the Cartesian operators take their
    // slowness terms without GB300's narrow FP64 multiplies.  Their factored branch reads the
    // raw cells.  (In FP32 the same change measured no faster.)
    constexpr bool SCALED = UNIFORM && !BATCH && sizeof(T) == 8;
    const T sHuge = SCALED ? a.h * huge : huge;   // the slowness of a cell beyond the walk

    // helper lanes stand in for the virtual upwind lanes of the halo row/column
    const bool helper = lane < HZ + LY;
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
        const int f = item.x, b = item.y, c = item.z;
        if (st.converged[f]) continue;
        bool init = INITMODE == 1;
        int residualSlot = a.residualSlot;
        long long fieldOffset = static_cast<long long>(f) * a.fieldStride;
        if constexpr (INITMODE == 2) {
            // the slot's field: started at sweep si.x of the stream, in buffer si.y
            const int2 si = a.slots[f];
            const int phase = a.sweepIndex - si.x;
            if (si.x < 0 || phase < 0) continue;   // an idle slot
            init = a.initSweeps && phase < 8;
            residualSlot = phase + (a.initSweeps ? 0 : 8);
            fieldOffset = static_cast<long long>(si.y) * a.fieldStride;
        }
        const SourceT<T> src = a.srcs[f];

        // grid of this work item: the launch's (one model) or the unit's (batch)
        const Grid3Unit<T> *unit = BATCH ? a.units + f : nullptr;
        const int Px = BATCH ? unit->Px : a.pitch;
        const int nx = BATCH ? unit->nx : a.nx, ny = BATCH ? unit->ny : a.ny, nz = BATCH ? unit->nz : a.nz;
        const int tilesY = BATCH ? unit->tilesY : a.tilesY;
        const int spPitch = BATCH ? unit->spPitch : a.spPitch;
        const long long spPlane = BATCH ? unit->spPlane : a.spPlane;
        const T *sp = BATCH ? (REV ? unit->spNeg : unit->spPos)
                            : SCALED ? (REV ? a.hsNeg : a.hsPos) : (REV ? a.spNeg : a.spPos);
        T *field = BATCH ? unit->tt : a.tt + fieldOffset;
        const long long faceWords = static_cast<long long>(LY + LZ) * Px * W;
        unsigned long long *fieldBox =
            BATCH ? unit->mbox : st.mbox + static_cast<long long>(f) * a.tilesZ * a.tilesY * faceWords;
        const T h = BATCH ? unit->h : a.h;
        const int nChunks = Px / V;
        const int y0 = b * LY, z0 = c * LZ;
        const int yp = y0 + ly, zp = z0 + lz;
        const bool laneValid = yp < ny && zp < nz;
        const int ya = laneValid ? reflect(yp, ny, fy) : 0;
        const int za = laneValid ? reflect(zp, nz, fz) : 0;
        int xlo, xhi, ylo, yhi, zlo, zhi;
        axisBounds(nx, REV, init, src.isx, xlo, xhi);
        axisBounds(ny, fy, init, src.isy, ylo, yhi);
        axisBounds(nz, fz, init, src.isz, zlo, zhi);
        // Initialisation pass: the update range along x' starts at the source's column, so
        // the field's lanes all walk from the chunk before the one holding it (whose last
        // values are the first updated node's x'-1 neighbours; it updates nothing) instead
        // of from chunk 0.  kBase is the same for every block of a field, so the mailbox
        // chunks a block waits for are the ones its upstream blocks publish.
        int kBase = 0;
        if (init) kBase = max(0, (REV ? Px - 1 - xhi : xlo) / V - 1);
        const int nSteps = nChunks - kBase + LY + LZ - 2;
        // Initialisation pass: the update range starts at y' = yp0, z' = zp0 and runs to the
        // end of each axis.  Warp blocks wholly before it update nothing: they are left out,
        // and the blocks after them read those rows from the field, which the sweep does not
        // change, instead of from the mailbox.
        int bStart = 0, cStart = 0;
        if (init) {
            bStart = (fy ? ny - 1 - yhi : ylo) / LY;
            cStart = (fz ? nz - 1 - zhi : zlo) / LZ;
            if (b < bStart || c < cStart) continue;
        }
        const bool yzUpd = laneValid && ya >= ylo && ya <= yhi && za >= zlo && za <= zhi;
        // the factored branch applies within `radius` cells of the source cell on every axis
        const bool yzNear = abs(src.isy - ya) <= a.radius && abs(src.isz - za) <= a.radius;
        // walk positions of the factored x-range (empty when the lane's y', z' are not near;
        // the radius clamped to the pitch, which no |isx - x| reaches)
        const int rx = min(a.radius, Px);
        const int nxa = src.isx - rx, nxb = src.isx + rx;
        const int nearLo = !yzNear ? 1 << 30 : REV ? Px - 1 - nxb : nxa;
        const int nearHi = !yzNear ? -1 : REV ? Px - 1 - nxa : nxb;
        T *row = field + (static_cast<long long>(za) * ny + ya) * Px;
        const T *srow = sp + static_cast<long long>(za + (fz ? 0 : 1)) * spPlane +
                        static_cast<long long>(ya + (fy ? 0 : 1)) * spPitch;
        // chunk k of a row in walk order: forward rows start at the row, reversed rows end there
        auto tChunk = [&](T *r, int k) { return REV ? r + Px - (k + 1) * V : r + k * V; };
        auto sChunk = [&](const T *r, int k) { return REV ? r + Px - (k + 1) * V : r + (k + 1) * V; };
        auto walk = [&](const Vec<T> &m) { return REV ? reversed(m) : m; };   // memory <-> walk order
        // the own pencil's chunk of step sv into slot sv % kPre; one commit group per step
        auto prefetch = [&](int sv) {
            const int kv = sv - ly - lz + kBase;
            if (laneValid && kv >= kBase && kv < nChunks) {
                Vec<T> *slot = pre + (sv & (kPre - 1)) * 64;
                cpAsync16(slot, tChunk(row, kv));
                cpAsync16(slot + 32, sChunk(srow, kv));
            }
            cpAsyncCommit();
        };
#pragma unroll
        for (int sv = 0; sv < kAhead; ++sv) prefetch(sv);

        // mailbox: this block's faces, and the upstream face row a helper lane reads
        unsigned long long *box = fieldBox + (static_cast<long long>(c) * tilesY + b) * faceWords;
        unsigned long long *yFace = box + static_cast<long long>(lz) * Px * W;          // ly == LY-1
        unsigned long long *zFace = box + static_cast<long long>(LZ + ly) * Px * W;    // lz == LZ-1
        const int vyp = y0 + vly, vzp = z0 + vlz;
        const bool vValid = helper && vyp >= 0 && vzp >= 0 && vyp < ny && vzp < nz;
        // the virtual lane's block was left out: its row is read from the field (vbox then
        // holds the row's address)
        const bool vField = init && vValid && ((vly < 0 && b - 1 < bStart) || (vlz < 0 && c - 1 < cStart));
        const unsigned long long *vbox = box;
        const T *vsrow = sp;
        if (vValid) {
            const int vya = reflect(vyp, ny, fy), vza = reflect(vzp, nz, fz);
            if (vField) {
                vbox = reinterpret_cast<const unsigned long long *>(field + (static_cast<long long>(vza) * ny + vya) * Px);
            } else if (vly < 0) {
                // block (b-1, c), or the corner block (b-1, c-1): its y' face row
                vbox = box - (vlz >= 0 ? faceWords : (tilesY + 1) * faceWords) +
                       static_cast<long long>(vlz >= 0 ? vlz : LZ - 1) * Px * W;
            } else {
                // block (b, c-1): its z' face row
                vbox = box - tilesY * faceWords + static_cast<long long>(LZ + vly) * Px * W;
            }
            vsrow = sp + static_cast<long long>(vza + (fz ? 0 : 1)) * spPlane +
                    static_cast<long long>(vya + (fy ? 0 : 1)) * spPitch;
        }

        // Halo pipeline: the chunk a virtual lane produces at step sv goes into ring slot
        // sv; its mailbox words are loaded one step ahead and checked at step sv.
        auto haloChunk = [&](int sv) { return sv - vly - vlz + kBase; };
        auto haloValid = [&](int kv) { return vValid && kv >= kBase && kv < nChunks; };
        auto haloStore = [&](int sv, const Vec<T> &tv, const Vec<T> &sv_) {
            const int slot = (sv & (kRingC - 1)) * kPlane + vslot;
            tring[slot] = tv;
            sring[slot] = sv_;
        };
        MailChunk<T> mslot;
        Vec<T> sslot = splat(sHuge);
        auto issue = [&](int sv) {
            const int kv = haloChunk(sv);
            if (helper && haloValid(kv)) {
                if (init && vField) {
                    T *vrow = const_cast<T *>(reinterpret_cast<const T *>(vbox));
                    tagWords(tag, walk(ldVec(tChunk(vrow, kv))), mslot.w);
                } else {
                    mslot.issue(vbox + static_cast<long long>(kv) * V * W);
                }
                sslot = ldVec(sChunk(vsrow, kv));
            }
        };
        auto consume = [&](int sv) -> bool {
            bool good = true;
            if (helper) {
                const int kv = haloChunk(sv);
                Vec<T> tv = splat(huge), svv = splat(sHuge);
                if (haloValid(kv)) {
                    good = mslot.take(vbox + static_cast<long long>(kv) * V * W, tag, st.abortFlag, st.spinLimit);
                    tv = mslot.value();
                    svv = walk(sslot);
                }
                haloStore(sv, tv, svv);
            }
            return __all_sync(kFull, good);
        };

        issue(-2);
        bool ok = consume(-2);
        if (ok) {
            issue(-1);
            ok = consume(-1);
        }
        if (ok) issue(0);
        // x'-1 values of the chunks read the step before (walk position k*V - 1)
        T cT1 = huge, cT3 = huge, cT4 = huge, cT7 = huge;
        T cS1 = sHuge, cS2 = sHuge, cS5 = sHuge, cS7 = sHuge;
        T res = 0;
        for (int s = 0; s < nSteps && ok; ++s) {
            ok = consume(s);
            if (!ok) break;
            issue(s + 1);
            const int k = s - ly - lz + kBase;
            const bool active = laneValid && k >= kBase && k < nChunks;
            prefetch(s + kAhead);
            cpAsyncWait<kAhead>();   // this step's group has landed
            Vec<T> tOwn = splat(huge), sOwn = splat(sHuge);
            if (active) {
                const Vec<T> *slot = pre + (s & (kPre - 1)) * 64;
                tOwn = walk(slot[0]);
                sOwn = walk(slot[32]);
            }
            const int cur = (s & (kRingC - 1)) * kPlane;
            const int p1 = ((s - 1) & (kRingC - 1)) * kPlane;
            const int p2 = ((s - 2) & (kRingC - 1)) * kPlane;
            sring[cur + myslot] = sOwn;
            __syncwarp();
            const Vec<T> tY = tring[p1 + myslot - 1];          // lane (ly-1, lz): same chunk
            const Vec<T> tZ = tring[p1 + myslot - HY];         // lane (ly, lz-1)
            const Vec<T> tYZ = tring[p2 + myslot - HY - 1];    // lane (ly-1, lz-1)
            const Vec<T> sY = sring[p1 + myslot - 1];
            const Vec<T> sZ = sring[p1 + myslot - HY];
            const Vec<T> sYZ = sring[p2 + myslot - HY - 1];
            Vec<T> out = tOwn;
            bool changed = false;
#pragma unroll
            for (int e = 0; e < V; ++e) {
                const int xp = k * V + e;
                const int xa = REV ? Px - 1 - xp : xp;
                if (active && yzUpd && xa >= xlo && xa <= xhi) {
                    Stencil3<T> n;
                    n.t1 = e ? out.v[e - 1] : cT1;
                    n.t3 = tY.v[e];
                    n.t2 = e ? tY.v[e - 1] : cT3;
                    n.t4 = tZ.v[e];
                    n.t5 = e ? tZ.v[e - 1] : cT4;
                    n.t7 = tYZ.v[e];
                    n.t6 = e ? tYZ.v[e - 1] : cT7;
                    n.s0 = e ? sYZ.v[e - 1] : cS1;
                    n.s1 = sYZ.v[e];
                    n.s2 = sZ.v[e];
                    n.s3 = e ? sZ.v[e - 1] : cS2;
                    n.s4 = e ? sY.v[e - 1] : cS5;
                    n.s5 = sY.v[e];
                    n.s7 = e ? sOwn.v[e - 1] : cS7;
                    const bool near = xp >= nearLo && xp <= nearHi;
                    const T t0 = out.v[e];
                    T tu;
                    if (NEAR64 && near) {
                        // FP32 only, so the stencil holds raw slowness values
                        if constexpr (UNIFORM) tu = nearUniform64<T>(h, src, a.srcs64 + f, sg, xa, ya, za, n);
                        else tu = nearNonUniform64<T>(BATCH ? unit->sp3 : a.sp3, src, a.srcs64 + f, sg, xa, ya, za, n);
                    } else if (SCALED) {
                        // the Cartesian operators with lower-bound exits: min(t0, tu) is the
                        // same bit for bit as with fd3UniformFar
                        tu = near ? nearUniformRaw<T>(h, src, sg, xa, ya, za, n, a.cells, a.cells64, nx, ny, nz)
                                  : fd3UniformFarBounded<T, true>(h, n, t0);
                    } else if (UNIFORM) {
                        tu = near ? nearUniform<T>(h, src, sg, xa, ya, za, n) : fd3UniformFarBounded<T>(h, n, t0);
                    } else {
                        const Spacing3<T> &g = BATCH ? unit->sp3 : a.sp3;
                        tu = near ? nearNonUniform<T>(g, src, sg, xa, ya, za, n) : fd3NonUniformFar<T>(g, n);
                    }
                    if (tu < t0) {
                        out.v[e] = tu;
                        changed = true;
                        res = dmax(res, t0 - tu);
                    }
                }
            }
            tring[cur + myslot] = out;
            if (active) {
                if (changed) stVec(tChunk(row, k), walk(out));
                if (ly == LY - 1) putChunk(yFace + static_cast<long long>(k) * V * W, tag, out);
                if (lz == LZ - 1) putChunk(zFace + static_cast<long long>(k) * V * W, tag, out);
            }
            cT1 = out.v[V - 1]; cT3 = tY.v[V - 1]; cT4 = tZ.v[V - 1]; cT7 = tYZ.v[V - 1];
            cS1 = sYZ.v[V - 1]; cS2 = sZ.v[V - 1]; cS5 = sY.v[V - 1]; cS7 = sOwn.v[V - 1];
        }
        cpAsyncWait<0>();   // no copy into the slots outlives the work item
        if (!ok) break;
        const double r = warpMax(static_cast<double>(res));
        if (lane == 0 && r > 0)
            atomicMax(st.residual + static_cast<long long>(f) * st.residualStride + residualSlot,
                      static_cast<unsigned long long>(__double_as_longlong(r)));
    }
}

template <class T, bool UNIFORM, bool REV, bool BATCH, int LY, int LZ, int INITMODE>
__global__ void __launch_bounds__(kThreadsC) sweep3ChunkKernel(const Sweep3Args<T> a) {
    sweep3ChunkBody<T, UNIFORM, REV, BATCH, LY, LZ, INITMODE, false>(a);
}
// Held to 128 registers (the default kernels' 4 blocks per SM); the out-of-line FP64
// branch spills what it needs beyond them.
template <class T, bool UNIFORM, bool REV, bool BATCH, int LY, int LZ, int INITMODE>
__global__ void __launch_bounds__(kThreadsC) sweep3ChunkNear64Kernel(const Sweep3Args<T> a) {
    sweep3ChunkBody<T, UNIFORM, REV, BATCH, LY, LZ, INITMODE, true>(a);
}

template <int LY, int LZ> constexpr size_t smemBytes() {
    return (2 * kRingC * (LY + 1) * (LZ + 1) + kPre * 64) * 16 * kWarpsPerBlock;
}

template <class T, bool U, bool R, bool B, int LY, int LZ>
void launchOne(const Sweep3Args<T> &a, int blocks, cudaStream_t s) {
    const size_t smem = smemBytes<LY, LZ>();
    // the stream mode's instances exist for one-model launches only
    const int mode = !B && a.slots ? 2 : a.init ? 1 : 0;
    if constexpr (sizeof(T) == 4) {
        if (a.srcs64) {
            if (mode == 1) sweep3ChunkNear64Kernel<T, U, R, B, LY, LZ, 1><<<blocks, kThreadsC, smem, s>>>(a);
            else if (mode == 0) sweep3ChunkNear64Kernel<T, U, R, B, LY, LZ, 0><<<blocks, kThreadsC, smem, s>>>(a);
            else if constexpr (!B) sweep3ChunkNear64Kernel<T, U, R, B, LY, LZ, 2><<<blocks, kThreadsC, smem, s>>>(a);
            return;
        }
    }
    if (mode == 1) sweep3ChunkKernel<T, U, R, B, LY, LZ, 1><<<blocks, kThreadsC, smem, s>>>(a);
    else if (mode == 0) sweep3ChunkKernel<T, U, R, B, LY, LZ, 0><<<blocks, kThreadsC, smem, s>>>(a);
    else if constexpr (!B) sweep3ChunkKernel<T, U, R, B, LY, LZ, 2><<<blocks, kThreadsC, smem, s>>>(a);
}

template <class T, bool B, int LY, int LZ>
void launchShape(const Sweep3Args<T> &a, bool uniform, int blocks, cudaStream_t s) {
    const bool rev = (a.sweep & 1) != 0;
    if (uniform) {
        if (rev) launchOne<T, true, true, B, LY, LZ>(a, blocks, s);
        else launchOne<T, true, false, B, LY, LZ>(a, blocks, s);
    } else {
        if (rev) launchOne<T, false, true, B, LY, LZ>(a, blocks, s);
        else launchOne<T, false, false, B, LY, LZ>(a, blocks, s);
    }
}

template <class T, bool B, int LY, int LZ> int blocksPerSM(bool uniform) {
    // the persistent grid is sized for the refinement sweeps (the two directions differ only
    // in addressing; take the lower occupancy).  An initialisation sweep whose kernel fits
    // fewer blocks runs the rest as they free up: a block dequeues work only once resident
    // and waits only on work dequeued before it, so no wait depends on a block not running.
    const void *k[2];
    if (uniform) {
        k[0] = reinterpret_cast<const void *>(sweep3ChunkKernel<T, true, false, B, LY, LZ, 0>);
        k[1] = reinterpret_cast<const void *>(sweep3ChunkKernel<T, true, true, B, LY, LZ, 0>);
    } else {
        k[0] = reinterpret_cast<const void *>(sweep3ChunkKernel<T, false, false, B, LY, LZ, 0>);
        k[1] = reinterpret_cast<const void *>(sweep3ChunkKernel<T, false, true, B, LY, LZ, 0>);
    }
    int best = 1 << 30;
    for (const void *f : k) {
        int n = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, kThreadsC, smemBytes<LY, LZ>());
        best = n < best ? n : best;
    }
    return best > 0 ? best : 1;
}

}  // namespace chunk

// Launch and occupancy entry points of one warp-block shape (one translation unit each).
#define EIKX_CHUNK_SHAPE(LY_, LZ_)                                                                    \
    template <class T>                                                                                \
    cudaError_t launchSweep3Chunk_##LY_##x##LZ_(const Sweep3Args<T> &a, bool uniform, int blocks,     \
                                                cudaStream_t s) {                                     \
        if (a.units) {                                                                                \
            chunk::launchShape<T, true, LY_, LZ_>(a, uniform, blocks, s);                             \
        } else {                                                                                      \
            if (sizeof(T) == 8 && uniform && (!a.hsPos || !a.hsNeg || !a.cells))                     \
                return cudaErrorInvalidValue;                                                         \
            chunk::launchShape<T, false, LY_, LZ_>(a, uniform, blocks, s);                            \
        }                                                                                             \
        return cudaGetLastError();                                                                    \
    }                                                                                                 \
    template <class T> int sweep3ChunkBlocksPerSM_##LY_##x##LZ_(bool uniform, bool batch) {           \
        return batch ? chunk::blocksPerSM<T, true, LY_, LZ_>(uniform)                                 \
                     : chunk::blocksPerSM<T, false, LY_, LZ_>(uniform);                               \
    }                                                                                                 \
    template cudaError_t launchSweep3Chunk_##LY_##x##LZ_<float>(const Sweep3Args<float> &, bool, int, \
                                                                cudaStream_t);                        \
    template cudaError_t launchSweep3Chunk_##LY_##x##LZ_<double>(const Sweep3Args<double> &, bool,    \
                                                                 int, cudaStream_t);                  \
    template int sweep3ChunkBlocksPerSM_##LY_##x##LZ_<float>(bool, bool);                             \
    template int sweep3ChunkBlocksPerSM_##LY_##x##LZ_<double>(bool, bool);

}  // namespace eikx
