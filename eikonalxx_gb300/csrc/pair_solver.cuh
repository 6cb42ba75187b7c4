// The 3D uniform-grid local solver evaluated for two fields at once.
//
// Two fields (two sources on the same model) share the node, its seven cell slownesses
// and every slowness-only quantity; their travel times differ.  The travel-time
// arithmetic runs on the packed FP32 pipe (add/sub/mul.rn.f32x2: two IEEE binary32
// operations, each rounded to nearest exactly as its scalar form), the comparisons,
// min/max and square roots per field.  Every operation of a field is the one
// fd3Uniform performs, in the same order, so each half equals fd3Uniform bit for bit
// (solverUtilities3d.hpp:258-370, Cartesian operators).  The factored branch near a
// source is left to the scalar fd3Uniform.
#pragma once
#include <cuda_runtime.h>
#include "local_solver.cuh"

namespace eikx {

// Two FP32 values in one 64-bit register pair.
struct F2 {
    unsigned long long v;
};
__device__ __forceinline__ F2 f2(float a, float b) {
    F2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ F2 f2(float a) { return f2(a, a); }
__device__ __forceinline__ float lo(F2 a) { return __uint_as_float(static_cast<unsigned>(a.v)); }
__device__ __forceinline__ float hi(F2 a) { return __uint_as_float(static_cast<unsigned>(a.v >> 32)); }
__device__ __forceinline__ F2 operator+(F2 a, F2 b) {
    F2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 operator-(F2 a, F2 b) {
    F2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 operator*(F2 a, F2 b) {
    F2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 neg(F2 a) { return f2(-lo(a), -hi(a)); }
// Products whose result feeds an addition or subtraction are formed per field with the
// scalar mul.rn.f32: measured on sm_103a, a packed mul.rn.f32x2 feeding a packed
// add/sub.rn.f32x2 is contracted into a fused multiply-add (different rounding) even
// under --fmad=false, whereas a scalar product feeding a packed sum is not.
__device__ __forceinline__ F2 mulSep(F2 a, F2 b) { return f2(lo(a) * lo(b), hi(a) * hi(b)); }
__device__ __forceinline__ F2 sq(F2 a) { return mulSep(a, a); }

struct Stencil3Pair {
    float s0, s1, s2, s3, s4, s5, s7;   // shared by both fields
    F2 t1, t2, t3, t4, t5, t6, t7;       // (field 0, field 1)
};

// One field of a Stencil3Pair as the scalar stencil.
__device__ __forceinline__ Stencil3<float> fieldStencil(const Stencil3Pair &n, int k) {
    Stencil3<float> r;
    r.s0 = n.s0; r.s1 = n.s1; r.s2 = n.s2; r.s3 = n.s3; r.s4 = n.s4; r.s5 = n.s5; r.s7 = n.s7;
    auto pick = [k](F2 a) { return k == 0 ? lo(a) : hi(a); };
    r.t1 = pick(n.t1); r.t2 = pick(n.t2); r.t3 = pick(n.t3); r.t4 = pick(n.t4);
    r.t5 = pick(n.t5); r.t6 = pick(n.t6); r.t7 = pick(n.t7);
    return r;
}

// Cartesian (non-factored) update of both fields, fd3Uniform's operators.
__device__ __forceinline__ F2 fd3CartesianPair(float h, const Stencil3Pair &n) {
    const float huge = 1.e10f;
    const float one = 1.0f;
    // slowness-only terms (computed once for both fields)
    const float minS0S3 = fminf(n.s0, n.s3);
    const float minS0S1 = fminf(n.s0, n.s1);
    const float minS0S4 = fminf(n.s0, n.s4);
    const F2 h1 = f2(h * fminf(minS0S3, fminf(n.s4, n.s7)));
    const F2 h2 = f2(h * fminf(minS0S4, fminf(n.s1, n.s5)));
    const F2 h3 = f2(h * fminf(minS0S1, fminf(n.s2, n.s3)));
    const float hs03 = h * minS0S3, hs01 = h * minS0S1, hs04 = h * minS0S4;
    const F2 hs03v = f2(hs03), hs01v = f2(hs01), hs04v = f2(hs04);
    const F2 q03 = f2(2 * (hs03 * hs03)), q01 = f2(2 * (hs01 * hs01)), q04 = f2(2 * (hs04 * hs04));
    const float hs0 = h * n.s0;
    const F2 c27 = f2(27 * hs0 * hs0);
    const F2 t1 = n.t1, t2 = n.t2, t3 = n.t3, t4 = n.t4, t5 = n.t5, t6 = n.t6, t7 = n.t7;
    // 1D head-wave operators
    const F2 a1 = t1 + h1, a2 = t3 + h2, a3 = t4 + h3;
    const float t1dA = fminf(fminf(lo(a1), lo(a2)), lo(a3));
    const float t1dB = fminf(fminf(hi(a1), hi(a2)), hi(a3));
    // 2D diagonal operators in the XZ, YZ and XY planes
    const F2 dXZ = t1 - t4, dYZ = t3 - t4, dXY = t1 - t3;
    const F2 detXZ = q03 - sq(dXZ), detYZ = q01 - sq(dYZ), detXY = q04 - sq(dXY);
    const F2 t1p03 = t1 + hs03v, t4p03 = t4 + hs03v;
    const F2 t4p01 = t4 + hs01v, t3p01 = t3 + hs01v;
    const F2 t1p04 = t1 + hs04v, t3p04 = t3 + hs04v;
    const bool cXZa = lo(detXZ) > 0 && lo(t4) <= lo(t1p03) && lo(t1) <= lo(t4p03);
    const bool cXZb = hi(detXZ) > 0 && hi(t4) <= hi(t1p03) && hi(t1) <= hi(t4p03);
    const bool cYZa = lo(detYZ) > 0 && lo(t3) <= lo(t4p01) && lo(t4) <= lo(t3p01);
    const bool cYZb = hi(detYZ) > 0 && hi(t3) <= hi(t4p01) && hi(t4) <= hi(t3p01);
    const bool cXYa = lo(detXY) > 0 && lo(t3) <= lo(t1p04) && lo(t1) <= lo(t3p04);
    const bool cXYb = hi(detXY) > 0 && hi(t3) <= hi(t1p04) && hi(t1) <= hi(t3p04);
    const F2 rXZ = f2(sqrtf(cXZa ? lo(detXZ) : one), sqrtf(cXZb ? hi(detXZ) : one));
    const F2 rYZ = f2(sqrtf(cYZa ? lo(detYZ) : one), sqrtf(cYZb ? hi(detYZ) : one));
    const F2 rXY = f2(sqrtf(cXYa ? lo(detXY) : one), sqrtf(cXYb ? hi(detXY) : one));
    const F2 eXZ = t5 + rXZ, eYZ = t7 + rYZ, eXY = t2 + rXY;
    const float t2dA = fminf(fminf(cXZa ? lo(eXZ) : huge, cYZa ? lo(eYZ) : huge), cXYa ? lo(eXY) : huge);
    const float t2dB = fminf(fminf(cXZb ? hi(eXZ) : huge, cYZb ? hi(eYZ) : huge), cXYb ? hi(eXY) : huge);
    // 8-point operator
    const F2 hf = f2(0.5f);
    const F2 Tx = ((t1 + mulSep(hf, ((neg(t4) + t5) - t3) + t2)) - t7) + t6;
    const F2 Ty = ((t3 + mulSep(hf, ((neg(t4) + t7) - t1) + t2)) - t5) + t6;
    const F2 Tz = ((t4 + mulSep(hf, ((neg(t1) + t5) - t3) + t7)) - t2) + t6;
    const F2 dxy = Tx - Ty, dxz = Tx - Tz, dyz = Ty - Tz;
    const F2 det = ((c27 - sq(dxy)) - sq(dxz)) - sq(dyz);
    const bool c3a = fminf(t1dA, t2dA) > fmaxf(fmaxf(lo(t1), lo(t4)), lo(t3)) && lo(det) >= 0;
    const bool c3b = fminf(t1dB, t2dB) > fmaxf(fmaxf(hi(t1), hi(t4)), hi(t3)) && hi(det) >= 0;
    const F2 r3 = f2(sqrtf(c3a ? lo(det) : one), sqrtf(c3b ? hi(det) : one));
    const F2 e3 = f2(static_cast<float>(0.33333333333333333333333)) * (((Tx + Ty) + Tz) + r3);
    const float t3dA = c3a ? lo(e3) : huge, t3dB = c3b ? hi(e3) : huge;
    return f2(fminf(t1dA, fminf(t2dA, t3dA)), fminf(t1dB, fminf(t2dB, t3dB)));
}

}  // namespace eikx
