// Reduced-precision storage: float32 distributions (IMEX_F32) and float16
// deviations from the lattice weights, 2^12 (f - w) (IMEX_F16DEV).  Both
// collide in float32; diagnostics accumulate in float64.
//
// The float32 collision works in deviation space for both formats: with
// h_a = f_a - w_a (exact in float32 for f_a in [w_a / 2, 2 w_a]), sum h = 3p - 1,
// sum h e = u (sum w e = 0), and the equilibrium deviation is
//   heq_a = w_a (sum h + 3 e.u + 4.5 (e.u)^2 - 1.5 u.u)
// (src/lbm.cpp:153-162 with w_a subtracted).  The moments then come from
// O(0.01) numbers instead of O(0.1) ones.
//
// Relaxation.  The reference's f - (f - feq) omega with omega = 1/(tau0+0.5)
// (src/lbm.cpp:133,163) is written as
//   h <- 2 heq - h + eps (h - heq),   eps = 2 - omega = 2 tau0 / (tau0 + 0.5)
// because omega is close to 2 at the Reynolds numbers of interest: a
// float32 omega carries a 6e-8 absolute error, which is a 6e-5 relative
// error in the viscosity at tau0 = 5e-4 and makes the kinetic energy decay
// at the wrong rate.  eps itself is exact to 6e-8 relative, and so is the
// viscosity.
//
// Momentum.  Opposite directions get heq = A +- B with B = b_a (e.u): the
// equilibrium's momentum is sum over pairs of 2 b_a (e_a.u) e_a, which is u
// only if 2 (b_axis + 4 b_face + 4 b_corner) = 1 holds exactly.  With each
// b = 3 w rounded to float32 separately it is off by ~1e-8, every collision
// then scales the momentum by (1 + 2e-8), and the kinetic energy drifts by
// ~3e-8 per step (2e-4 after 5000 steps).  The b are therefore chosen on
// binary grids where b_axis = 1/2 - 4 b_face - 4 b_corner is exact; the
// drift falls to rounding noise (~1e-8 after 200 steps at 32^3).
#pragma once

#include <cuda_fp16.h>

#include "d3q27.cuh"
#include "imexlbm.h"
#include "kernels_lowp.cuh"

namespace imex {
namespace lowp {

template <int P>
struct Storage;

// 32-bit hash of (cell index, step seed) for stochastic rounding: the
// murmur3 finaliser of their combination.
__device__ __forceinline__ uint32_t sr_hash(unsigned long long idx, uint32_t seed)
{
    uint32_t x = (uint32_t)idx ^ ((uint32_t)(idx >> 32) * 0x9E3779B9u) ^ (seed * 0x85EBCA6Bu);
    x ^= x >> 16;
    x *= 0x85EBCA6Bu;
    x ^= x >> 13;
    x *= 0xC2B2AE35u;
    x ^= x >> 16;
    return x;
}

// Random bits of the stochastic rounding, shared by every kernel so that a
// lattice's result does not depend on which kernel stepped it: cells 2p and
// 2p + 1 of a lattice (flat index, z fastest) share the 32-bit word
// sr_word(hash(p, step), a) = hash + a * phi for direction a (phi = 2^32 /
// golden ratio, a Weyl sequence: each word uniform because the hash is;
// across a pair's directions the draws are stratified rather than
// independent).  Cell 2p takes bits 0..12 and cell 2p + 1 bits 16..28 -
// the operand layout of cvt.rs.f16x2.f32 with cell 2p in the low half.
__device__ __forceinline__ uint32_t sr_word(uint32_t pair_hash, int a) { return pair_hash + (uint32_t)a * 0x9E3779B9u; }

// Store 27 float16 deviations of one cell, converting two at a time
// (values already on the float16 grid convert exactly).
template <class Dst>
__device__ __forceinline__ void store_f16_cell(const float (&y)[kQ], Dst&& at)
{
#pragma unroll
    for (int a = 0; a + 1 < kQ; a += 2) {
        const __half2 v = __floats2half2_rn(y[a], y[a + 1]);
        at(a) = __low2half(v);
        at(a + 1) = __high2half(v);
    }
    at(kQ - 1) = __float2half_rn(y[kQ - 1]);
}

// Stochastic rounding of a float32 pair to float16 in one instruction
// (cvt.rs.f16x2.f32 of the sm_100 family).  Each value moves to one of its
// two float16 neighbours, up (in magnitude) with probability equal to its
// distance from the lower one in units of their gap, resolved to 13 bits:
// the value's dropped bits plus 13 random bits, carried into the kept part.
// `hi` (upper half of the result) takes random bits 16..28 of `rbits`, `lo`
// bits 0..12.  A normal float16 result (|x| >= 2^-14) drops exactly 13 bits,
// so the expected stored value is x exactly; for subnormal results the
// probability is truncated to a multiple of 2^-13, a bias toward zero below
// 2^-37 per value.
__device__ __forceinline__ uint32_t cvt_rs_f16x2(float hi, float lo, uint32_t rbits)
{
    uint32_t d;
    asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
    return d;
}

// Store 27 float16 deviations of one cell with stochastic rounding: the
// cell's half of its pair's random words (see sr_word).
template <class Dst>
__device__ __forceinline__ void store_f16_cell_sr(const float (&y)[kQ], unsigned long long cell, uint32_t seed,
                                                  Dst&& at)
{
    const uint32_t ph = sr_hash(cell >> 1, seed);
    const bool odd = cell & 1;
#pragma unroll
    for (int a = 0; a < kQ; ++a) {
        const uint32_t w = sr_word(ph, a);
        const uint32_t d = odd ? cvt_rs_f16x2(y[a], 0.0f, w) >> 16 : cvt_rs_f16x2(0.0f, y[a], w) & 0xffffu;
        at(a) = __ushort_as_half((unsigned short)d);
    }
}

// kScale: the collision works on kScale * (f - w).  float32 storage keeps f
// itself (kScale 1); float16 storage keeps (f - w) * 2^12, so that
// deviations down to 2^-26 (rather than 2^-14) are normal float16 numbers
// with the full 11-bit significand - deviations of populations whose e.u is
// near zero are of order w u^2, below 2^-14 at u ~ 0.01.  The largest
// storable deviation, 65504 / 2^12 = 16, is far above any f - w of a
// physical state (|f - w| < 1).
template <>
struct Storage<IMEX_F32> {
    using T = float;
    static constexpr float kScale = 1.0f;
    static __device__ __forceinline__ float load(const float* p, int a)
    {
        return __ldg(p) - (float)weight(a);
    }
    static __device__ __forceinline__ float load_plain(const float* p, int a) { return *p - (float)weight(a); }
    static __device__ __forceinline__ float dev(float v, int a) { return v - (float)weight(a); }
    static __device__ __forceinline__ float store(float h, int a) { return (float)weight(a) + h; }
    static __device__ __forceinline__ double to_f64(float v, int) { return (double)v; }
    static __device__ __forceinline__ float from_f64(double f, int) { return __double2float_rn(f); }
};

template <>
struct Storage<IMEX_F16DEV> {
    using T = __half;
    static constexpr float kScale = 4096.0f;
    static __device__ __forceinline__ float load(const __half* p, int) { return __half2float(__ldg(p)); }
    static __device__ __forceinline__ float load_plain(const __half* p, int) { return __half2float(*p); }
    static __device__ __forceinline__ float dev(__half v, int) { return __half2float(v); }
    static __device__ __forceinline__ __half store(float h, int) { return __float2half_rn(h); }
    static __device__ __forceinline__ double to_f64(__half v, int a)
    {
        return weight(a) + (double)__half2float(v) * (1.0 / kScale);
    }
    static __device__ __forceinline__ __half from_f64(double f, int a)
    {
        return __float2half_rn((float)((f - weight(a)) * kScale));
    }
};

// Arithmetic of one float32 lane (float) or of two cells in lock step
// (float2, the packed f32x2 instructions of the sm_100 family).  The packed
// operations are two independent IEEE operations each, so a float2 lane
// gives exactly the bits the float code gives for that cell.  The float
// operations are the _rn intrinsics, which the compiler never contracts
// into a fused multiply-add (as it may contract a * b + c), so every
// product and sum rounds exactly where the code says.
struct F1 {
    using V = float;
    static __device__ __forceinline__ V splat(float x) { return x; }
    static __device__ __forceinline__ V add(V a, V b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ V sub(V a, V b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ V mul(V a, V b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ V fma(V a, V b, V c) { return __fmaf_rn(a, b, c); }
};
struct F2 {
    using V = float2;
    static __device__ __forceinline__ V splat(float x) { return make_float2(x, x); }
    static __device__ __forceinline__ V add(V a, V b) { return __fadd2_rn(a, b); }
    // a - b rounded once: b * (-1) is exact, so the fused form rounds a - b
    static __device__ __forceinline__ V sub(V a, V b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
    static __device__ __forceinline__ V mul(V a, V b) { return __fmul2_rn(a, b); }
    static __device__ __forceinline__ V fma(V a, V b, V c) { return __ffma2_rn(a, b, c); }
};

// float32 BGK collision of the deviations h = kScale (f - w) (see the file
// header), for one cell (A = F1) or two (A = F2).  Moments and the
// relaxation are linear in h; only the quadratic terms of the equilibrium
// carry 1 / kScale, folded into their constants.  kScale is a power of two,
// so every intermediate is exactly kScale^k times the unscaled one and the
// result is exactly kScale times the unscaled collision's: both storage
// formats run the same float32 arithmetic.  2 heq - h is formed as
// (heq + heq) - h: heq + heq is exact, so it rounds like fma(2, heq, -h).
template <int P, class A>
__device__ __forceinline__ void collide_dev(typename A::V (&h)[kQ], const CollideF32& cp)
{
    using V = typename A::V;
    constexpr float c15 = -1.5f / Storage<P>::kScale, c45 = 4.5f / Storage<P>::kScale;
    V d[kPairs + 1], s[kPairs + 1];
#pragma unroll
    for (int k = 1; k <= kPairs; ++k) {
        d[k] = A::sub(h[2 * k - 1], h[2 * k]);
        s[k] = A::add(h[2 * k - 1], h[2 * k]);
    }
    const V sig = A::add(A::add(A::add(A::add(s[1], s[2]), A::add(s[3], s[4])), A::add(A::add(s[5], s[6]), A::add(s[7], s[8]))),
                         A::add(A::add(A::add(s[9], s[10]), A::add(s[11], s[12])), A::add(s[13], h[0])));
    V u[3];
#pragma unroll
    for (int dim = 0; dim < 3; ++dim) {
        bool first = true;
#pragma unroll
        for (int k = 1; k <= kPairs; ++k) {
            const int e = ex(2 * k - 1, dim);
            if (e == 0) continue;
            // 0 + d and 0 - d are exact: the first term starts the sum
            if (first) u[dim] = e == 1 ? d[k] : A::sub(A::splat(0.f), d[k]);
            else u[dim] = e == 1 ? A::add(u[dim], d[k]) : A::sub(u[dim], d[k]);
            first = false;
        }
    }
    const V udu = A::fma(u[2], u[2], A::fma(u[1], u[1], A::mul(u[0], u[0])));
    const V base = A::fma(A::splat(c15), udu, sig);
    const V eps = A::splat(cp.eps);
    {
        const V heq = A::mul(A::splat(cp.w[0]), base);
        h[0] = A::fma(eps, A::sub(h[0], heq), A::sub(A::add(heq, heq), h[0]));
    }
#pragma unroll
    for (int k = 1; k <= kPairs; ++k) {
        const int a = 2 * k - 1;
        const int cls = weight216(a) == 16 ? 1 : weight216(a) == 4 ? 2 : 3;
        V edu;
        bool first = true;
#pragma unroll
        for (int dim = 0; dim < 3; ++dim) {
            const int e = ex(a, dim);
            if (e != 0) {
                edu = first ? (e == 1 ? u[dim] : A::sub(A::splat(0.f), u[dim]))
                            : (e == 1 ? A::add(edu, u[dim]) : A::sub(edu, u[dim]));
                first = false;
            }
        }
        const V Aq = A::mul(A::splat(cp.w[cls]), A::fma(A::mul(A::splat(c45), edu), edu, base));
        const V Bq = A::mul(A::splat(cp.w3[cls]), edu);
        const V ep = A::add(Aq, Bq), em = A::sub(Aq, Bq);
        h[a] = A::fma(eps, A::sub(h[a], ep), A::sub(A::add(ep, ep), h[a]));
        h[a + 1] = A::fma(eps, A::sub(h[a + 1], em), A::sub(A::add(em, em), h[a + 1]));
    }
}

template <int P>
__device__ __forceinline__ void collide_dev_f32(float (&h)[kQ], const CollideF32& cp)
{
    collide_dev<P, F1>(h, cp);
}

}  // namespace lowp
}  // namespace imex
