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
// sr_word(hash(p, step), ., a) = hash + a * phi for direction a (phi = 2^32 /
// golden ratio, a Weyl sequence: each word uniform because the hash is;
// across a pair's directions the draws are stratified rather than
// independent).  Cell 2p takes bits 0..12 and cell 2p + 1 bits 16..28 -
// the operand layout of cvt.rs.f16x2.f32 with cell 2p in the low half.
//
// The eight corner populations (directions kFirstCorner..26) absorb the
// other populations' rounding errors before they are rounded themselves
// (round_f16_conserving).  A corner's draw must then be independent of the
// others' draws: the low bits of hash + a * phi are a function of the low
// bits of the hash alone, and a corner draw tied to the draws that set its
// correction would round it up more often than its value asks (a kinetic-
// energy drift of ~4e-6 per 1000 steps at 512^3).  The corners therefore
// draw from a second word of the pair, sr_corner_hash(hash), a full mix of
// all 32 bits.
constexpr int kFirstCorner = 2 * 10 - 1;  // pairs 10..13 are the corners (d3q27.cuh)

__device__ __forceinline__ uint32_t sr_corner_hash(uint32_t pair_hash)
{
    uint32_t x = pair_hash ^ 0x5BD1E995u;
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}

__device__ __forceinline__ uint32_t sr_word(uint32_t pair_hash, uint32_t corner_hash, int a)
{
    return (a >= kFirstCorner ? corner_hash : pair_hash) + (uint32_t)a * 0x9E3779B9u;
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
// formats run the same float32 arithmetic.
//
// Per population, with t = h - heq: h <- heq - t + eps t, formed as
// fma(eps, t, heq - t) - three operations, each rounding below the
// population's own size (t, the non-equilibrium part, is small).  With
// float32 storage the rest population is sum h minus the 26 others' results
// (see the end).  The
// equilibrium of an opposite pair is A +- B with A = w (4.5 (e.u)^2 / kScale
// + base) = (w 4.5 / kScale) (e.u)^2 + w base and B = b (e.u), each side one
// fused multiply-add: fma(+-b, e.u, A).
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
    // w base for the four weight classes (rest, axis, face diagonal, corner)
    const V wb[4] = {A::mul(A::splat(cp.w[0]), base), A::mul(A::splat(cp.w[1]), base),
                     A::mul(A::splat(cp.w[2]), base), A::mul(A::splat(cp.w[3]), base)};
    constexpr bool kRestTakesMass = P == IMEX_F32;
    if constexpr (!kRestTakesMass) {
        const V t = A::sub(h[0], wb[0]);
        h[0] = A::fma(eps, t, A::sub(wb[0], t));
    }
    V ps[kPairs + 1];  // the pairs' relaxed sums, for the rest population
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
        const V Aq = A::fma(A::mul(A::splat(cp.w[cls] * c45), edu), edu, wb[cls]);
        const V ep = A::fma(A::splat(cp.w3[cls]), edu, Aq), em = A::fma(A::splat(-cp.w3[cls]), edu, Aq);
        const V tp = A::sub(h[a], ep), tm = A::sub(h[a + 1], em);
        h[a] = A::fma(eps, tp, A::sub(ep, tp));
        h[a + 1] = A::fma(eps, tm, A::sub(em, tm));
        if constexpr (kRestTakesMass) ps[k] = A::add(h[a], h[a + 1]);
    }
    // float32 storage: the rest population takes what the mass leaves, sig
    // minus the other 26 relaxed values.  In exact arithmetic that is its BGK
    // value; in float32 it also absorbs the other populations' rounding, so
    // the collision keeps each cell's mass to the rounding of these sums (the
    // drift of the total mass over 2000 steps at 512^3 fell from 7.4e-8 to
    // 4.5e-10).  Float16-deviation storage keeps the BGK form: there the 25
    // more operations cost 3% of the step (the FMA pipe is half busy), and
    // its own stochastic rounding sets the mass drift.
    if constexpr (kRestTakesMass) {
        const V m = A::add(A::add(A::add(A::add(ps[1], ps[2]), A::add(ps[3], ps[4])),
                                  A::add(A::add(ps[5], ps[6]), A::add(ps[7], ps[8]))),
                           A::add(A::add(A::add(ps[9], ps[10]), A::add(ps[11], ps[12])), ps[13]));
        h[0] = A::sub(sig, m);
    }
}

template <int P>
__device__ __forceinline__ void collide_dev_f32(float (&h)[kQ], const CollideF32& cp)
{
    collide_dev<P, F1>(h, cp);
}

// float(r) - v for a float16 r and a float32 v in one instruction (the
// mixed-precision sub.f32.f16 of the sm_100 family: r widens exactly, then
// one rounding, as in __fsub_rn(__half2float(r), v)).
__device__ __forceinline__ float sub_f16_f32(__half r, float v)
{
    float d;
    asm("sub.rn.f32.f16 %0, %1, %2;" : "=f"(d) : "h"(__half_as_ushort(r)), "f"(v));
    return d;
}

// Rounding of one cell's (A = F1) or two cells' (A = F2) 27 float32
// deviations to float16 that keeps each cell's momentum.
//
// A float16 step of an axis or face-diagonal population is 4 to 16 times
// that of a corner population (the deviations scale with the weights 2/27,
// 1/54, 1/216).  Rounding every value on its own leaves a momentum error of
// the order of an axis population's step in every cell and every step; that
// noise drives the flow, and on coarse lattices over a few thousand steps
// it moved the kinetic energy by up to 2.4e-4 from the float64 result.
// Here the 19 rest, axis and face-diagonal populations are rounded first
// and the momentum of their rounding errors is summed, p = sum e_a (r_a -
// y_a).  The eight corner populations s = (+-1, +-1, +-1) absorb it before
// they are rounded: each moves by -s.p / 8, and since the corners' s sum to
// 0 and their s s^T to 8 I, the moves take p out of the momentum exactly and
// leave the mass alone.  What remains is the corners' own rounding, 4 to 16
// times smaller.  The moves are a few float16 steps of a corner population;
// under stochastic rounding the errors they undo have zero mean and the
// corners draw independent random bits (sr_corner_hash), so the corners
// stay unbiased.  (Taking the mass error into the corners as well, by
// -(m + s.p) / 8, cost 3% of the step and did not lower the kinetic-energy
// error further.)
//
// `rnd(a, v)` rounds v (for direction a) to float16, stores it, and returns
// the rounding error r - v (exact: r and v are within a float16 step of
// each other).  The sums use A's operations in a fixed order, so one-cell
// and two-cell kernels store the same bits.
template <class A, class Rnd>
__device__ __forceinline__ void round_f16_conserving(const typename A::V (&y)[kQ], Rnd&& rnd)
{
    using V = typename A::V;
    // D_k = r_a - y_a - (r_b - y_b) for the 9 non-corner pairs (a, b) =
    // (2k - 1, 2k): the pair's momentum error along e_a.  The rest
    // population carries no momentum.
    V D[10];
    rnd(0, y[0]);
#pragma unroll
    for (int k = 1; k < 10; ++k) {
        const V da = rnd(2 * k - 1, y[2 * k - 1]);
        const V db = rnd(2 * k, y[2 * k]);
        D[k] = A::sub(da, db);
    }
    // p[dim] = sum over the five pairs moving along dim of e_dim D_k, the
    // axis pair (e_dim = +1) first
    V p[3];
#pragma unroll
    for (int dim = 0; dim < 3; ++dim) {
        V acc = D[dim + 1];
#pragma unroll
        for (int k = 4; k < 10; ++k) {
            const int e = ex(2 * k - 1, dim);
            if (e == 1) acc = A::add(acc, D[k]);
            else if (e == -1) acc = A::sub(acc, D[k]);
        }
        p[dim] = acc;
    }
    const V neg8 = A::splat(-0.125f);
#pragma unroll
    for (int a = kFirstCorner; a < kQ; a += 2) {
        // s.p for the pair's first member s; the opposite member has -s.p
        const V sx = ex(a, 0) == 1 ? p[0] : A::sub(A::splat(0.f), p[0]);
        const V sxy = ex(a, 1) == 1 ? A::add(sx, p[1]) : A::sub(sx, p[1]);
        const V sp = ex(a, 2) == 1 ? A::add(sxy, p[2]) : A::sub(sxy, p[2]);
        rnd(a, A::fma(neg8, sp, y[a]));
        rnd(a + 1, A::fma(neg8, A::sub(A::splat(0.f), sp), y[a + 1]));
    }
}

// Store the 27 float16 deviations of one cell (flat index `cell`), rounded
// to nearest or stochastically (the cell's half of its pair's random words,
// see sr_word), through round_f16_conserving.
template <class Dst>
__device__ __forceinline__ void store_f16_cell(const float (&y)[kQ], bool sr, unsigned long long cell, uint32_t seed,
                                               Dst&& at)
{
    if (sr) {
        const uint32_t ph = sr_hash(cell >> 1, seed), pc = sr_corner_hash(ph);
        const bool odd = cell & 1;
        round_f16_conserving<F1>(y, [&](int a, float v) -> float {
            const uint32_t w = sr_word(ph, pc, a);
            const uint32_t d = odd ? cvt_rs_f16x2(v, 0.0f, w) >> 16 : cvt_rs_f16x2(0.0f, v, w) & 0xffffu;
            const __half r = __ushort_as_half((unsigned short)d);
            at(a) = r;
            return sub_f16_f32(r, v);
        });
    } else {
        round_f16_conserving<F1>(y, [&](int a, float v) -> float {
            const __half r = __float2half_rn(v);
            at(a) = r;
            return sub_f16_f32(r, v);
        });
    }
}

}  // namespace lowp
}  // namespace imex
