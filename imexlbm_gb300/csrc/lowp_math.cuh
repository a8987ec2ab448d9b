// Reduced-precision storage: float32 distributions (IMEX_F32) and float16
// deviations from the lattice weights, h = f - w (IMEX_F16DEV).  Both
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

// Random bits for direction a of a cell: the Weyl sequence r0 + a * phi
// (mod 2^32, phi = 2^32 / golden ratio) from the cell's hash r0.  Each value
// is uniform because r0 is; across the 27 directions the draws are
// stratified rather than independent, which if anything lowers the
// variance of the cell's summed rounding error.
__device__ __forceinline__ uint32_t sr_bits(uint32_t cell_hash, int a) { return cell_hash + (uint32_t)a * 0x9E3779B9u; }

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

template <>
struct Storage<IMEX_F32> {
    using T = float;
    static __device__ __forceinline__ float load(const float* p, int a)
    {
        return __ldg(p) - (float)weight(a);
    }
    static __device__ __forceinline__ float load_plain(const float* p, int a) { return *p - (float)weight(a); }
    static __device__ __forceinline__ float store(float h, int a) { return (float)weight(a) + h; }
    static __device__ __forceinline__ double to_f64(float v, int) { return (double)v; }
    static __device__ __forceinline__ float from_f64(double f, int) { return __double2float_rn(f); }
};

template <>
struct Storage<IMEX_F16DEV> {
    using T = __half;
    static __device__ __forceinline__ float load(const __half* p, int) { return __half2float(__ldg(p)); }
    static __device__ __forceinline__ float load_plain(const __half* p, int) { return __half2float(*p); }
    static __device__ __forceinline__ __half store(float h, int) { return __float2half_rn(h); }
    static __device__ __forceinline__ double to_f64(__half v, int a) { return weight(a) + (double)__half2float(v); }
    // Stochastic rounding to float16, as float32 bits: h moved up or down to
    // a neighbouring float16 value with probabilities that make the expected
    // result exactly h.  `bits` is a uniform 32-bit random number.  Adding
    // `drop` random bits below the float16 precision of |h| and clearing
    // them rounds the magnitude up with probability (dropped part) / 2^drop;
    // a carry into the exponent lands on the next float16 value, the correct
    // upper neighbour.  drop = 13 in the normal float16 range (|h| >= 2^-14)
    // and one more per binade below (float16 subnormals are 2^-24 apart),
    // up to the 23 float32 mantissa bits.  The result is exactly
    // representable in float16, so any rounding conversion stores it as is.
    static __device__ __forceinline__ float round_sr(float h, uint32_t bits)
    {
        const uint32_t x = __float_as_uint(h);
        const int e = (int)((x >> 23) & 0xffu);
        const uint32_t mask = (1u << min(max(126 - e, 13), 23)) - 1u;
        return __uint_as_float((x + (bits & mask)) & ~mask);  // |h| < 65504: no carry into the sign
    }
    static __device__ __forceinline__ __half from_f64(double f, int a) { return __float2half_rn((float)(f - weight(a))); }
};

// float32 BGK collision of the deviations h (see the file header).
__device__ __forceinline__ void collide_dev_f32(float (&h)[kQ], const CollideF32& cp)
{
    float d[kPairs + 1], s[kPairs + 1];
#pragma unroll
    for (int k = 1; k <= kPairs; ++k) {
        d[k] = h[2 * k - 1] - h[2 * k];
        s[k] = h[2 * k - 1] + h[2 * k];
    }
    const float sig = ((((s[1] + s[2]) + (s[3] + s[4])) + ((s[5] + s[6]) + (s[7] + s[8]))) +
                       (((s[9] + s[10]) + (s[11] + s[12])) + (s[13] + h[0])));
    float u[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int dim = 0; dim < 3; ++dim)
#pragma unroll
        for (int k = 1; k <= kPairs; ++k) {
            const int e = ex(2 * k - 1, dim);
            if (e == 1) u[dim] += d[k];
            if (e == -1) u[dim] -= d[k];
        }
    const float udu = fmaf(u[2], u[2], fmaf(u[1], u[1], u[0] * u[0]));
    const float base = fmaf(-1.5f, udu, sig);
    const float eps = cp.eps;
    {
        const float heq = cp.w[0] * base;
        h[0] = fmaf(eps, h[0] - heq, fmaf(2.f, heq, -h[0]));
    }
#pragma unroll
    for (int k = 1; k <= kPairs; ++k) {
        const int a = 2 * k - 1;
        const int cls = weight216(a) == 16 ? 1 : weight216(a) == 4 ? 2 : 3;
        float edu = 0.f;
        bool first = true;
#pragma unroll
        for (int dim = 0; dim < 3; ++dim) {
            const int e = ex(a, dim);
            if (e != 0) {
                edu = first ? (e == 1 ? u[dim] : -u[dim]) : (e == 1 ? edu + u[dim] : edu - u[dim]);
                first = false;
            }
        }
        const float A = cp.w[cls] * fmaf(4.5f * edu, edu, base);
        const float B = cp.w3[cls] * edu;
        const float ep = A + B, em = A - B;
        h[a] = fmaf(eps, h[a] - ep, fmaf(2.f, ep, -h[a]));
        h[a + 1] = fmaf(eps, h[a + 1] - em, fmaf(2.f, em, -h[a + 1]));
    }
}

}  // namespace lowp
}  // namespace imex
