// Native float64 BGK collision of one cell (shared by the native engine and
// the fixed-point engine's exact fallback).
#pragma once

#include "kernels_f64.cuh"

namespace imex {

// ---------------------------------------------------------------- collide --
// BGK collision of one cell, src/lbm.cpp:140-164:
//   p = sum f / 3, u = sum f e, feq_a = w_a (3p + 3 e.u + 4.5 (e.u)^2 - 1.5 u.u),
//   f_a <- f_a - (f_a - feq_a) / (tau0 + 0.5).
// Rewritten per opposite pair (a, a') with c = 3p - 1.5 u.u + 4.5 (e.u)^2:
//   f_a  <- (1 - w) f_a  + (w w_a) c + (3 w w_a) e.u
//   f_a' <- (1 - w) f_a' + (w w_a) c - (3 w w_a) e.u        (w = omega)
__device__ __forceinline__ void collide_f64(double (&f)[kQ], const CollideF64& cp)
{
    double d[kPairs + 1], s[kPairs + 1];
#pragma unroll
    for (int k = 1; k <= kPairs; ++k) {
        d[k] = f[2 * k - 1] - f[2 * k];
        s[k] = f[2 * k - 1] + f[2 * k];
    }
    // 3p = sum of all 27 values (tree order)
    const double S = ((((s[1] + s[2]) + (s[3] + s[4])) + ((s[5] + s[6]) + (s[7] + s[8]))) +
                      (((s[9] + s[10]) + (s[11] + s[12])) + (s[13] + f[0])));
    double u[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int dim = 0; dim < 3; ++dim)
#pragma unroll
        for (int k = 1; k <= kPairs; ++k) {
            const int e = ex(2 * k - 1, dim);
            if (e == 1) u[dim] += d[k];
            if (e == -1) u[dim] -= d[k];
        }
    const double udu = fma(u[2], u[2], fma(u[1], u[1], u[0] * u[0]));
    const double base = fma(-1.5, udu, S);
    const double c1 = cp.one_minus_omega;
    f[0] = fma(c1, f[0], cp.ow[0] * base);
#pragma unroll
    for (int k = 1; k <= kPairs; ++k) {
        const int a = 2 * k - 1;
        const int cls = weight216(a) == 16 ? 1 : weight216(a) == 4 ? 2 : 3;
        double edu = 0.0;
        bool first = true;
#pragma unroll
        for (int dim = 0; dim < 3; ++dim) {
            const int e = ex(a, dim);
            if (e != 0) {
                edu = first ? (e == 1 ? u[dim] : -u[dim]) : (e == 1 ? edu + u[dim] : edu - u[dim]);
                first = false;
            }
        }
        const double c = fma(4.5 * edu, edu, base);
        const double A = cp.ow[cls] * c;
        const double B = cp.tow[cls] * edu;
        f[a] = fma(c1, f[a], A + B);
        f[a + 1] = fma(c1, f[a + 1], A - B);
    }
}

}  // namespace imex
