// Taylor-Green initial field and its equilibrium distributions for one cell,
// src/lbm.cpp:78-108.  The trigonometric factors depend on one coordinate
// each and come in as per-axis tables t[3 i + {0, 1, 2}] = sin, cos, cos 2x
// of x = (double)i / (double)n * 2.0 * 3.1415926, computed on the host with
// that expression.  Products and sums use round-to-nearest intrinsics in the
// reference's order, so no FMA contraction changes its rounding.
#pragma once

#include "d3q27.cuh"

namespace imex {

__device__ __forceinline__ void tg_init_cell(double (&fe)[kQ], const double* __restrict__ tx,
                                             const double* __restrict__ ty, const double* __restrict__ tz, int i,
                                             int j, int k, double rho0, double u0)
{
    const double sx = tx[3 * i], cx = tx[3 * i + 1], c2x = tx[3 * i + 2];
    const double sy = ty[3 * j], cy = ty[3 * j + 1], c2y = ty[3 * j + 2];
    const double cz = tz[3 * k + 1], c2z = tz[3 * k + 2];
    const double cs2 = 1.0 / 3.0;
    const double u = __dmul_rn(__dmul_rn(__dmul_rn(u0, sx), cy), cz);
    const double v = __dmul_rn(__dmul_rn(__dmul_rn(-u0, cx), sy), cz);
    const double w = 0.0;
    const double amp = __ddiv_rn(__dmul_rn(__dmul_rn(rho0, u0), u0), 16.0);
    const double p = __dadd_rn(__dmul_rn(rho0, cs2), __dmul_rn(__dmul_rn(amp, __dadd_rn(c2x, c2y)), __dadd_rn(c2z, 2.0)));
    const double udu = __dadd_rn(__dadd_rn(__dmul_rn(u, u), __dmul_rn(v, v)), __dmul_rn(w, w));
#pragma unroll
    for (int a = 0; a < kQ; ++a) {
        // e(a,0)*u + e(a,1)*v + e(a,2)*w with integer e, as written
        const double edu = __dadd_rn(__dadd_rn(__dmul_rn((double)ex(a, 0), u), __dmul_rn((double)ex(a, 1), v)),
                                     __dmul_rn((double)ex(a, 2), w));
        const double br = __dsub_rn(__dadd_rn(__dadd_rn(__dmul_rn(3.0, p), __dmul_rn(3.0, edu)),
                                              __dmul_rn(__dmul_rn(4.5, edu), edu)),
                                    __dmul_rn(1.5, udu));
        fe[a] = __dmul_rn(weight(a), br);
    }
}

}  // namespace imex
