// Declarations of the native float64 kernels' launchers.
#pragma once

#include <cuda_runtime.h>

#include "kernels_common.cuh"

namespace imex {

// Launch modes of the step kernels.
constexpr int kModeFused = 0;    // dst = C(S(src))
constexpr int kModeCollide = 1;  // dst = C(src)
constexpr int kModeStream = 2;   // dst = S(src)

// Constants of the float64 collision: omega = 1 / (tau0 + 0.5) and the
// per-weight-class products omega * w and 3 * omega * w
// (class 0 rest, 1 axis, 2 face diagonal, 3 corner).
struct CollideF64 {
    double omega, one_minus_omega;
    double ow[4], tow[4];
};

CollideF64 make_collide_f64(double tau0);

// out[0] = max |a - b|, out[1] = max |b| over 3 arrays of n values each
// (component-major), as float64 bit patterns.
cudaError_t launch_maxdiff3(const double* a, const double* b, size_t n, unsigned long long* out, cudaStream_t s);

size_t conserved_partials(const Geom& g);

cudaError_t launch_init_f64(double* f, const Geom& g, const double* tx, const double* ty, const double* tz, double rho0,
                            double u0, cudaStream_t s);
cudaError_t launch_step_f64(int mode, const double* src, double* dst, const Geom& g, const CollideF64& cp, cudaStream_t s);
cudaError_t launch_reduce_partials(const double* partial, size_t n, double* out, cudaStream_t s);
cudaError_t launch_conserved_f64(bool pull, const double* src, const Geom& g, double* partial, double* out, cudaStream_t s);
cudaError_t launch_macro_f64(bool pull, const double* src, const Geom& g, double* p, double* u, double* v, double* w,
                             cudaStream_t s);

}  // namespace imex
