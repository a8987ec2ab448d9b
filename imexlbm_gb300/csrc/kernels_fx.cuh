// Fixed-point float64 engine: declarations.
#pragma once

#include <cuda_runtime.h>

#include "kernels_f64.cuh"

namespace imex {

// Launch constants of the exact fixed-point collision.
struct FxParams {
    int frac_bits;  // F: a value v is held as the integer round(v * 2^F)
    int pad;
};

// Fill `out` for relaxation time tau0 and density rho0; false when the
// lattice's values cannot be held exactly in 64-bit fixed point (the engine
// is then not used).
bool make_fx_params(double tau0, double rho0, FxParams* out);

cudaError_t launch_step_fx(int mode, const double* src, double* dst, const Geom& g, const FxParams& fx,
                           const CollideF64& cp, unsigned long long* fallback, cudaStream_t s);
cudaError_t launch_conserved_fx(bool pull, const double* src, const Geom& g, const FxParams& fx, double* partial,
                                double* out, cudaStream_t s);

}  // namespace imex
