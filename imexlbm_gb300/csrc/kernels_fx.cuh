// Fixed-point float64 engine: declarations.
#pragma once

#include <cuda_runtime.h>

#include "fx_params.hpp"
#include "kernels_f64.cuh"

namespace imex {

cudaError_t launch_step_fx(int mode, const double* src, double* dst, const Geom& g, const FxParams& fx,
                           const CollideF64& cp, unsigned long long* fallback, cudaStream_t s);
struct RowConfig;
// Row-staged fused fixed-point step (rows.cuh); eligible when a row of nz
// float64 is a multiple of 16 bytes and two stages fit in shared memory.
bool rows_fx_eligible(const Geom& g);
cudaError_t launch_rows_fx(const double* src, double* dst, const Geom& g, const FxParams& fx, const CollideF64& cp,
                           unsigned long long* fallback, const RowConfig& rc, unsigned* err, cudaStream_t s);
cudaError_t launch_conserved_fx(bool pull, const double* src, const Geom& g, const FxParams& fx, double* partial,
                                double* out, cudaStream_t s);

}  // namespace imex
