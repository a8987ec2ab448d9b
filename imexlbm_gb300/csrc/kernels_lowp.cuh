// Reduced-precision storage kernels (IMEX_F32, IMEX_F16DEV): declarations.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "imexlbm.h"
#include "kernels_f64.cuh"

namespace imex {

// float32 collision constants: eps = 2 - omega, and per weight class (0
// rest, 1 axis, 2 face diagonal, 3 corner) the weight w and the e.u
// coefficient w3 ~ 3 w (chosen so the momentum identity is exact).
struct CollideF32 {
    float eps;
    float w[4], w3[4];
    int sr;         // float16 storage: 1 stochastic rounding, 0 round to nearest
    uint32_t seed;  // stochastic-rounding seed of this step
};

CollideF32 make_collide_f32(double tau0);

struct RowConfig;
// Largest bytes per direction in a stage of the reduced-precision row kernel.
constexpr int kRowsLowpDirMax = 4096;
bool rows_lowp_eligible(int prec, const Geom& g);
size_t rows_lowp_stage_bytes(int prec, int nz);
cudaError_t launch_rows_lowp(int prec, const void* src, void* dst, const Geom& g, const CollideF32& cp,
                             const RowConfig& rc, unsigned* err, cudaStream_t s);
cudaError_t launch_init_lowp(int prec, void* f, const Geom& g, const double* tx, const double* ty, const double* tz,
                             double rho0, double u0, cudaStream_t s);
cudaError_t launch_step_lowp(int prec, int mode, const void* src, void* dst, const Geom& g, const CollideF32& cp,
                             cudaStream_t s);
// float64 reference-order f -> storage
cudaError_t launch_from_f64(int prec, const double* f, void* out, const Geom& g, cudaStream_t s);
// storage -> float64 reference-order f (pulled through streaming when `pull`)
cudaError_t launch_to_f64(int prec, bool pull, const void* src, const Geom& g, double* out, cudaStream_t s);
cudaError_t launch_macro_lowp(int prec, bool pull, const void* src, const Geom& g, double* p, double* u, double* v,
                              double* w, cudaStream_t s);
cudaError_t launch_conserved_lowp(int prec, bool pull, const void* src, const Geom& g, double* partial, double* out,
                                  cudaStream_t s);

}  // namespace imex
