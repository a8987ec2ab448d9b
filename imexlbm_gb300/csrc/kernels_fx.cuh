// Fixed-point float64 engine: declarations.
#pragma once

#include <cuda_runtime.h>

#include "fx_params.hpp"
#include "kernels_f64.cuh"

namespace imex {

cudaError_t launch_step_fx(int mode, const double* src, double* dst, const Geom& g, const FxParams& fx,
                           const CollideF64& cp, unsigned long long* fallback, cudaStream_t s);
// Launch j (1-based) of a run of n >= 2 fused steps whose state is held as
// X on the float64 grid between launches (launch 1 reads float64, launch n
// writes float64).  *fail must be above n before launch 1; it ends as the
// first step whose cell left the exact range (the run's later launches do
// nothing, and the state after step *fail - 1 is in that step's source
// buffer, as X unless *fail is 1).
cudaError_t launch_step_fx_run(const double* src, double* dst, const Geom& g, const FxParams& fx, int j, int n,
                               int* fail, cudaStream_t s);
// Two fused steps in one pass (k_two_fxs): state as X in and out.  The
// control block names the row-ticket counter, the per-row flags of both
// phases (epoch-stamped, never reset), the L2-resident ring of
// two_step_ring_values(g) values, the launch's epoch (> every earlier one),
// the bounded wait in SM clocks and the error flag a wait that runs out sets.
struct TwoStepCtl {
    unsigned* counter;
    int* flag_a;
    int* flag_b;
    unsigned long long* mid;
    int ring;  // recycled x-planes of the ring (R)
    int lag;   // tickets between the first A row and the first B row (two_step_lag)
    int epoch;
    long long cycles;
    unsigned* err;
};
constexpr int kTwoRingMin = 4, kTwoRingMax = 16, kTwoRingDefault = 12;
int two_step_lag(const Geom& g, int ring);
bool two_step_eligible(const Geom& g, int ring);
size_t two_step_ring_values(const Geom& g, int ring);
// Steps j and j + 1 of a fixed-point run (X in, X out; *fail as for
// launch_step_fx_run, set to j if either step leaves the exact range).
cudaError_t launch_two_step_fx(const double* src, double* dst, const Geom& g, const FxParams& fx, const TwoStepCtl& ts,
                               int ctas_per_sm, int j, int* fail, cudaStream_t s);
// X on the float64 grid -> float64, in place, n values.
cudaError_t launch_fx_to_f64(double* buf, size_t n, cudaStream_t s);
struct RowConfig;
// Row-staged fused fixed-point step (rows.cuh); eligible when a row of nz
// float64 is a multiple of 16 bytes and two stages fit in shared memory.
bool rows_fx_eligible(const Geom& g);
cudaError_t launch_rows_fx(const double* src, double* dst, const Geom& g, const FxParams& fx, const CollideF64& cp,
                           unsigned long long* fallback, const RowConfig& rc, unsigned* err, cudaStream_t s);
cudaError_t launch_conserved_fx(bool pull, const double* src, const Geom& g, const FxParams& fx, double* partial,
                                double* out, cudaStream_t s);

}  // namespace imex
