// Internal layout of a lattice handle (struct imex_lattice of the C ABI),
// shared by the translation units that drive its buffers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "kernels_f64.cuh"
#include "kernels_fx.cuh"
#include "kernels_lowp.cuh"
#include "phase_timer.hpp"
#include "rows.cuh"

using imex::CollideF32;
using imex::CollideF64;
using imex::FxParams;
using imex::Geom;
using imex::RowConfig;

// kExact: the device buffer is the reference's f.  kPendingStream: the
// reference's f is S(buffer) (the last streaming is not applied yet).
enum Tag { kUninit = 0, kExact = 1, kPendingStream = 2 };

struct imex_lattice {
    Geom g{};
    size_t ncells = 0;
    double tau0 = 0, rho0 = 0, u0 = 0;
    int precision = IMEX_F64;
    int engine = IMEX_ENGINE_AUTO;
    void* buf[2] = {nullptr, nullptr};
    int cur = 0;
    Tag tag = kUninit;
    int64_t steps = 0;
    int64_t launches = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    int device = 0;
    unsigned char* scratch = nullptr;  // one allocation holding d_partial .. d_fail
    double* d_partial = nullptr;  // conserved partials (5 per block)
    double* d_out = nullptr;      // 5 reduced values
    unsigned long long* d_fallback = nullptr;  // fixed-point engine fallback counter
    size_t bytes = 0;
    CollideF64 cf64{};
    CollideF32 cf32{};
    FxParams fx{};
    bool fx_ok = false;  // fixed-point engine usable for this lattice
    unsigned* d_err = nullptr;  // set by kernels whose bounded waits ran out
    int* d_fail = nullptr;      // first failing step of a fixed-point run (imex_step)
    int64_t fx_reruns = 0;      // fixed-point runs redone from a failing step
    int fx_skip = 0;            // imex_step calls left that step one at a time after a failed run
    // two fused steps per launch (launch_two_step_fx): ticket counter, row
    // flags of both phases and the L2-resident ring, allocated on first use
    unsigned char* two_mem = nullptr;
    int two_ring = 0;        // ring depth two_mem holds
    size_t two_bytes = 0;
    imex::TwoStepCtl two{};
    int two_epoch = 0;
    int fx_backoff = 0;         // calls skipped after the last failure (doubles per failure, up to 64)
    RowConfig rows{};           // launch shape of the fused step (stages 0: one thread per cell)
    int shape_mode = -1;        // -1 autotune on first use, 0 one thread per cell, 1 row-staged
    bool shape_pinned = false;  // shape set by imex_set_launch rather than the autotuner
    imex::PhaseTimer prof;      // per-phase device time (imex_profile_*)
    std::string err;
};

namespace imex {

// Both defined in lattice.cu.
int lattice_fail(imex_lattice* h, int code, const std::string& msg);
size_t lattice_elem_size(int precision);

}  // namespace imex
