// Host-side parameters of the fixed-point float64 engine.
#pragma once

#include "fx_math.cuh"

namespace imex {

struct FxParams {
    FxConst k;
    bool om_ge1;    // omega >= 1: the (1 - omega) f term is subtracted
    int frac_bits;  // a value v is held as the integer v * 2^frac_bits
};

// Fill `out` for relaxation time tau0 and density rho0; false when the
// lattice's values cannot be held exactly in 64-bit fixed point (the engine
// is then not used).
bool make_fx_params(double tau0, double rho0, FxParams* out);

}  // namespace imex
