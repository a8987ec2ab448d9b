// Host-side constants of the fixed-point float64 engine (see fx_math.cuh).
#include <cmath>
#include <cstdint>

#include "fx_params.hpp"

namespace imex {

namespace {

// Exact product of two doubles times 2^64, rounded to nearest, for
// products in [0, 1).
uint64_t fixed64_of_product(double a, double b, int mult)
{
    int ea, eb;
    const double fa = std::frexp(a, &ea), fb = std::frexp(b, &eb);
    const unsigned __int128 ma = (unsigned __int128)(uint64_t)std::ldexp(fa, 53);
    const unsigned __int128 mb = (unsigned __int128)(uint64_t)std::ldexp(fb, 53);
    const unsigned __int128 p = ma * mb * (unsigned)mult;   // value = p * 2^(ea + eb - 106)
    const int sh = 106 - 64 - ea - eb;                       // value * 2^64 = p >> sh
    if (sh <= 0 || sh >= 127) return 0;
    const unsigned __int128 r = (p + ((unsigned __int128)1 << (sh - 1))) >> sh;
    return r >> 64 ? 0 : (uint64_t)r;
}

}  // namespace

bool make_fx_params(double tau0, double rho0, FxParams* out)
{
    *out = FxParams{};
    const double omega = 1.0 / (tau0 + 0.5);   // src/lbm.cpp:133
    // The exact range is laid out for rho0 ~ 1 (3p ~ 1); other densities
    // and omega outside (2^-10, 2) use the native float64 engine.
    if (!(rho0 >= 0.75 && rho0 <= 1.25) || !(omega > 0x1p-10 && omega < 2.0)) return false;
    const double w[4] = {8.0 / 27.0, 2.0 / 27.0, 1.0 / 54.0, 1.0 / 216.0};  // src/lbm.cpp:10-17
    for (int cl = 0; cl < 4; ++cl) {
        out->k.c_ow[cl] = fixed64_of_product(omega, w[cl], 1);
        // the rest particle has no e.u term
        out->k.c_3ow[cl] = cl == 0 ? 0 : fixed64_of_product(omega, w[cl], 3);
        if (!out->k.c_ow[cl] || (cl > 0 && !out->k.c_3ow[cl])) return false;
    }
    // |omega - 1| * 2^64, exact: omega = m 2^(e - 53) with e + 11 >= 0
    int e;
    const double fm = std::frexp(omega, &e);
    const __int128 om = (__int128)(uint64_t)std::ldexp(fm, 53) << (e + 11);
    const __int128 d = om - ((__int128)1 << 64);
    const __int128 ad = d < 0 ? -d : d;
    if (ad >> 64) return false;
    out->k.c_om1 = (uint64_t)ad;
    out->om_ge1 = d >= 0;
    out->frac_bits = fx::kFrac;
    return true;
}


}  // namespace imex
