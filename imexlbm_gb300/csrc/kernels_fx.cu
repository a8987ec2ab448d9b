// Fixed-point float64 engine (not yet enabled).
#include "kernels_fx.cuh"

namespace imex {

bool make_fx_params(double, double, FxParams* out)
{
    out->frac_bits = 0;
    out->pad = 0;
    return false;
}

cudaError_t launch_step_fx(int, const double*, double*, const Geom&, const FxParams&, const CollideF64&,
                           unsigned long long*, cudaStream_t)
{
    return cudaErrorNotSupported;
}

cudaError_t launch_conserved_fx(bool, const double*, const Geom&, const FxParams&, double*, double*, cudaStream_t)
{
    return cudaErrorNotSupported;
}

}  // namespace imex
