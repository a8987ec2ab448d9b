// imex_conserved_noalloc: the conserved-quantity reduction for callers that
// cannot allocate device memory.
//
// Who needs it: a host code whose device memory is owned by its own pool
// allocator (and which must not take memory behind that allocator's back),
// or a latency-critical loop in which cudaMalloc's implicit device-wide
// synchronisation is not acceptable.  Such a caller keeps the distributions
// in its own buffer and wants the diagnostics of src/lbm.cpp:266-306
// without creating a lattice handle (imex_create allocates).
//
// How: the reduction's per-block partial sums live in a file-scope static
// device array of fixed size instead of a cudaMalloc'd buffer.  Every GPU
// that loads this library holds that array (5 MiB) until the process exits.
// The array's name in host code is a host-side stand-in, not a device
// address, so the host looks up its device address once per device with
// cudaGetSymbolAddress and passes that pointer to the kernels.
#include <mutex>
#include <string>

#include "imexlbm.h"
#include "imexlbm_internal.hpp"
#include "kernels_f64.cuh"

namespace {

// One partial sum of 5 doubles per block of 128 z-cells of one (x, y) row:
// at most 131072 blocks, e.g. a 256^3 lattice.
constexpr size_t kMaxPartials = 131072;

static __device__ __align__(256) double g_partials[kMaxPartials * 5];

constexpr int kMaxDevices = 64;
std::mutex g_lock;
double* g_partials_dev[kMaxDevices] = {};

// Device address of g_partials on the current device (looked up on the
// first call per device and kept: a cudaDeviceReset, which unloads the
// library's device code, would leave the kept address stale - the header
// tells callers not to use this entry point after a reset).
int partials_address(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return imex::set_thread_error(IMEX_ERR_CUDA, std::string("imex_conserved_noalloc: cudaGetDevice: ") +
                                                         cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices)
        return imex::set_thread_error(IMEX_ERR_ARG, "imex_conserved_noalloc: device index above 63");
    std::lock_guard<std::mutex> guard(g_lock);
    if (!g_partials_dev[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_partials);
        if (e != cudaSuccess || !p)
            return imex::set_thread_error(IMEX_ERR_CUDA, std::string("imex_conserved_noalloc: cudaGetSymbolAddress: ") +
                                                             cudaGetErrorString(e));
        g_partials_dev[dev] = static_cast<double*>(p);
    }
    *out = g_partials_dev[dev];
    return IMEX_OK;
}

}  // namespace

extern "C" int imex_conserved_noalloc(const double* f_dev, int nx, int ny, int nz, double* out_dev, void* stream)
{
    if (!f_dev || !out_dev) return imex::set_thread_error(IMEX_ERR_ARG, "imex_conserved_noalloc: null pointer");
    if (nx < 1 || ny < 1 || nz < 1 || nx > 65535 || ny > 65535)
        return imex::set_thread_error(IMEX_ERR_ARG, "imex_conserved_noalloc: need 1 <= nx, ny <= 65535 and nz >= 1");
    imex::Geom g;
    g.nx = nx;
    g.ny = ny;
    g.nz = nz;
    g.plane = (size_t)nx * ny * nz;
    const size_t need = imex::conserved_partials(g);
    if (need > kMaxPartials)
        return imex::set_thread_error(
            IMEX_ERR_ARG, "imex_conserved_noalloc: lattice needs " + std::to_string(need) +
                              " partial sums (one per 128 z-cells of a row); the static scratch holds 131072 "
                              "(for example 256x256x256)");
    double* partials = nullptr;
    int rc = partials_address(&partials);
    if (rc) return rc;
    // Each call writes every partial it later reads, so nothing carries over
    // from the previous call's contents.
    cudaError_t e = imex::launch_conserved_f64(false, f_dev, g, partials, out_dev, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return imex::set_thread_error(IMEX_ERR_CUDA, std::string("imex_conserved_noalloc: launch: ") +
                                                         cudaGetErrorString(e));
    return IMEX_OK;
}
