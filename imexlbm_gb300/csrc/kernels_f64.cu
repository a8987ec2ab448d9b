// Native float64 kernels: Taylor-Green initialisation, collide (in place),
// pull-stream, the fused pull-stream + collide step, and the moment
// reductions.  These are the "plain FP64" engine and the exact fallback of
// the fixed-point engine.
//
// On this GPU the float64 pipe issues about 1.7 FMA per clock per SM (the
// float32 pipe about 120), so the collision below is arranged to use as few
// float64 operations as possible (~190 per cell, versus ~300 written
// direction by direction): opposite directions share e.u, the quadratic
// term and the weight, and the relaxation is one FMA per direction.
#include "kernels_f64.cuh"
#include "collide_f64.cuh"
#include "tg_init.cuh"

namespace imex {

// ------------------------------------------------------------------- init --
__global__ void __launch_bounds__(kStepBlock) k_init_f64(double* __restrict__ f, Geom g, const double* __restrict__ tx,
                                                         const double* __restrict__ ty, const double* __restrict__ tz,
                                                         double rho0, double u0)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    double fe[kQ];
    tg_init_cell(fe, tx, ty, tz, i, j, k, rho0, u0);
    const size_t cell = ((size_t)i * g.ny + j) * g.nz + k;
#pragma unroll
    for (int a = 0; a < kQ; ++a) f[(size_t)a * g.plane + cell] = fe[a];
}

// ------------------------------------------------------------------- step --
// PULL: gather from x - e_a (streaming); COLLIDE: BGK after the gather.
//   PULL && COLLIDE   fused step  dst = C(S(src))
//   !PULL && COLLIDE  collision   dst = C(src)   (src == dst allowed: each
//                                 thread reads, then writes, only its cell)
//   PULL && !COLLIDE  streaming   dst = S(src)   (src != dst)
template <bool PULL, bool COLLIDE>
__global__ void __launch_bounds__(kStepBlock) k_step_f64(const double* src, double* dst, Geom g, CollideF64 cp)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const PullIndex pi(g, i, j, k, PULL);
    double f[kQ];
#pragma unroll
    for (int a = 0; a < kQ; ++a) f[a] = 0.0;
    if constexpr (PULL) {
        gather27<double>(src, g, pi, f);
    } else {
        const size_t cell = ((size_t)i * g.ny + j) * g.nz + k;
#pragma unroll
        for (int a = 0; a < kQ; ++a) f[a] = src[(size_t)a * g.plane + cell];
    }
    if constexpr (COLLIDE) collide_f64(f, cp);
    const size_t cell = ((size_t)i * g.ny + j) * g.nz + k;
#pragma unroll
    for (int a = 0; a < kQ; ++a) dst[(size_t)a * g.plane + cell] = f[a];
}

// -------------------------------------------------------------- reductions --
// Moments of one cell in the reference's order (src/lbm.cpp:277-285).
__device__ __forceinline__ void moments_f64(const double (&f)[kQ], double& pl, double& ul, double& vl, double& wl)
{
    pl = 0.0;
    ul = 0.0;
    vl = 0.0;
    wl = 0.0;
#pragma unroll
    for (int a = 0; a < kQ; ++a) {
        pl += f[a];
        if (ex(a, 0) == 1) ul += f[a];
        if (ex(a, 0) == -1) ul -= f[a];
        if (ex(a, 1) == 1) vl += f[a];
        if (ex(a, 1) == -1) vl -= f[a];
        if (ex(a, 2) == 1) wl += f[a];
        if (ex(a, 2) == -1) wl -= f[a];
    }
}

// Per-block partial sums of {mass, px, py, pz, ke} (src/lbm.cpp:271-294)
// over the block's cells; one partial per block, in block order.
template <bool PULL>
__global__ void __launch_bounds__(kStepBlock) k_conserved_f64(const double* __restrict__ src, Geom g, double* __restrict__ partial)
{
    __shared__ double smem[32 * 5];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (k < g.nz) {
        const PullIndex pi(g, i, j, k, PULL);
        double f[kQ];
        gather27<double>(src, g, pi, f);
        double pl, ul, vl, wl;
        moments_f64(f, pl, ul, vl, wl);
        v[0] = pl;
        v[1] = ul;
        v[2] = vl;
        v[3] = wl;
        v[4] = 0.5 * (ul * ul + vl * vl + wl * wl);
    }
    block_sum<5>(v, smem);
    if (threadIdx.x == 0) {
        const size_t b = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
#pragma unroll
        for (int q = 0; q < 5; ++q) partial[b * 5 + q] = v[q];
    }
}

// Sum `n` partials of 5 values in a fixed order (one block).
__global__ void __launch_bounds__(1024) k_reduce_partials(const double* __restrict__ partial, size_t n, double* __restrict__ out)
{
    __shared__ double smem[32 * 5];
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (size_t b = threadIdx.x; b < n; b += blockDim.x)
#pragma unroll
        for (int q = 0; q < 5; ++q) v[q] += partial[b * 5 + q];
    block_sum<5>(v, smem);
    if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < 5; ++q) out[q] = v[q];
}

// Per-cell p, u, v, w (src/lbm.cpp:218-236).
template <bool PULL>
__global__ void __launch_bounds__(kStepBlock) k_macro_f64(const double* __restrict__ src, Geom g, double* __restrict__ p,
                                                          double* __restrict__ u, double* __restrict__ v, double* __restrict__ w)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const PullIndex pi(g, i, j, k, PULL);
    double f[kQ];
    gather27<double>(src, g, pi, f);
    double pl, ul, vl, wl;
    moments_f64(f, pl, ul, vl, wl);
    const size_t cell = ((size_t)i * g.ny + j) * g.nz + k;
    if (p) p[cell] = pl * (1.0 / 3.0);
    u[cell] = ul;
    v[cell] = vl;
    w[cell] = wl;
}

// max over cells of |a - b| and of |b| for three component arrays of n
// values; results as the bit patterns of non-negative doubles (ordered like
// unsigned integers), combined with atomicMax.
__global__ void k_maxdiff3(const double* __restrict__ a, const double* __restrict__ b, size_t n,
                           unsigned long long* __restrict__ out)
{
    double md = 0.0, mb = 0.0;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            md = fmax(md, fabs(a[c * n + q] - b[c * n + q]));
            mb = fmax(mb, fabs(b[c * n + q]));
        }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        md = fmax(md, __shfl_down_sync(0xffffffffu, md, o));
        mb = fmax(mb, __shfl_down_sync(0xffffffffu, mb, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, (unsigned long long)__double_as_longlong(md));
        atomicMax(out + 1, (unsigned long long)__double_as_longlong(mb));
    }
}

// ---------------------------------------------------------------- launchers --
static dim3 step_grid(const Geom& g) { return dim3((g.nz + kStepBlock - 1) / kStepBlock, g.ny, g.nx); }

size_t conserved_partials(const Geom& g)
{
    const dim3 gr = step_grid(g);
    return (size_t)gr.x * gr.y * gr.z;
}

cudaError_t launch_init_f64(double* f, const Geom& g, const double* tx, const double* ty, const double* tz, double rho0,
                            double u0, cudaStream_t s)
{
    k_init_f64<<<step_grid(g), kStepBlock, 0, s>>>(f, g, tx, ty, tz, rho0, u0);
    return cudaGetLastError();
}

cudaError_t launch_step_f64(int mode, const double* src, double* dst, const Geom& g, const CollideF64& cp, cudaStream_t s)
{
    switch (mode) {
    case kModeFused: k_step_f64<true, true><<<step_grid(g), kStepBlock, 0, s>>>(src, dst, g, cp); break;
    case kModeCollide: k_step_f64<false, true><<<step_grid(g), kStepBlock, 0, s>>>(src, dst, g, cp); break;
    case kModeStream: k_step_f64<true, false><<<step_grid(g), kStepBlock, 0, s>>>(src, dst, g, cp); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_conserved_f64(bool pull, const double* src, const Geom& g, double* partial, double* out, cudaStream_t s)
{
    if (pull)
        k_conserved_f64<true><<<step_grid(g), kStepBlock, 0, s>>>(src, g, partial);
    else
        k_conserved_f64<false><<<step_grid(g), kStepBlock, 0, s>>>(src, g, partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_reduce_partials(partial, conserved_partials(g), out, s);
}

cudaError_t launch_reduce_partials(const double* partial, size_t n, double* out, cudaStream_t s)
{
    k_reduce_partials<<<1, 1024, 0, s>>>(partial, n, out);
    return cudaGetLastError();
}

cudaError_t launch_macro_f64(bool pull, const double* src, const Geom& g, double* p, double* u, double* v, double* w,
                             cudaStream_t s)
{
    if (pull)
        k_macro_f64<true><<<step_grid(g), kStepBlock, 0, s>>>(src, g, p, u, v, w);
    else
        k_macro_f64<false><<<step_grid(g), kStepBlock, 0, s>>>(src, g, p, u, v, w);
    return cudaGetLastError();
}

cudaError_t launch_maxdiff3(const double* a, const double* b, size_t n, unsigned long long* out, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(out, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    k_maxdiff3<<<current_sm_count() * 8, 256, 0, s>>>(a, b, n, out);
    return cudaGetLastError();
}

CollideF64 make_collide_f64(double tau0)
{
    CollideF64 cp;
    const double omega = 1.0 / (tau0 + 0.5);  // src/lbm.cpp:133
    cp.omega = omega;
    cp.one_minus_omega = 1.0 - omega;
    const double w[4] = {8.0 / 27.0, 2.0 / 27.0, 1.0 / 54.0, 1.0 / 216.0};
    for (int c = 0; c < 4; ++c) {
        cp.ow[c] = omega * w[c];
        cp.tow[c] = 3.0 * omega * w[c];
    }
    return cp;
}

}  // namespace imex
