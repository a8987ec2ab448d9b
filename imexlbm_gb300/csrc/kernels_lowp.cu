// Reduced-precision storage kernels: float32 distributions (IMEX_F32) and
// float16 deviations 2^12 (f - w) (IMEX_F16DEV), collided in float32 by
// lowp::collide_dev_f32 (lowp_math.cuh, which explains the arithmetic);
// diagnostics accumulate in float64.
#include <atomic>
#include <cmath>

#include <cuda_fp16.h>

#include "kernels_lowp.cuh"
#include "lowp_math.cuh"
#include "rows.cuh"
#include "rows_lowp.cuh"
#include "tg_init.cuh"

namespace imex {

namespace {

using lowp::Storage;
using lowp::collide_dev_f32;

template <int P, bool PULL, bool COLLIDE>
__global__ void __launch_bounds__(kStepBlock) k_step_lowp(const typename Storage<P>::T* src, typename Storage<P>::T* dst,
                                                          Geom g, CollideF32 cp)
{
    using S = Storage<P>;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const PullIndex pi(g, i, j, k, PULL);
    const size_t cell = ((size_t)i * g.ny + j) * g.nz + k;
    if constexpr (!COLLIDE) {
        // streaming alone moves the stored bits unchanged
#pragma unroll
        for (int a = 0; a < kQ; ++a) dst[(size_t)a * g.plane + cell] = src[pi.at_dyn(g, a)];
        return;
    }
    float h[kQ];
    if constexpr (PULL) {
#pragma unroll
        for (int a = 0; a < kQ; ++a) h[a] = S::load(src + pi.at_dyn(g, a), a);
    } else {
#pragma unroll
        for (int a = 0; a < kQ; ++a) h[a] = S::load_plain(src + (size_t)a * g.plane + cell, a);
    }
    collide_dev_f32<P>(h, cp);
    if constexpr (P == IMEX_F16DEV) {
        auto at = [&](int a) -> __half& { return dst[(size_t)a * g.plane + cell]; };
        lowp::store_f16_cell(h, cp.sr, cell, cp.seed, at);
    } else {
#pragma unroll
        for (int a = 0; a < kQ; ++a) dst[(size_t)a * g.plane + cell] = S::store(h[a], a);
    }
}

// Taylor-Green initial state (float64 equilibrium, src/lbm.cpp:78-108),
// rounded once into the storage format.
template <int P>
__global__ void __launch_bounds__(kStepBlock) k_init_lowp(typename Storage<P>::T* __restrict__ f, Geom g,
                                                          const double* __restrict__ tx, const double* __restrict__ ty,
                                                          const double* __restrict__ tz, double rho0, double u0)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    double fe[kQ];
    tg_init_cell(fe, tx, ty, tz, i, j, k, rho0, u0);
    const size_t cell = ((size_t)i * g.ny + j) * g.nz + k;
#pragma unroll
    for (int a = 0; a < kQ; ++a) f[(size_t)a * g.plane + cell] = Storage<P>::from_f64(fe[a], a);
}

// Conversions between float64 reference-order f and the storage format.
template <int P>
__global__ void k_from_f64(const double* __restrict__ f, typename Storage<P>::T* __restrict__ out, size_t plane)
{
    const size_t n = (size_t)kQ * plane;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        out[q] = Storage<P>::from_f64(f[q], (int)(q / plane));
}

template <int P, bool PULL>
__global__ void __launch_bounds__(kStepBlock) k_to_f64(const typename Storage<P>::T* __restrict__ src, Geom g,
                                                       double* __restrict__ out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const PullIndex pi(g, i, j, k, PULL);
    const size_t cell = ((size_t)i * g.ny + j) * g.nz + k;
#pragma unroll
    for (int a = 0; a < kQ; ++a) out[(size_t)a * g.plane + cell] = Storage<P>::to_f64(src[pi.at_dyn(g, a)], a);
}

// Partial sums of {mass, px, py, pz, ke} (src/lbm.cpp:271-294), one partial
// per block.  A cell's moments are float32 sums of its deviations h (the
// stored values' own precision: float32 f - w is exact, float16 values are
// exact in float32), pair by pair as the collision forms them: mass =
// 1 + sum h, momentum = sum h e (sum w = 1, sum w e = 0).  They become
// float64 for the kinetic energy and the block and global sums.  Float64
// arithmetic per value would make this reduction bound by the float64 pipe
// (1.67 op/clk/SM): 5.2 ms at 256^3 instead of a fraction of a step.
template <int P, bool PULL>
__global__ void __launch_bounds__(kStepBlock) k_conserved_lowp(const typename Storage<P>::T* __restrict__ src, Geom g,
                                                               double* __restrict__ partial)
{
    using A = lowp::F1;
    __shared__ double smem[32 * 5];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (k < g.nz) {
        const PullIndex pi(g, i, j, k, PULL);
        float h[kQ];
#pragma unroll
        for (int a = 0; a < kQ; ++a) h[a] = Storage<P>::dev(src[pi.at_dyn(g, a)], a);
        float d[kPairs + 1], sp[kPairs + 1];
#pragma unroll
        for (int q = 1; q <= kPairs; ++q) {
            d[q] = A::sub(h[2 * q - 1], h[2 * q]);
            sp[q] = A::add(h[2 * q - 1], h[2 * q]);
        }
        float sig = h[0];
#pragma unroll
        for (int q = 1; q <= kPairs; ++q) sig = A::add(sig, sp[q]);
        float u[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int dim = 0; dim < 3; ++dim)
#pragma unroll
            for (int q = 1; q <= kPairs; ++q) {
                const int e = ex(2 * q - 1, dim);
                if (e == 1) u[dim] = A::add(u[dim], d[q]);
                if (e == -1) u[dim] = A::sub(u[dim], d[q]);
            }
        constexpr double inv = 1.0 / Storage<P>::kScale;
        const double ul = (double)u[0] * inv, vl = (double)u[1] * inv, wl = (double)u[2] * inv;
        v[0] = 1.0 + (double)sig * inv;
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

// Per-cell p, u, v, w in float64 from the stored values (src/lbm.cpp:218-236).
template <int P, bool PULL>
__global__ void __launch_bounds__(kStepBlock) k_macro_lowp(const typename Storage<P>::T* __restrict__ src, Geom g,
                                                           double* __restrict__ p, double* __restrict__ u,
                                                           double* __restrict__ v, double* __restrict__ w)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const PullIndex pi(g, i, j, k, PULL);
    double pl = 0.0, ul = 0.0, vl = 0.0, wl = 0.0;
#pragma unroll
    for (int a = 0; a < kQ; ++a) {
        const double fv = Storage<P>::to_f64(src[pi.at_dyn(g, a)], a);
        pl += fv;
        if (ex(a, 0) == 1) ul += fv;
        if (ex(a, 0) == -1) ul -= fv;
        if (ex(a, 1) == 1) vl += fv;
        if (ex(a, 1) == -1) vl -= fv;
        if (ex(a, 2) == 1) wl += fv;
        if (ex(a, 2) == -1) wl -= fv;
    }
    const size_t cell = ((size_t)i * g.ny + j) * g.nz + k;
    if (p) p[cell] = pl * (1.0 / 3.0);
    u[cell] = ul;
    v[cell] = vl;
    w[cell] = wl;
}

dim3 step_grid(const Geom& g) { return dim3((g.nz + kStepBlock - 1) / kStepBlock, g.ny, g.nx); }

template <int P>
cudaError_t step_impl(int mode, const void* src, void* dst, const Geom& g, const CollideF32& cp, cudaStream_t s)
{
    using T = typename Storage<P>::T;
    const T* a = static_cast<const T*>(src);
    T* b = static_cast<T*>(dst);
    switch (mode) {
    case kModeFused: k_step_lowp<P, true, true><<<step_grid(g), kStepBlock, 0, s>>>(a, b, g, cp); break;
    case kModeCollide: k_step_lowp<P, false, true><<<step_grid(g), kStepBlock, 0, s>>>(a, b, g, cp); break;
    case kModeStream: k_step_lowp<P, true, false><<<step_grid(g), kStepBlock, 0, s>>>(a, b, g, cp); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace

CollideF32 make_collide_f32(double tau0)
{
    CollideF32 cp;
    const double omega = 1.0 / (tau0 + 0.5);  // src/lbm.cpp:133
    cp.eps = (float)(2.0 - omega);              // exact in float64 for omega in [1, 2]
    const double w[4] = {8.0 / 27.0, 2.0 / 27.0, 1.0 / 54.0, 1.0 / 216.0};  // src/lbm.cpp:10-17
    for (int c = 0; c < 4; ++c) cp.w[c] = (float)w[c];
    // e.u coefficients 3 w with the momentum identity exact in float32:
    // b_face on the 2^-27 grid, b_corner on the 2^-28 grid, so that
    // 1/2 - 4 b_face - 4 b_corner lands on the 2^-26 grid of b_axis.
    const double bf = std::nearbyint(3.0 * w[2] * 0x1p27) * 0x1p-27;
    const double bc = std::nearbyint(3.0 * w[3] * 0x1p28) * 0x1p-28;
    const double ba = 0.5 - 4.0 * bf - 4.0 * bc;
    cp.w3[0] = 0.f;
    cp.w3[1] = (float)ba;
    cp.w3[2] = (float)bf;
    cp.w3[3] = (float)bc;
    cp.sr = 0;
    cp.seed = 0;
    return cp;
}

cudaError_t launch_init_lowp(int prec, void* f, const Geom& g, const double* tx, const double* ty, const double* tz,
                             double rho0, double u0, cudaStream_t s)
{
    if (prec == IMEX_F32)
        k_init_lowp<IMEX_F32><<<step_grid(g), kStepBlock, 0, s>>>(static_cast<float*>(f), g, tx, ty, tz, rho0, u0);
    else
        k_init_lowp<IMEX_F16DEV><<<step_grid(g), kStepBlock, 0, s>>>(static_cast<__half*>(f), g, tx, ty, tz, rho0, u0);
    return cudaGetLastError();
}

cudaError_t launch_step_lowp(int prec, int mode, const void* src, void* dst, const Geom& g, const CollideF32& cp,
                             cudaStream_t s)
{
    return prec == IMEX_F32 ? step_impl<IMEX_F32>(mode, src, dst, g, cp, s)
                            : step_impl<IMEX_F16DEV>(mode, src, dst, g, cp, s);
}

bool rows_lowp_eligible(int prec, const Geom& g)
{
    const size_t row = (size_t)g.nz * (prec == IMEX_F32 ? 4 : 2);
    return row % 16 == 0 && row <= (size_t)kRowsLowpDirMax && (size_t)g.nx * g.ny < 0x7fffffffu;
}

template <int D, int MINB>
cudaError_t launch_rows_lowp_d(int prec, const void* src, void* dst, const Geom& g, const CollideF32& cp,
                               const RowConfig& rc, unsigned* err, cudaStream_t s, unsigned grid)
{
    const size_t smem = rowslp::smem_bytes(D, rc.stages);
    // raise the kernel's shared-memory limit once per device and size, not
    // per launch (the attribute belongs to the device's context)
    static std::atomic<int> allowed[64];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev >= 64 || (int)smem > allowed[dev].load()) {
        e = cudaFuncSetAttribute(rowslp::k_rows_lowp<D, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess) return e;
        if (dev < 64) allowed[dev].store((int)smem);
    }
    rowslp::k_rows_lowp<D, MINB><<<grid, rowslp::kThreads, smem, s>>>(src, dst, g, prec, rc.rows, cp, rc.stages,
                                                                       make_wait_ctl(err));
    return cudaGetLastError();
}

cudaError_t launch_rows_lowp(int prec, const void* src, void* dst, const Geom& g, const CollideF32& cp,
                             const RowConfig& rc, unsigned* err, cudaStream_t s)
{
    const int sms = current_sm_count();
    const size_t es = prec == IMEX_F32 ? 4 : 2;
    if (rc.rows < 1 || (size_t)rc.rows * g.nz * es > (size_t)rc.dir_bytes || rc.stages < 2)
        return cudaErrorInvalidValue;
    const long long items = (long long)g.nx * rowslp::y_blocks(g.ny, rc.rows);
    long long grid = (long long)sms * rc.ctas_per_sm;
    if (grid > items) grid = items;
    const bool one = rc.ctas_per_sm <= 1;  // one resident CTA: the full register file
    switch (rc.dir_bytes) {
    case 1024:
        return one ? launch_rows_lowp_d<1024, 1>(prec, src, dst, g, cp, rc, err, s, (unsigned)grid)
                   : launch_rows_lowp_d<1024, 2>(prec, src, dst, g, cp, rc, err, s, (unsigned)grid);
    case 2048:
        return one ? launch_rows_lowp_d<2048, 1>(prec, src, dst, g, cp, rc, err, s, (unsigned)grid)
                   : launch_rows_lowp_d<2048, 2>(prec, src, dst, g, cp, rc, err, s, (unsigned)grid);
    case 4096: return launch_rows_lowp_d<4096, 1>(prec, src, dst, g, cp, rc, err, s, (unsigned)grid);
    default: return cudaErrorInvalidValue;
    }
}

size_t rows_lowp_stage_bytes(int prec, int nz) { return (size_t)kQ * nz * (prec == IMEX_F32 ? 4 : 2); }

cudaError_t launch_from_f64(int prec, const double* f, void* out, const Geom& g, cudaStream_t s)
{
    const int blocks = current_sm_count() * 8;
    if (prec == IMEX_F32)
        k_from_f64<IMEX_F32><<<blocks, 256, 0, s>>>(f, static_cast<float*>(out), g.plane);
    else
        k_from_f64<IMEX_F16DEV><<<blocks, 256, 0, s>>>(f, static_cast<__half*>(out), g.plane);
    return cudaGetLastError();
}

cudaError_t launch_to_f64(int prec, bool pull, const void* src, const Geom& g, double* out, cudaStream_t s)
{
    if (prec == IMEX_F32) {
        const float* p = static_cast<const float*>(src);
        if (pull) k_to_f64<IMEX_F32, true><<<step_grid(g), kStepBlock, 0, s>>>(p, g, out);
        else k_to_f64<IMEX_F32, false><<<step_grid(g), kStepBlock, 0, s>>>(p, g, out);
    } else {
        const __half* p = static_cast<const __half*>(src);
        if (pull) k_to_f64<IMEX_F16DEV, true><<<step_grid(g), kStepBlock, 0, s>>>(p, g, out);
        else k_to_f64<IMEX_F16DEV, false><<<step_grid(g), kStepBlock, 0, s>>>(p, g, out);
    }
    return cudaGetLastError();
}

cudaError_t launch_macro_lowp(int prec, bool pull, const void* src, const Geom& g, double* p, double* u, double* v,
                              double* w, cudaStream_t s)
{
    if (prec == IMEX_F32) {
        const float* q = static_cast<const float*>(src);
        if (pull) k_macro_lowp<IMEX_F32, true><<<step_grid(g), kStepBlock, 0, s>>>(q, g, p, u, v, w);
        else k_macro_lowp<IMEX_F32, false><<<step_grid(g), kStepBlock, 0, s>>>(q, g, p, u, v, w);
    } else {
        const __half* q = static_cast<const __half*>(src);
        if (pull) k_macro_lowp<IMEX_F16DEV, true><<<step_grid(g), kStepBlock, 0, s>>>(q, g, p, u, v, w);
        else k_macro_lowp<IMEX_F16DEV, false><<<step_grid(g), kStepBlock, 0, s>>>(q, g, p, u, v, w);
    }
    return cudaGetLastError();
}

cudaError_t launch_conserved_lowp(int prec, bool pull, const void* src, const Geom& g, double* partial, double* out,
                                  cudaStream_t s)
{
    if (prec == IMEX_F32) {
        const float* p = static_cast<const float*>(src);
        if (pull) k_conserved_lowp<IMEX_F32, true><<<step_grid(g), kStepBlock, 0, s>>>(p, g, partial);
        else k_conserved_lowp<IMEX_F32, false><<<step_grid(g), kStepBlock, 0, s>>>(p, g, partial);
    } else {
        const __half* p = static_cast<const __half*>(src);
        if (pull) k_conserved_lowp<IMEX_F16DEV, true><<<step_grid(g), kStepBlock, 0, s>>>(p, g, partial);
        else k_conserved_lowp<IMEX_F16DEV, false><<<step_grid(g), kStepBlock, 0, s>>>(p, g, partial);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_reduce_partials(partial, conserved_partials(g), out, s);
}

}  // namespace imex
