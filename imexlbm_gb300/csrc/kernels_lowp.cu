// Reduced-precision storage: float32 distributions (IMEX_F32) and float16
// deviations from the lattice weights, h = f - w (IMEX_F16DEV).  Both
// collide in float32; diagnostics accumulate in float64.
//
// The float32 collision works in deviation space for both formats: with
// h_a = f_a - w_a (exact in float32 for f_a in [w_a / 2, 2 w_a]), sum h = 3p - 1,
// sum h e = u (sum w e = 0), and the equilibrium deviation is
//   heq_a = w_a (sum h + 3 e.u + 4.5 (e.u)^2 - 1.5 u.u)
// (src/lbm.cpp:153-162 with w_a subtracted).  The moments then come from
// O(0.01) numbers instead of O(0.1) ones.
//
// Relaxation.  The reference's f - (f - feq) omega with omega = 1/(tau0+0.5)
// (src/lbm.cpp:133,163) is written as
//   h <- 2 heq - h + eps (h - heq),   eps = 2 - omega = 2 tau0 / (tau0 + 0.5)
// because omega is close to 2 at the Reynolds numbers of interest: a
// float32 omega carries a 6e-8 absolute error, which is a 6e-5 relative
// error in the viscosity at tau0 = 5e-4 and makes the kinetic energy decay
// at the wrong rate.  eps itself is exact to 6e-8 relative, and so is the
// viscosity.
//
// Momentum.  Opposite directions get heq = A +- B with B = b_a (e.u): the
// equilibrium's momentum is sum over pairs of 2 b_a (e_a.u) e_a, which is u
// only if 2 (b_axis + 4 b_face + 4 b_corner) = 1 holds exactly.  With each
// b = 3 w rounded to float32 separately it is off by ~1e-8, every collision
// then scales the momentum by (1 + 2e-8), and the kinetic energy drifts by
// ~3e-8 per step (2e-4 after 5000 steps).  The b are therefore chosen on
// binary grids where b_axis = 1/2 - 4 b_face - 4 b_corner is exact; the
// drift falls to rounding noise (~1e-8 after 200 steps at 32^3).
#include <cmath>

#include <cuda_fp16.h>

#include "kernels_lowp.cuh"
#include "rows.cuh"
#include "tg_init.cuh"

namespace imex {

namespace {

template <int P>
struct Storage;

template <>
struct Storage<IMEX_F32> {
    using T = float;
    static __device__ __forceinline__ float load(const float* p, int a)
    {
        return __ldg(p) - (float)weight(a);
    }
    static __device__ __forceinline__ float load_plain(const float* p, int a) { return *p - (float)weight(a); }
    static __device__ __forceinline__ float store(float h, int a) { return (float)weight(a) + h; }
    static __device__ __forceinline__ double to_f64(float v, int) { return (double)v; }
    static __device__ __forceinline__ float from_f64(double f, int) { return __double2float_rn(f); }
};

template <>
struct Storage<IMEX_F16DEV> {
    using T = __half;
    static __device__ __forceinline__ float load(const __half* p, int) { return __half2float(__ldg(p)); }
    static __device__ __forceinline__ float load_plain(const __half* p, int) { return __half2float(*p); }
    static __device__ __forceinline__ __half store(float h, int) { return __float2half_rn(h); }
    static __device__ __forceinline__ double to_f64(__half v, int a) { return weight(a) + (double)__half2float(v); }
    static __device__ __forceinline__ __half from_f64(double f, int a) { return __float2half_rn((float)(f - weight(a))); }
};

// float32 BGK collision of the deviations h (see the file header).
__device__ __forceinline__ void collide_dev_f32(float (&h)[kQ], const CollideF32& cp)
{
    float d[kPairs + 1], s[kPairs + 1];
#pragma unroll
    for (int k = 1; k <= kPairs; ++k) {
        d[k] = h[2 * k - 1] - h[2 * k];
        s[k] = h[2 * k - 1] + h[2 * k];
    }
    const float sig = ((((s[1] + s[2]) + (s[3] + s[4])) + ((s[5] + s[6]) + (s[7] + s[8]))) +
                       (((s[9] + s[10]) + (s[11] + s[12])) + (s[13] + h[0])));
    float u[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int dim = 0; dim < 3; ++dim)
#pragma unroll
        for (int k = 1; k <= kPairs; ++k) {
            const int e = ex(2 * k - 1, dim);
            if (e == 1) u[dim] += d[k];
            if (e == -1) u[dim] -= d[k];
        }
    const float udu = fmaf(u[2], u[2], fmaf(u[1], u[1], u[0] * u[0]));
    const float base = fmaf(-1.5f, udu, sig);
    const float eps = cp.eps;
    {
        const float heq = cp.w[0] * base;
        h[0] = fmaf(eps, h[0] - heq, fmaf(2.f, heq, -h[0]));
    }
#pragma unroll
    for (int k = 1; k <= kPairs; ++k) {
        const int a = 2 * k - 1;
        const int cls = weight216(a) == 16 ? 1 : weight216(a) == 4 ? 2 : 3;
        float edu = 0.f;
        bool first = true;
#pragma unroll
        for (int dim = 0; dim < 3; ++dim) {
            const int e = ex(a, dim);
            if (e != 0) {
                edu = first ? (e == 1 ? u[dim] : -u[dim]) : (e == 1 ? edu + u[dim] : edu - u[dim]);
                first = false;
            }
        }
        const float A = cp.w[cls] * fmaf(4.5f * edu, edu, base);
        const float B = cp.w3[cls] * edu;
        const float ep = A + B, em = A - B;
        h[a] = fmaf(eps, h[a] - ep, fmaf(2.f, ep, -h[a]));
        h[a + 1] = fmaf(eps, h[a + 1] - em, fmaf(2.f, em, -h[a + 1]));
    }
}

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
    collide_dev_f32(h, cp);
#pragma unroll
    for (int a = 0; a < kQ; ++a) dst[(size_t)a * g.plane + cell] = S::store(h[a], a);
}

// Row-kernel engine: float32 collision of one staged cell.
template <int P>
struct EngLowp {
    using T = typename Storage<P>::T;
    static constexpr int kMinBlocks = 4;
    CollideF32 cp;

    __device__ __forceinline__ void run(const T* __restrict__ st, int astride, int nz, int z, T* __restrict__ dst,
                                        size_t plane, size_t rowoff) const
    {
        const int zm = z == 0 ? nz - 1 : z - 1, zp = z == nz - 1 ? 0 : z + 1;
        float h[kQ];
#pragma unroll
        for (int a = 0; a < kQ; ++a) h[a] = Storage<P>::load_plain(st + a * astride + pull_z(ex(a, 2), z, zm, zp), a);
        collide_dev_f32(h, cp);
#pragma unroll
        for (int a = 0; a < kQ; ++a) dst[(size_t)a * plane + rowoff + z] = Storage<P>::store(h[a], a);
    }
};

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

// Partial sums of {mass, px, py, pz, ke} with float64 per-cell moments of
// the stored values (src/lbm.cpp:271-294), one partial per block.
template <int P, bool PULL>
__global__ void __launch_bounds__(kStepBlock) k_conserved_lowp(const typename Storage<P>::T* __restrict__ src, Geom g,
                                                               double* __restrict__ partial)
{
    __shared__ double smem[32 * 5];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (k < g.nz) {
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
    return prec == IMEX_F32 ? rows_eligible<float>(g) : rows_eligible<__half>(g);
}

cudaError_t launch_rows_lowp(int prec, const void* src, void* dst, const Geom& g, const CollideF32& cp,
                             const RowConfig& rc, unsigned* err, cudaStream_t s)
{
    if (prec == IMEX_F32)
        return launch_rows(static_cast<const float*>(src), static_cast<float*>(dst), g, EngLowp<IMEX_F32>{cp}, rc, err, s);
    return launch_rows(static_cast<const __half*>(src), static_cast<__half*>(dst), g, EngLowp<IMEX_F16DEV>{cp}, rc,
                       err, s);
}

size_t rows_lowp_stage_bytes(int prec, int nz) { return (size_t)kQ * nz * (prec == IMEX_F32 ? 4 : 2); }

cudaError_t launch_from_f64(int prec, const double* f, void* out, const Geom& g, cudaStream_t s)
{
    const int blocks = 152 * 8;
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
