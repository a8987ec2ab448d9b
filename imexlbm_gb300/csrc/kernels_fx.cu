// Fixed-point float64 engine: the fused pull-stream + BGK collision with the
// float64 arithmetic replaced by exact 64-bit fixed-point arithmetic on the
// integer pipes.
//
// Why.  This GPU's float64 pipe issues about 1.7 operations per clock per SM
// (conversions to and from float64 included), the integer pipes about 64
// each and IMAD.WIDE about 30.  A native float64 D3Q27 collision needs ~190
// float64 operations per cell and tops out near 20% of the HBM roofline; the
// same collision in integers costs ~1100 instructions per cell spread over
// the ALU and IMAD pipes, which is below the HBM time of a cell.
//
// The arithmetic itself is in fx_math.cuh.  Cells outside its exact range
// (any negative, tiny or huge value, NaN/Inf) are recomputed with the
// native float64 collision from their original inputs and counted; for the
// Taylor-Green decks (rho0 = 1, u0 <= 0.08) no cell leaves it.
#include <cstdint>
#include <cmath>

#include "collide_f64.cuh"
#include "fx_math.cuh"
#include "kernels_fx.cuh"
#include "rows.cuh"

namespace imex {

namespace {

// Native float64 redo of one cell (cells outside the exact range).
__device__ __noinline__ void fallback_cell(const double* __restrict__ src, double* __restrict__ dst, Geom g, int i,
                                           int j, int k, CollideF64 cp, unsigned long long* fallback)
{
    const PullIndex pi(g, i, j, k, true);
    double h[kQ];
    gather27<double>(src, g, pi, h);
    collide_f64(h, cp);
    const size_t cell = ((size_t)i * g.ny + j) * g.nz + k;
#pragma unroll
    for (int a = 0; a < kQ; ++a) dst[(size_t)a * g.plane + cell] = h[a];
    atomicAdd(fallback, 1ull);
}

// Fused pull-stream + fixed-point collision.  OM_GE1: omega >= 1, so the
// (1 - omega) f term is subtracted.  Five resident blocks per SM (96
// registers, 20 warps): at 256^3 90.3% of the copy bandwidth, against 87.8%
// at the compiler's 116 registers (4 blocks) and 87.6% at 80 registers (6
// blocks, with spills).  The kernel is bound by memory-level parallelism.
template <bool OM_GE1>
__global__ void __launch_bounds__(kStepBlock, 5) k_step_fx(const double* __restrict__ src, double* __restrict__ dst, Geom g,
                                                        FxConst c, CollideF64 cp, unsigned long long* __restrict__ fallback)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    double f[kQ];
    {
        const PullIndex pi(g, i, j, k, true);
        gather27<double>(src, g, pi, f);
    }

    bool ok = true;
    double out[kQ];
    fx::collide_cell<OM_GE1>(f, out, c, ok);

    const size_t cell = ((size_t)i * g.ny + j) * g.nz + k;
#pragma unroll
    for (int a = 0; a < kQ; ++a) dst[(size_t)a * g.plane + cell] = out[a];

    // Outside the exact range: redo this cell with native float64 from its
    // original inputs (src is not written by this kernel); those stores
    // overwrite the ones above.
    if (!ok) fallback_cell(src, dst, g, i, j, k, cp, fallback);
}

// In-place collision of the fixed-point engine (a Collision() on a state
// whose streaming is not pending: the first step of a run, or after the
// distributions were set).  The same cell arithmetic as the fused kernels,
// so every call order gives the same bits; a cell outside the exact range is
// collided in native float64 from the inputs it still holds.
template <bool OM_GE1>
__global__ void __launch_bounds__(kStepBlock, 5) k_collide_fx(double* __restrict__ f, Geom g, FxConst c, CollideF64 cp,
                                                           unsigned long long* __restrict__ fallback)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    const size_t cell = ((size_t)i * g.ny + j) * g.nz + k;
    double v[kQ], out[kQ];
#pragma unroll
    for (int a = 0; a < kQ; ++a) v[a] = f[(size_t)a * g.plane + cell];
    bool ok = true;
    fx::collide_cell<OM_GE1>(v, out, c, ok);
    if (!ok) {
        collide_f64(v, cp);
#pragma unroll
        for (int a = 0; a < kQ; ++a) out[a] = v[a];
        atomicAdd(fallback, 1ull);
    }
#pragma unroll
    for (int a = 0; a < kQ; ++a) f[(size_t)a * g.plane + cell] = out[a];
}

// The fused step inside a run of steps that keeps the state as X between
// its launches (see launch_step_fx_run): IN_FX / OUT_FX read / write X on
// the float64 grid instead of float64, which saves the 27 conversions each
// way (4% of the step at 256^3: the integer ALU pipe bounds this kernel).
// The results are the same numbers either way.  A cell outside the exact
// range cannot be stored as X, so instead of redoing it the launch records
// its step number j in *fail; launches of later steps then return at once
// and the host redoes the run from the last complete step with k_step_fx.
template <bool OM_GE1, bool IN_FX, bool OUT_FX>
__global__ void __launch_bounds__(kStepBlock, 5)
    k_step_fxs(const unsigned long long* __restrict__ src, unsigned long long* __restrict__ dst, Geom g, FxConst c,
               int j, int* __restrict__ fail)
{
    if (*fail < j) return;  // an earlier step of the run failed
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int jj = blockIdx.y, i = blockIdx.z;
    if (k >= g.nz) return;
    unsigned long long f[kQ];
    {
        const PullIndex pi(g, i, jj, k, true);
        gather27<unsigned long long>(src, g, pi, f);
    }
    uint64_t in[kQ], out[kQ];
#pragma unroll
    for (int a = 0; a < kQ; ++a) in[a] = f[a];
    bool ok = true;
    fx::collide_cell_io<OM_GE1, IN_FX, OUT_FX>(in, out, c, ok);
    const size_t cell = ((size_t)i * g.ny + jj) * g.nz + k;
#pragma unroll
    for (int a = 0; a < kQ; ++a) dst[(size_t)a * g.plane + cell] = out[a];
    if (!ok) atomicMin(fail, j);
}

// X (on the float64 grid) -> float64, in place.
__global__ void k_fx_to_f64(unsigned long long* __restrict__ buf, size_t n)
{
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        bool ok = true;
        buf[q] = fx::bits_of(fx::from_fixed(buf[q], ok));
    }
}

template <bool OM_GE1>
cudaError_t launch_fxs(const unsigned long long* src, unsigned long long* dst, const Geom& g, const FxConst& c, int j,
                       int n, int* fail, cudaStream_t s)
{
    const dim3 grid((g.nz + kStepBlock - 1) / kStepBlock, g.ny, g.nx);
    const bool in_fx = j > 1, out_fx = j < n;
    if (in_fx && out_fx) k_step_fxs<OM_GE1, true, true><<<grid, kStepBlock, 0, s>>>(src, dst, g, c, j, fail);
    else if (in_fx) k_step_fxs<OM_GE1, true, false><<<grid, kStepBlock, 0, s>>>(src, dst, g, c, j, fail);
    else if (out_fx) k_step_fxs<OM_GE1, false, true><<<grid, kStepBlock, 0, s>>>(src, dst, g, c, j, fail);
    else k_step_fxs<OM_GE1, false, false><<<grid, kStepBlock, 0, s>>>(src, dst, g, c, j, fail);
    return cudaGetLastError();
}

// Native float64 redo of one cell of a staged row.
__device__ __noinline__ void fallback_staged(const double* __restrict__ st, int astride, int nz, int z, CollideF64 cp,
                                             double* __restrict__ dst, size_t plane, size_t rowoff,
                                             unsigned long long* fallback)
{
    const int zm = z == 0 ? nz - 1 : z - 1, zp = z == nz - 1 ? 0 : z + 1;
    double h[kQ];
#pragma unroll
    for (int a = 0; a < kQ; ++a) h[a] = st[a * astride + pull_z(ex(a, 2), z, zm, zp)];
    collide_f64(h, cp);
#pragma unroll
    for (int a = 0; a < kQ; ++a) dst[(size_t)a * plane + rowoff + z] = h[a];
    atomicAdd(fallback, 1ull);
}

// Row-kernel engine: fixed-point collision of one staged cell.
template <bool OM_GE1, int MINB>
struct EngFx {
    using T = double;
    static constexpr int kMinBlocks = MINB;
    FxConst c;
    CollideF64 cp;
    unsigned long long* fallback;

    __device__ __forceinline__ void run(const double* __restrict__ st, int astride, int nz, int z,
                                        double* __restrict__ dst, size_t plane, size_t rowoff) const
    {
        const int zm = z == 0 ? nz - 1 : z - 1, zp = z == nz - 1 ? 0 : z + 1;
        double f[kQ];
#pragma unroll
        for (int a = 0; a < kQ; ++a) f[a] = st[a * astride + pull_z(ex(a, 2), z, zm, zp)];
        bool ok = true;
        double out[kQ];
        fx::collide_cell<OM_GE1>(f, out, c, ok);
#pragma unroll
        for (int a = 0; a < kQ; ++a) dst[(size_t)a * plane + rowoff + z] = out[a];
        if (!ok) fallback_staged(st, astride, nz, z, cp, dst, plane, rowoff, fallback);
    }
};

}  // namespace

bool rows_fx_eligible(const Geom& g) { return rows_eligible<double>(g); }

cudaError_t launch_rows_fx(const double* src, double* dst, const Geom& g, const FxParams& fx, const CollideF64& cp,
                           unsigned long long* fallback, const RowConfig& rc, unsigned* err, cudaStream_t s)
{
    // One resident CTA per SM lets the compiler keep the whole cell in
    // registers; two cap it at 128 registers per thread.
    if (rc.ctas_per_sm <= 1)
        return fx.om_ge1 ? launch_rows(src, dst, g, EngFx<true, 1>{fx.k, cp, fallback}, rc, err, s)
                         : launch_rows(src, dst, g, EngFx<false, 1>{fx.k, cp, fallback}, rc, err, s);
    return fx.om_ge1 ? launch_rows(src, dst, g, EngFx<true, 2>{fx.k, cp, fallback}, rc, err, s)
                     : launch_rows(src, dst, g, EngFx<false, 2>{fx.k, cp, fallback}, rc, err, s);
}

cudaError_t launch_step_fx(int mode, const double* src, double* dst, const Geom& g, const FxParams& fx,
                           const CollideF64& cp, unsigned long long* fallback, cudaStream_t s)
{
    // Streaming alone moves values and is engine-independent.
    if (mode == kModeStream) return launch_step_f64(mode, src, dst, g, cp, s);
    const dim3 grid((g.nz + kStepBlock - 1) / kStepBlock, g.ny, g.nx);
    if (mode == kModeCollide) {
        if (src != dst) return cudaErrorInvalidValue;  // the collision is in place
        if (fx.om_ge1) k_collide_fx<true><<<grid, kStepBlock, 0, s>>>(dst, g, fx.k, cp, fallback);
        else k_collide_fx<false><<<grid, kStepBlock, 0, s>>>(dst, g, fx.k, cp, fallback);
        return cudaGetLastError();
    }
    if (fx.om_ge1)
        k_step_fx<true><<<grid, kStepBlock, 0, s>>>(src, dst, g, fx.k, cp, fallback);
    else
        k_step_fx<false><<<grid, kStepBlock, 0, s>>>(src, dst, g, fx.k, cp, fallback);
    return cudaGetLastError();
}

cudaError_t launch_step_fx_run(const double* src, double* dst, const Geom& g, const FxParams& fx, int j, int n,
                               int* fail, cudaStream_t s)
{
    if (j < 1 || j > n) return cudaErrorInvalidValue;
    const auto* in = reinterpret_cast<const unsigned long long*>(src);
    auto* out = reinterpret_cast<unsigned long long*>(dst);
    return fx.om_ge1 ? launch_fxs<true>(in, out, g, fx.k, j, n, fail, s)
                     : launch_fxs<false>(in, out, g, fx.k, j, n, fail, s);
}

cudaError_t launch_fx_to_f64(double* buf, size_t n, cudaStream_t s)
{
    k_fx_to_f64<<<current_sm_count() * 8, 256, 0, s>>>(reinterpret_cast<unsigned long long*>(buf), n);
    return cudaGetLastError();
}

namespace {

// Partial sums of {mass, px, py, pz, ke} (src/lbm.cpp:271-294), one partial
// per block.  A cell's 27 values are summed exactly as 64-bit fixed point
// (the collision's moments, fx_math.cuh) and each moment is rounded once to
// float64; a cell outside the exact range sums in float64 as the reference
// does.  Per-value float64 additions (~60 a cell on a float64 pipe of 1.67
// operations per clock per SM) made this reduction 3.7 ms at 256^3, three
// steps' worth.
template <bool PULL>
__global__ void __launch_bounds__(kStepBlock) k_conserved_fx(const double* __restrict__ src, Geom g,
                                                             double* __restrict__ partial)
{
    __shared__ double smem[32 * 5];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y, i = blockIdx.z;
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (k < g.nz) {
        const PullIndex pi(g, i, j, k, PULL);
        double f[kQ];
        gather27<double>(src, g, pi, f);
        bool ok = true;
        uint64_t X[kQ];
#pragma unroll
        for (int a = 0; a < kQ; ++a) X[a] = fx::to_fixed(f[a], a == 0 ? 8u : 5u, ok);
        double pl, ul, vl, wl;
        if (ok) {  // f_0 < 1, others < 1/8: every unsigned sum below 2^64
            uint64_t S = 0, P[3] = {0, 0, 0}, M[3] = {0, 0, 0};
#pragma unroll
            for (int a = 0; a < kQ; ++a) {
                S += X[a];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    if (ex(a, d) == 1) P[d] += X[a];
                    if (ex(a, d) == -1) M[d] += X[a];
                }
            }
            constexpr double scale = 1.0 / (double)(1ull << fx::kFrac);
            pl = __ull2double_rn(S) * scale;
            ul = __ll2double_rn((long long)(P[0] - M[0])) * scale;
            vl = __ll2double_rn((long long)(P[1] - M[1])) * scale;
            wl = __ll2double_rn((long long)(P[2] - M[2])) * scale;
        } else {
            pl = ul = vl = wl = 0.0;
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

}  // namespace

cudaError_t launch_conserved_fx(bool pull, const double* src, const Geom& g, const FxParams&, double* partial,
                                double* out, cudaStream_t s)
{
    const dim3 grid((g.nz + kStepBlock - 1) / kStepBlock, g.ny, g.nx);
    if (pull)
        k_conserved_fx<true><<<grid, kStepBlock, 0, s>>>(src, g, partial);
    else
        k_conserved_fx<false><<<grid, kStepBlock, 0, s>>>(src, g, partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_reduce_partials(partial, conserved_partials(g), out, s);
}

}  // namespace imex
