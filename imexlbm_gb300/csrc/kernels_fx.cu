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

// ------------------------------------------------------ two steps a pass --
// Two fused steps in one pass over HBM.  Phase A of a row (x, y) pulls
// rows (x - ex, y - ey) of the source lattice and writes its collided
// values (step j) into a ring of x-planes in device memory; phase B of row
// (x, y) pulls from the ring and writes step j + 1 into the destination.
// The ring - two pinned planes (x = 0 and 1, which the last rows of phase B
// read) and R recycled ones - is meant to stay in L2, so per two cell
// updates HBM sees one read of the source and one write of the destination
// instead of two of each.
//
// Order.  CTAs take tickets from a counter; a ticket names one row of one
// phase: A rows in x-major order, B rows (planes 1 .. nx-1, then plane 0;
// in a plane rows 1 .. ny-1, then row 0, whose pull wraps to row ny-1)
// interleaved `lag` tickets behind.  B(x, y) needs A of rows (x +- 1,
// y +- 1); A(x, y) of a recycled ring slot needs B of the rows of planes
// x - R - 1 .. x - R + 1 that read it.  With lag = (R + 1) ny / 2 + 2 both
// kinds of wait are on tickets at least about (R - 3) ny / 2 earlier (the
// slack the tickets in flight need before a wait becomes a stall), and every row a
// ticket waits for has a smaller ticket (checked on the host for R 4..16
// and a range of shapes with lag <= nx ny).  A waiting CTA reads the rows'
// flags (the launch's epoch once the row is written) with acquire semantics,
// one flag per lane of its first warp; a CTA publishes a row by a
// __syncthreads, a fence and a release store of its flag.  The rows waited
// for are held by CTAs that took their tickets earlier and are running (a
// CTA takes its next ticket while it works on the current one, which still
// leaves the smallest unfinished ticket free to proceed), so every wait
// ends; each is bounded all the same, and one that runs out sets the error
// flag and ends the CTA.  Ring values are read with ld.global.cg (L2, never
// a stale L1 line of a recycled slot).  The cell arithmetic is k_step_fxs's,
// fixed point in and out, so the results are those of two single launches,
// bit for bit.
__device__ __forceinline__ int ld_acquire(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int* p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Ring slot of x-plane x.
__device__ __forceinline__ int two_slot(int x, int R) { return x < 2 ? x : 2 + (x - 2) % R; }

// L2 policy that keeps the ring's lines in L2 ahead of the streams of the
// source and the destination.
__device__ __forceinline__ uint64_t l2_keep_policy()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ uint64_t ld_ring(const unsigned long long* p, uint64_t pol)
{
    uint64_t v;
    asm volatile("ld.global.cg.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(v) : "l"(p), "l"(pol));
    return v;
}

__device__ __forceinline__ void st_ring(unsigned long long* p, uint64_t v, uint64_t pol)
{
    asm volatile("st.global.cg.L2::cache_hint.u64 [%0], %1, %2;" ::"l"(p), "l"(v), "l"(pol) : "memory");
}

template <bool OM_GE1, int MINB>
__global__ void __launch_bounds__(kStepBlock, MINB)
    k_two_fxs(const unsigned long long* __restrict__ src, unsigned long long* __restrict__ dst, Geom g, FxConst c,
              TwoStepCtl ts, int j, int* __restrict__ fail)
{
    __shared__ int s_next[2], s_abort;
    if (*fail < j) return;  // an earlier step of the run failed
    const int nx = g.nx, ny = g.ny, nz = g.nz, R = ts.ring;
    const int N = nx * ny, L = ts.lag, T = 2 * N;
    const size_t mplane = (size_t)(R + 2) * ny * nz;  // ring values per direction
    unsigned long long* mid = ts.mid;
    const uint64_t keep = l2_keep_policy();
    if (threadIdx.x == 0) {
        s_next[0] = (int)atomicAdd(ts.counter, 1u);
        s_abort = 0;
    }
    __syncthreads();
    int t = s_next[0];
    for (int it = 1; t < T; it ^= 1) {
        // the next ticket, taken now so that its latency hides behind this row
        int next = 0;
        if (threadIdx.x == 0) next = (int)atomicAdd(ts.counter, 1u);
        // the ticket's phase and row
        bool isA;
        int r;
        if (t < L) { isA = true; r = t; }
        else if (t < T - L) { const int u = t - L; isA = u & 1; r = isA ? L + (u >> 1) : (u >> 1); }
        else { isA = false; r = t - N; }
        int x, y;
        if (isA) {
            x = r / ny;
            y = r - x * ny;
        } else {  // planes 1 .. nx-1 then 0; in a plane rows 1 .. ny-1 then 0
            const int p = r / ny, q = r - p * ny;
            x = p < nx - 1 ? p + 1 : 0;
            y = q < ny - 1 ? q + 1 : 0;
        }
        // wait for the rows this one reads (B) or whose ring slot it reuses (A):
        // lane i of warp 0 watches row (x0 + i / 3, y - 1 + i % 3)
        if (threadIdx.x < 32 && (!isA || x >= R + 2)) {
            const int lane = threadIdx.x;
            const int* f = nullptr;
            if (lane < 9) {
                int xx = (isA ? x - R - 1 : x - 1) + lane / 3;
                xx = xx < 0 ? xx + nx : xx >= nx ? xx - nx : xx;
                int yy = y - 1 + lane % 3;
                yy = yy < 0 ? yy + ny : yy >= ny ? yy - ny : yy;
                f = (isA ? ts.flag_b : ts.flag_a) + (size_t)xx * ny + yy;
            }
            const long long t0 = clock64();
            bool timed_out = false;
            for (;;) {
                const bool mine = lane >= 9 || ld_acquire(f) == ts.epoch;
                if (__all_sync(0xffffffffu, mine)) break;
                if (__any_sync(0xffffffffu, clock64() - t0 > ts.cycles)) {
                    timed_out = true;
                    break;
                }
            }
            if (timed_out && lane == 0) {
                atomicOr(ts.err, 1u);
                s_abort = 1;
            }
        }
        __syncthreads();
        if (s_abort) return;
        const int xm = x == 0 ? nx - 1 : x - 1, xp = x == nx - 1 ? 0 : x + 1;
        const int ym = y == 0 ? ny - 1 : y - 1, yp = y == ny - 1 ? 0 : y + 1;
        // source planes by e + 1 (the pull reads x - e): lattice planes for A, ring slots for B
        const int ps[3] = {isA ? xp : two_slot(xp, R), isA ? x : two_slot(x, R), isA ? xm : two_slot(xm, R)};
        for (int k = threadIdx.x; k < nz; k += blockDim.x) {
            const int km = k == 0 ? nz - 1 : k - 1, kp = k == nz - 1 ? 0 : k + 1;
            const int ys[3] = {yp, y, ym}, zs[3] = {kp, k, km};
            uint64_t in[kQ], out[kQ];
            if (isA) {
#pragma unroll
                for (int a = 0; a < kQ; ++a)
                    in[a] = __ldg(src + (size_t)a * g.plane +
                                  ((size_t)ps[ex(a, 0) + 1] * ny + ys[ex(a, 1) + 1]) * nz + zs[ex(a, 2) + 1]);
            } else {
#pragma unroll
                for (int a = 0; a < kQ; ++a)
                    in[a] = ld_ring(mid + (size_t)a * mplane +
                                        ((size_t)ps[ex(a, 0) + 1] * ny + ys[ex(a, 1) + 1]) * nz + zs[ex(a, 2) + 1],
                                    keep);
            }
            bool ok = true;
            fx::collide_cell_io<OM_GE1, true, true>(in, out, c, ok);
            if (isA) {
                const size_t cell = ((size_t)two_slot(x, R) * ny + y) * nz + k;
#pragma unroll
                for (int a = 0; a < kQ; ++a) st_ring(mid + (size_t)a * mplane + cell, out[a], keep);
            } else {
                const size_t cell = ((size_t)x * ny + y) * nz + k;
#pragma unroll
                for (int a = 0; a < kQ; ++a) __stcs(dst + (size_t)a * g.plane + cell, out[a]);
            }
            if (!ok) atomicMin(fail, j);
        }
        // s_next[it] was last read before this ticket's wait barrier
        if (threadIdx.x == 0) s_next[it] = next;
        __syncthreads();  // every value of the row is stored; the next ticket is shared
        if (threadIdx.x == 0)  // release: cumulative over the CTA's stores ordered by the barrier
            st_release((isA ? ts.flag_a : ts.flag_b) + (size_t)x * ny + y, ts.epoch);
        t = s_next[it];
    }
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

int two_step_lag(const Geom& g, int ring) { return (ring + 1) * g.ny / 2 + 2; }

bool two_step_eligible(const Geom& g, int ring)
{
    return ring >= kTwoRingMin && ring <= kTwoRingMax && g.nx >= 8 && g.ny >= 4 && (size_t)g.nx * g.ny < (1u << 30) &&
           (size_t)two_step_lag(g, ring) <= (size_t)g.nx * g.ny;
}

size_t two_step_ring_values(const Geom& g, int ring) { return (size_t)kQ * (ring + 2) * g.ny * g.nz; }

cudaError_t launch_two_step_fx(const double* src, double* dst, const Geom& g, const FxParams& fx, const TwoStepCtl& ts,
                               int ctas_per_sm, int j, int* fail, cudaStream_t s)
{
    if (!two_step_eligible(g, ts.ring) || ts.lag != two_step_lag(g, ts.ring) || ctas_per_sm < 1 || ctas_per_sm > 6)
        return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(ts.counter, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    // persistent: at most the CTAs that can be resident (6 per SM: the
    // instantiation held to 80 registers; up to 5: the one at 96)
    const unsigned grid = (unsigned)(current_sm_count() * ctas_per_sm);
    const auto* in = reinterpret_cast<const unsigned long long*>(src);
    auto* out = reinterpret_cast<unsigned long long*>(dst);
    if (ctas_per_sm == 6) {
        if (fx.om_ge1) k_two_fxs<true, 6><<<grid, kStepBlock, 0, s>>>(in, out, g, fx.k, ts, j, fail);
        else k_two_fxs<false, 6><<<grid, kStepBlock, 0, s>>>(in, out, g, fx.k, ts, j, fail);
    } else {
        if (fx.om_ge1) k_two_fxs<true, 5><<<grid, kStepBlock, 0, s>>>(in, out, g, fx.k, ts, j, fail);
        else k_two_fxs<false, 5><<<grid, kStepBlock, 0, s>>>(in, out, g, fx.k, ts, j, fail);
    }
    return cudaGetLastError();
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
