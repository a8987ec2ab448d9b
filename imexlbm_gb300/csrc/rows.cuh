// Row-staged fused step of the float64 fixed-point engine (the reduced-
// precision formats have their own, rows_lowp.cuh): persistent CTAs stream
// blocks of source rows through a multi-stage shared-memory ring with
// asynchronous bulk copies.
//
// The pull of cell (x, y, z) along direction a reads row (x - ex, y - ey) of
// plane a, shifted by ez along z.  A work item is B consecutive destination
// rows (x, y0 .. y0+B-1); for each direction their source rows are B
// consecutive rows of one plane - one contiguous run of B*nz values, or two
// where the periodic wrap in y splits it - so 27 to 54 bulk copies bring a
// whole item into shared memory.  The z shift and its periodic wrap are
// applied when reading shared memory.  The copies for item t + S - 1 are in
// flight while item t is computed, so HBM latency is hidden by the copy
// engine rather than by registers and resident warps; each source value is
// still read from HBM exactly once per step.
//
// Measured on GB300 (256^3 float32, copies only): issuing the 27 copies of
// a row from the lanes of one warp serialises them (~50 ns each, 3.1 TB/s);
// spreading them over the CTA's warps and staging B = 2..4 rows per copy
// reaches 7.2 TB/s of reads.  So every warp issues a few directions' copies.
//
// Requirements: nz * sizeof(T) a multiple of 16 bytes (bulk-copy
// granularity), B dividing ny, S * 27 * B * nz * sizeof(T) bytes of shared
// memory per CTA.
//
// Engine interface (EngFx, kernels_fx.cu):
//   using T;                                    storage element type
//   static constexpr int kMinBlocks;            resident CTAs of 256 threads
//                                               the registers must allow
//   __device__ void run(const T* st, int astride, int nz, int z, T* dst,
//                       size_t plane, size_t rowoff) const;
//       collide cell z of a staged row - direction a's source row is
//       st + a * astride - and store its 27 outputs at dst + a * plane +
//       rowoff + z
#pragma once

#include <cuda_runtime.h>

#include "bulk.cuh"
#include "kernels_common.cuh"

namespace imex {

constexpr int kRowThreadsMax = 256;
constexpr int kRowBarrierBytes = 128;  // room for up to 16 mbarriers

// Offset of the source z for direction a: the value pulled into z comes from
// z - ez (wrapped).  Returns the index into the stage row.
__device__ __forceinline__ int pull_z(int ez, int z, int zm, int zp) { return ez == 1 ? zm : ez == -1 ? zp : z; }

template <class E>
__global__ void __launch_bounds__(kRowThreadsMax, E::kMinBlocks)
    k_rows(const typename E::T* __restrict__ src, typename E::T* __restrict__ dst, Geom g, E eng, int stages, int B,
           WaitCtl wc)
{
    using T = typename E::T;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
    T* ring = reinterpret_cast<T*>(smem_raw + kRowBarrierBytes);
    const int nz = g.nz;
    const int astride = B * nz;                 // one direction's B rows
    const size_t stage_elems = (size_t)kQ * astride;
    const uint32_t row_bytes = (uint32_t)(nz * sizeof(T));
    const int yblocks = g.ny / B;
    const int items = g.nx * yblocks;
    const int G = gridDim.x;
    const int my = (int)blockIdx.x < items ? (items - 1 - (int)blockIdx.x) / G + 1 : 0;
    // Copy issue: lane l < ceil(27 / warps) of warp w handles direction w + warps * l.
    const int nwarps = blockDim.x >> 5;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int my_dir = warp + nwarps * lane;
    const bool issuer = lane * nwarps < kQ && my_dir < kQ;

    auto arm = [&](int t) {
        bulk::mbar_arrive_expect_tx(&full[t % stages], (uint32_t)kQ * B * row_bytes);
    };
    auto issue = [&](int t) {
        if (!issuer) return;
        if (t == 0 && (int)blockIdx.x == wc.starve_cta) return;  // test hook: stage 0 never fills
        const int item = (int)blockIdx.x + t * G;
        const int x = item / yblocks, y0 = (item - x * yblocks) * B;
        const int a = my_dir;
        int xs = x - ex(a, 0);
        xs = xs < 0 ? xs + g.nx : xs >= g.nx ? xs - g.nx : xs;
        const T* plane = src + (size_t)a * g.plane + (size_t)xs * g.ny * nz;
        T* st = ring + (size_t)(t % stages) * stage_elems + (size_t)a * astride;
        uint64_t* bar = &full[t % stages];
        const int lo = y0 - ex(a, 1);  // source row of the item's first row
        if (lo < 0) {                  // first row wraps to ny - 1
            bulk::copy_g2s(st, plane + (size_t)(g.ny - 1) * nz, row_bytes, bar);
            if (B > 1) bulk::copy_g2s(st + nz, plane, (uint32_t)(B - 1) * row_bytes, bar);
        } else if (lo + B > g.ny) {    // last row wraps to 0
            if (B > 1) bulk::copy_g2s(st, plane + (size_t)lo * nz, (uint32_t)(B - 1) * row_bytes, bar);
            bulk::copy_g2s(st + (size_t)(B - 1) * nz, plane, row_bytes, bar);
        } else {
            bulk::copy_g2s(st, plane + (size_t)lo * nz, (uint32_t)B * row_bytes, bar);
        }
    };

    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; ++s) bulk::mbar_init(&full[s], 1);
        bulk::fence_mbar_init();
        for (int t = 0; t < stages && t < my; ++t) arm(t);  // first item of every stage
    }
    __syncthreads();
    for (int t = 0; t < stages - 1 && t < my; ++t) issue(t);

    for (int t = 0; t < my; ++t) {
        // Item t + S - 1 goes into the stage item t - 1 used; the barrier at
        // the end of iteration t - 1 released it and thread 0 armed it.
        if (t + stages - 1 < my) issue(t + stages - 1);
        const int s = t % stages;
        const int ok = bulk::mbar_wait(&full[s], (uint32_t)((t / stages) & 1), wc.cycles);
        if (__syncthreads_or(!ok)) {
            // A copy did not complete: record it, wait (bounded) for the
            // copies this CTA still has in flight, and stop.
            if (threadIdx.x == 0) {
                atomicOr(wc.err, 1u);
                const int last = t + stages - 1 < my ? t + stages - 1 : my - 1;
                for (int q = t; q <= last; ++q)
                    bulk::mbar_wait(&full[q % stages], (uint32_t)((q / stages) & 1), wc.cycles);
            }
            __syncthreads();
            return;
        }
        const int item = (int)blockIdx.x + t * G;
        const int x = item / yblocks, y0 = (item - x * yblocks) * B;
        const T* st = ring + (size_t)s * stage_elems;
        for (int b = 0; b < B; ++b) {
            const size_t rowoff = ((size_t)x * g.ny + y0 + b) * nz;
            for (int z = threadIdx.x; z < nz; z += blockDim.x)
                eng.run(st + (size_t)b * nz, astride, nz, z, dst, g.plane, rowoff);
        }
        if (threadIdx.x == 0 && t + stages < my) arm(t + stages);  // stage s, next use
        __syncthreads();  // stage s may be refilled
    }
}

// Shared memory of one CTA for `stages` stages of B rows of nz values of T.
template <class T>
size_t rows_smem_bytes(int nz, int stages, int B)
{
    return kRowBarrierBytes + (size_t)stages * kQ * B * nz * sizeof(T);
}

// Whether the row-staged kernel applies to rows of nz values of T.
template <class T>
bool rows_eligible(const Geom& g)
{
    return (g.nz * sizeof(T)) % 16 == 0 && rows_smem_bytes<T>(g.nz, 2, 1) <= 227 * 1024 &&
           (size_t)g.nx * g.ny < 0x7fffffffu;
}

// Row-kernel launch shape.
struct RowConfig {
    int stages = 0;        // ring depth (0: not the row kernel)
    int rows = 1;          // B: consecutive y-rows per stage (divides ny for float64)
    int ctas_per_sm = 0;   // resident CTAs per SM (grid = SMs * this)
    int threads = 0;       // threads per CTA
    int dir_bytes = 0;     // reduced precision: bytes per direction in a stage
};

template <class E>
cudaError_t launch_rows(const typename E::T* src, typename E::T* dst, const Geom& g, const E& eng, const RowConfig& rc,
                        unsigned* err, cudaStream_t s)
{
    using T = typename E::T;
    const int sms = current_sm_count();
    const size_t smem = rows_smem_bytes<T>(g.nz, rc.stages, rc.rows);
    cudaError_t e = cudaFuncSetAttribute(k_rows<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (rc.rows < 1 || g.ny % rc.rows) return cudaErrorInvalidValue;
    const long long items = (long long)g.nx * (g.ny / rc.rows);
    long long grid = (long long)sms * rc.ctas_per_sm;
    if (grid > items) grid = items;
    k_rows<E><<<(unsigned)grid, rc.threads, smem, s>>>(src, dst, g, eng, rc.stages, rc.rows, make_wait_ctl(err));
    return cudaGetLastError();
}

}  // namespace imex
