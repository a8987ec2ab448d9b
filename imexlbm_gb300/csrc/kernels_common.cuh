// Shared device code: lattice geometry, periodic pull gather, block
// reductions.  Used by every engine's kernels.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

#include "d3q27.cuh"

namespace imex {

// Lattice of nx*ny*nz cells stored as f[a][x][y][z], z fastest; one
// direction plane holds nx*ny*nz values.
struct Geom {
    int nx, ny, nz;
    size_t plane;
};

// Threads of the step kernels: one block covers `kStepBlock` consecutive z
// cells of one (x, y) row; grid = (ceil(nz / kStepBlock), ny, nx).
constexpr int kStepBlock = 128;

// SM count of the calling thread's current device, for persistent grids.
// Queried per call: the runtime answers from its own cache, and a process
// that drives several devices gets each one's count.
inline int current_sm_count()
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) return 1;
    return sms;
}

// Source indices of the pull for cell (i, j, k): the value streaming into
// the cell along direction a comes from (i - ex, j - ey, k - ez), wrapped
// periodically.  This is the one-rank image of the reference's ghost layer
// (src/mpi_view_transfer.cpp:260-456 fills ghost cells with the periodic
// image; src/lbm.cpp:194-195 pulls from x - e).
struct PullIndex {
    size_t row[3][3];  // [ex + 1][ey + 1] -> offset of source row (x, y)
    int zk[3];         // [ez + 1] -> source z

    __device__ __forceinline__ PullIndex(const Geom& g, int i, int j, int k, bool pull)
    {
        const int im = i == 0 ? g.nx - 1 : i - 1, ip = i == g.nx - 1 ? 0 : i + 1;
        const int jm = j == 0 ? g.ny - 1 : j - 1, jp = j == g.ny - 1 ? 0 : j + 1;
        const int km = k == 0 ? g.nz - 1 : k - 1, kp = k == g.nz - 1 ? 0 : k + 1;
        // ex = +1 pulls from x - 1, ex = -1 from x + 1.
        const int xs[3] = {pull ? ip : i, i, pull ? im : i};
        const int ys[3] = {pull ? jp : j, j, pull ? jm : j};
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b)
                row[a][b] = ((size_t)xs[a] * g.ny + ys[b]) * g.nz;
        zk[0] = pull ? kp : k;
        zk[1] = k;
        zk[2] = pull ? km : k;
    }

    template <int A>
    __device__ __forceinline__ size_t at(const Geom& g) const
    {
        return (size_t)A * g.plane + row[ex(A, 0) + 1][ex(A, 1) + 1] + zk[ex(A, 2) + 1];
    }

    // Same for a direction that is a compile-time constant only after
    // unrolling.
    __device__ __forceinline__ size_t at_dyn(const Geom& g, int a) const
    {
        return (size_t)a * g.plane + row[ex(a, 0) + 1][ex(a, 1) + 1] + zk[ex(a, 2) + 1];
    }
};

template <int A, typename T>
__device__ __forceinline__ T ldg_pull(const T* __restrict__ src, const Geom& g, const PullIndex& p)
{
    return __ldg(src + p.at<A>(g));
}

// Unrolled gather of the 27 pulled (or in-place) values.
template <typename T, int A = 0>
__device__ __forceinline__ void gather27(const T* __restrict__ src, const Geom& g, const PullIndex& p, T (&f)[kQ])
{
    if constexpr (A < kQ) {
        f[A] = ldg_pull<A>(src, g, p);
        gather27<T, A + 1>(src, g, p, f);
    }
}

// Deterministic block sum of NV doubles: warp shuffle tree, then the warps'
// results in warp order.  Result valid in thread 0.  blockDim.x <= 1024.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* smem /* 32*NV */)
{
#pragma unroll
    for (int q = 0; q < NV; ++q)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) smem[warp * NV + q] = v[q];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = 0.0;
            for (int w = 0; w < nw; ++w) s += smem[w * NV + q];
            v[q] = s;
        }
    }
}

}  // namespace imex
