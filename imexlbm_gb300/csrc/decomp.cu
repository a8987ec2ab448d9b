// Spatial decomposition of one lattice into sub-domains - the reference's
// multi-rank layout (src/mpi_view_transfer.cpp) - held on one GPU.
//
// Plan (host, no GPU needed).  The rank grid rx x ry x rz is the reference's
// setup_Cartesian choice (src/mpi_view_transfer.cpp:53-95): among the
// factorisations of the rank count, in ascending (rx, ry) order, the first
// whose integer block extents nx/rx, ny/ry, nz/rz have the least spread
// about their mean.  Ranks are numbered me = px + rx*pz + rx*rz*py (:97-99)
// and own blocks of the closed-form distribution of setup_Local (:163-195):
// coordinates below n mod r own one cell more.  The 26 halo channels follow
// the reference's face / edge / corner tables (:101-161) in its order; a
// channel carries only the directions that cross it - 9 for a face, 3 for an
// edge, 1 for a corner (the pruning its Aurora notes propose,
// machines/aurora/README.md:79-82, and the unused d_dirset of src/lbm.hpp:153).
//
// Sub-domains (device).  Each block keeps its distributions in a padded box
// f[a][Lx+2][Ly+2][P] with a one-cell ghost shell (the reference keeps 3
// ghost layers and fills one, src/mpi_view_transfer.cpp:197-200; P pads a
// z-row so that its interior starts on a 32-byte sector).  The state machine
// is the single lattice's: the buffers hold C(f) with the streaming pending,
// and a step is one launch over every block of the fused pull + collision
// (the fixed-point engine's cell arithmetic; runs of steps hold the state as
// fixed point between launches, as the undivided lattice's do), reading the
// ghost shell where the pull leaves the block.  The halo exchange is part of
// the same launch: a boundary cell's new values that leave its block - the
// pruned directions of each channel only - are stored straight into the
// ghost shell of the block they stream into (push_halo), the one-GPU image
// of pack_f / exchange_f / unpack_f (src/mpi_view_transfer.cpp:260-456),
// whose sends would be peer stores over NVLink across several GPUs.
// Collision is per cell and streaming a permutation, so every f is bit-
// identical to the undivided lattice's whatever the decomposition
// (tests/test_decomp_gpu.py); only the order of the conserved sums differs,
// as it does across the reference's rank counts.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "collide_f64.cuh"
#include "fx_math.cuh"
#include "fx_params.hpp"
#include "imexlbm.h"
#include "imexlbm_internal.hpp"
#include "kernels_f64.cuh"
#include "kernels_fx.cuh"
#include "tg_init.cuh"

namespace imex {
namespace {

// ------------------------------------------------------------------ plan --

// Offsets (x, y, z) of the 26 channels in the reference's order: faces
// left, right, down, up, front, back (x is left/right, z down/up, y
// front/back; src/mpi_view_transfer.cpp:101-107), edges :109-121, corners
// :123-131.
constexpr int kChannel[26][3] = {
    {-1, 0, 0}, {1, 0, 0}, {0, 0, -1}, {0, 0, 1}, {0, -1, 0}, {0, 1, 0},                 // faces
    {-1, 0, 1}, {1, 0, 1}, {-1, 0, -1}, {1, 0, -1}, {0, -1, 1}, {0, -1, -1},             // edges
    {0, 1, 1}, {0, 1, -1}, {1, -1, 0}, {-1, -1, 0}, {1, 1, 0}, {-1, 1, 0},
    {1, 1, -1}, {1, -1, -1}, {1, -1, 1}, {1, 1, 1}, {-1, -1, 1}, {-1, 1, -1},            // corners
    {-1, -1, -1}, {-1, 1, 1}};

struct Plan {
    int n[3] = {0, 0, 0};
    int grid[3] = {1, 1, 1};
    int nranks = 1;
};

int plan_grid(int nranks, const int n[3], int grid[3])
{
    double best = 1e300;
    int found = 0;
    for (int i = 1; i <= nranks; ++i) {
        if (nranks % i) continue;
        for (int j = 1; j <= nranks / i; ++j) {
            if ((nranks / i) % j) continue;
            const int k = nranks / i / j;
            const double bx = n[0] / i, by = n[1] / j, bz = n[2] / k;  // integer extents, as doubles
            const double mean = (bx + by + bz) / 3.0;
            const double spread = (bx - mean) * (bx - mean) + (by - mean) * (by - mean) + (bz - mean) * (bz - mean);
            if (spread < best) {
                best = spread;
                grid[0] = i;
                grid[1] = j;
                grid[2] = k;
                found = 1;
            }
        }
    }
    return found;
}

void rank_coords(const int grid[3], int rank, int c[3])
{
    c[0] = rank % grid[0];
    c[2] = (rank / grid[0]) % grid[2];
    c[1] = rank / grid[0] / grid[2];
}

int rank_of(const int grid[3], const int c[3]) { return c[0] + grid[0] * c[2] + grid[0] * grid[2] * c[1]; }

void block_of(const Plan& p, int rank, imex_block* b)
{
    b->rank = rank;
    rank_coords(p.grid, rank, b->coord);
    for (int d = 0; d < 3; ++d) {
        const int base = p.n[d] / p.grid[d], rem = p.n[d] % p.grid[d], c = b->coord[d];
        b->len[d] = base + (c < rem ? 1 : 0);
        b->lo[d] = c * base + std::min(c, rem);
    }
}

int neighbour(const Plan& p, const imex_block& b, const int off[3])
{
    int c[3];
    for (int d = 0; d < 3; ++d) c[d] = ((b.coord[d] + off[d]) % p.grid[d] + p.grid[d]) % p.grid[d];
    return rank_of(p.grid, c);
}

void halo_msg(const Plan& p, int rank, int ch, imex_halo_msg* m)
{
    imex_block b;
    block_of(p, rank, &b);
    const int* o = kChannel[ch];
    const int back[3] = {-o[0], -o[1], -o[2]};
    m->channel = ch;
    for (int d = 0; d < 3; ++d) m->offset[d] = o[d];
    m->send_to = neighbour(p, b, o);
    m->recv_from = neighbour(p, b, back);
    for (int d = 0; d < 3; ++d) {
        // boundary layer on side o (padded coordinates: 0 and len+1 are ghosts)
        m->send_lo[d] = o[d] == -1 ? 1 : o[d] == 1 ? b.len[d] : 1;
        // ghost layer on side -o, filled by the neighbour behind us
        m->recv_lo[d] = o[d] == -1 ? b.len[d] + 1 : o[d] == 1 ? 0 : 1;
        m->ext[d] = o[d] == 0 ? b.len[d] : 1;
    }
    // directions that travel along the channel: e_a matches o on its non-zero axes
    m->ndir = 0;
    for (int a = 0; a < kQ; ++a) {
        bool along = true;
        for (int d = 0; d < 3; ++d)
            if (o[d] != 0 && ex(a, d) != o[d]) along = false;
        if (along) m->dirs[m->ndir++] = a;
    }
    for (int q = m->ndir; q < 9; ++q) m->dirs[q] = -1;
}

int check_plan_args(int nranks, int nx, int ny, int nz, const char* what, Plan* p)
{
    if (nranks < 1 || nx < 1 || ny < 1 || nz < 1)
        return set_thread_error(IMEX_ERR_ARG, std::string(what) + ": nranks and the lattice sizes must be >= 1");
    p->nranks = nranks;
    p->n[0] = nx;
    p->n[1] = ny;
    p->n[2] = nz;
    if (!plan_grid(nranks, p->n, p->grid))
        return set_thread_error(IMEX_ERR_ARG, std::string(what) + ": no rank grid");
    for (int d = 0; d < 3; ++d)
        if (p->grid[d] > p->n[d])
            return set_thread_error(IMEX_ERR_ARG, std::string(what) + ": more ranks along an axis than cells");
    return IMEX_OK;
}

// ----------------------------------------------------------------- device --

constexpr int kThreads = 128;

// A block's padded box: interior extents L, the z pitch P of a row and the
// values per direction plane, (Lx+2)(Ly+2)P.  Padded z coordinate k (0: the
// ghost below, 1..Lz: interior, Lz+1: the ghost above) sits at kZOff + k in
// its row; with P a multiple of 4 the interior of every row starts on a
// 32-byte sector, so a warp's 32 values are 8 whole sectors.
constexpr int kZOff = 3;
static_assert(kZOff == 3, "push_halo stores the low z ghost as the last word of its row's first 32-byte sector");
struct PadGeom {
    int L[3];
    int P;
    size_t plane;
};

inline int pad_pitch(int Lz) { return (Lz + 2 + kZOff + 3) & ~3; }

// One block on the device: its buffers, geometry and the block next to it
// at each offset (ox, oy, oz) in {-1, 0, 1}^3 (periodic; itself along an axis
// the grid does not split), entry (ox + 1) 9 + (oy + 1) 3 + (oz + 1).
struct BlockDev {
    double* buf[2];
    PadGeom g;
    int nb[27];
};

__host__ __device__ inline size_t pad_index(const PadGeom& b, int i, int j, int k)
{
    return ((size_t)i * (b.L[1] + 2) + j) * b.P + kZOff + k;
}

// The halo exchange, as stores from the producer.  When a step (or the
// first in-place collision) has the new values of a cell on its block's
// boundary, every value whose direction leaves the block - 9 through a face,
// 3 more through each edge, 1 through a corner: the reference's channels
// pruned to the directions that cross them - is also stored into the ghost
// shell of the block it streams into, at the ghost cell the next pull of
// that block reads (padded coordinate 0 when it enters the neighbour from
// below, L + 1 from above, unchanged along an axis it does not cross).  No
// exchange kernel, no pack buffer and no re-read of the boundary: on several
// GPUs these are the peer stores over NVLink that replace pack_f /
// exchange_f / unpack_f (src/mpi_view_transfer.cpp:260-456).  Interior
// cell (i, j, k) of block `self` (0-based), values v, ghost shells of
// buffer `buf`.
template <typename T>
__device__ __forceinline__ void push_halo(const BlockDev* __restrict__ blocks, int self, int buf, const PadGeom& g,
                                          int i, int j, int k, const T (&v)[kQ])
{
    const bool hx = i == g.L[0] - 1, lx = i == 0, hy = j == g.L[1] - 1, ly = j == 0, hz = k == g.L[2] - 1, lz = k == 0;
    const int faces = (int)hx + (int)lx + (int)hy + (int)ly + (int)hz + (int)lz;
    if (faces == 0) return;
    const int* nb = blocks[self].nb;
    if (faces == 1) {  // on one face only (most boundary cells): one neighbour, 9 values
        const int axis = (hx || lx) ? 0 : (hy || ly) ? 1 : 2;
        const int side = (hx || hy || hz) ? 1 : -1;
        const int o = axis == 0 ? (side + 1) * 9 + 4 : axis == 1 ? 9 + (side + 1) * 3 + 1 : 13 + side;
        const BlockDev& N = blocks[__ldg(&nb[o])];
        PadGeom ng;
        ng.L[0] = __ldg(&N.g.L[0]);
        ng.L[1] = __ldg(&N.g.L[1]);
        ng.L[2] = __ldg(&N.g.L[2]);
        ng.P = __ldg(&N.g.P);
        ng.plane = __ldg(&N.g.plane);
        int t[3] = {i + 1, j + 1, k + 1};
        t[axis] = side == 1 ? 0 : ng.L[axis] + 1;
        const size_t base = pad_index(ng, t[0], t[1], t[2]);
        T* dst = reinterpret_cast<T*>(N.buf[buf]);
        // A z-face ghost value is alone in its row's first (last) 32-byte
        // sector with pad words nothing reads; a single 8-byte store leaves
        // the sector partly written and costs a read-modify-write when it
        // leaves L2, so the whole sector is stored: the value and zeroed
        // pads, as two 16-byte stores.  The low ghost (padded z 0, word
        // kZOff of the row) always ends its row's first sector; the high one (word Lz + kZOff + 1) starts a sector when Lz is a
        // multiple of 4, the pitch then leaving three pad words after it.
        if (axis == 2 && (side == 1 || (ng.L[2] & 3) == 0)) {
            const size_t s0 = side == 1 ? base - kZOff : base;  // the sector's first word
#pragma unroll
            for (int a = 0; a < kQ; ++a)
                if (ex(a, 2) == side) {
                    unsigned long long w;
                    memcpy(&w, &v[a], sizeof w);
                    auto* q = reinterpret_cast<ulonglong2*>(dst + (size_t)a * ng.plane + s0);
                    q[0] = side == 1 ? make_ulonglong2(0ull, 0ull) : make_ulonglong2(w, 0ull);
                    q[1] = side == 1 ? make_ulonglong2(0ull, w) : make_ulonglong2(0ull, 0ull);
                }
            return;
        }
#pragma unroll
        for (int a = 0; a < kQ; ++a) {
            const int e = axis == 0 ? ex(a, 0) : axis == 1 ? ex(a, 1) : ex(a, 2);
            if (e == side) dst[(size_t)a * ng.plane + base] = v[a];
        }
        return;
    }
#pragma unroll
    for (int a = 0; a < kQ; ++a) {
        const int ox = (hx && ex(a, 0) == 1) ? 1 : (lx && ex(a, 0) == -1) ? -1 : 0;
        const int oy = (hy && ex(a, 1) == 1) ? 1 : (ly && ex(a, 1) == -1) ? -1 : 0;
        const int oz = (hz && ex(a, 2) == 1) ? 1 : (lz && ex(a, 2) == -1) ? -1 : 0;
        if (ox == 0 && oy == 0 && oz == 0) continue;
        const BlockDev& N = blocks[__ldg(&nb[(ox + 1) * 9 + (oy + 1) * 3 + (oz + 1)])];
        PadGeom ng;
        ng.L[0] = __ldg(&N.g.L[0]);
        ng.L[1] = __ldg(&N.g.L[1]);
        ng.L[2] = __ldg(&N.g.L[2]);
        ng.P = __ldg(&N.g.P);
        ng.plane = __ldg(&N.g.plane);
        const int tx = ox == 1 ? 0 : ox == -1 ? ng.L[0] + 1 : i + 1;
        const int ty = oy == 1 ? 0 : oy == -1 ? ng.L[1] + 1 : j + 1;
        const int tz = oz == 1 ? 0 : oz == -1 ? ng.L[2] + 1 : k + 1;
        T* dst = reinterpret_cast<T*>(N.buf[buf]);
        dst[(size_t)a * ng.plane + pad_index(ng, tx, ty, tz)] = v[a];
    }
}

// Padded source index of the value pulled into interior cell (I, J, K)
// (padded coordinates) along direction A: the cell at (I, J, K) - e_A.
template <int A>
__device__ __forceinline__ size_t pull_at(const PadGeom& b, int I, int J, int K)
{
    return (size_t)A * b.plane + pad_index(b, I - ex(A, 0), J - ex(A, 1), K - ex(A, 2));
}

template <int A = 0, typename T>
__device__ __forceinline__ void gather_pad(const T* __restrict__ src, const PadGeom& b, int I, int J, int K,
                                           T (&f)[kQ])
{
    if constexpr (A < kQ) {
        f[A] = __ldg(src + pull_at<A>(b, I, J, K));
        gather_pad<A + 1>(src, b, I, J, K, f);
    }
}

// Interior cell of a launch over every block (grid x: row segments of
// kThreads z-cells of the largest block, grid y: block): the block's
// geometry and padded coordinates (I, J, K) of this thread's cell; false
// for a thread past its block's cells.
struct DomCell {
    PadGeom g;
    int I, J, K;
};

__device__ __forceinline__ bool dom_cell(const BlockDev* __restrict__ blocks, DomCell& c)
{
    const BlockDev& B = blocks[blockIdx.y];
    c.g.L[0] = __ldg(&B.g.L[0]);
    c.g.L[1] = __ldg(&B.g.L[1]);
    c.g.L[2] = __ldg(&B.g.L[2]);
    c.g.P = __ldg(&B.g.P);
    c.g.plane = __ldg(&B.g.plane);
    const int nzs = (c.g.L[2] + kThreads - 1) / kThreads;
    const unsigned r = blockIdx.x / (unsigned)nzs;
    const int zs = (int)(blockIdx.x - r * (unsigned)nzs);
    const int j = (int)(r % (unsigned)c.g.L[1]), i = (int)(r / (unsigned)c.g.L[1]);
    const int k = zs * kThreads + threadIdx.x;
    c.I = i + 1;
    c.J = j + 1;
    c.K = k + 1;
    return i < c.g.L[0] && k < c.g.L[2];
}

__device__ __forceinline__ void load_cell(const double* __restrict__ src, const PadGeom& b, int I, int J, int K,
                                          double (&f)[kQ])
{
    const size_t c = pad_index(b, I, J, K);
#pragma unroll
    for (int a = 0; a < kQ; ++a) f[a] = src[(size_t)a * b.plane + c];
}

// Taylor-Green initial field of a block: interior cell (i, j, k) is global
// cell lo + (i, j, k); per-axis tables of the whole lattice.
__global__ void __launch_bounds__(kThreads) k_dom_init(double* __restrict__ f, PadGeom b, int lo0, int lo1, int lo2,
                                                      const double* __restrict__ tx, const double* __restrict__ ty,
                                                      const double* __restrict__ tz, double rho0, double u0)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= b.L[2]) return;
    double fe[kQ];
    tg_init_cell(fe, tx, ty, tz, lo0 + i, lo1 + j, lo2 + k, rho0, u0);
    const size_t c = pad_index(b, i + 1, j + 1, k + 1);
#pragma unroll
    for (int a = 0; a < kQ; ++a) f[(size_t)a * b.plane + c] = fe[a];
}

// In-place collision of every block's interior (the first Collision() of a
// run), with the undivided lattice's arithmetic: fixed point, native
// float64 for a cell outside its exact range.
template <bool OM_GE1>
__global__ void __launch_bounds__(kThreads, 5) k_dom_collide(const BlockDev* __restrict__ blocks, int cur, FxConst c,
                                                            CollideF64 cp, unsigned long long* __restrict__ fallback)
{
    DomCell dc;
    if (!dom_cell(blocks, dc)) return;
    double* f = blocks[blockIdx.y].buf[cur];
    double v[kQ], out[kQ];
    load_cell(f, dc.g, dc.I, dc.J, dc.K, v);
    bool ok = true;
    fx::collide_cell<OM_GE1>(v, out, c, ok);
    if (!ok) {
        collide_f64(v, cp);
#pragma unroll
        for (int a = 0; a < kQ; ++a) out[a] = v[a];
        atomicAdd(fallback, 1ull);
    }
    const size_t cell = pad_index(dc.g, dc.I, dc.J, dc.K);
#pragma unroll
    for (int a = 0; a < kQ; ++a) f[(size_t)a * dc.g.plane + cell] = out[a];
    // the ghost shells of this buffer are not read by this kernel
    push_halo(blocks, blockIdx.y, cur, dc.g, dc.I - 1, dc.J - 1, dc.K - 1, out);
}

// Native float64 redo of one cell outside the fixed-point range (its
// stores, halo included, replace the ones the caller made).
__device__ __noinline__ void dom_fallback(const BlockDev* __restrict__ blocks, int cur, PadGeom b, int I, int J, int K,
                                          CollideF64 cp, unsigned long long* fallback)
{
    const double* src = blocks[blockIdx.y].buf[cur];
    double* dst = blocks[blockIdx.y].buf[1 - cur];
    double v[kQ];
    gather_pad(src, b, I, J, K, v);
    collide_f64(v, cp);
    const size_t c = pad_index(b, I, J, K);
#pragma unroll
    for (int a = 0; a < kQ; ++a) dst[(size_t)a * b.plane + c] = v[a];
    push_halo(blocks, blockIdx.y, 1 - cur, b, I - 1, J - 1, K - 1, v);
    atomicAdd(fallback, 1ull);
}

// Fused pull + collision of every block's interior from buffer cur into
// 1 - cur, float64 in and out; the pull reads the ghost shell where it
// leaves the block.
template <bool OM_GE1>
__global__ void __launch_bounds__(kThreads, 5) k_dom_step(const BlockDev* __restrict__ blocks, int cur, FxConst c,
                                                         CollideF64 cp, unsigned long long* __restrict__ fallback)
{
    DomCell dc;
    if (!dom_cell(blocks, dc)) return;
    const double* src = blocks[blockIdx.y].buf[cur];
    double* dst = blocks[blockIdx.y].buf[1 - cur];
    double f[kQ], out[kQ];
    gather_pad(src, dc.g, dc.I, dc.J, dc.K, f);
    bool ok = true;
    fx::collide_cell<OM_GE1>(f, out, c, ok);
    const size_t cell = pad_index(dc.g, dc.I, dc.J, dc.K);
#pragma unroll
    for (int a = 0; a < kQ; ++a) dst[(size_t)a * dc.g.plane + cell] = out[a];
    push_halo(blocks, blockIdx.y, 1 - cur, dc.g, dc.I - 1, dc.J - 1, dc.K - 1, out);
    if (!ok) dom_fallback(blocks, cur, dc.g, dc.I, dc.J, dc.K, cp, fallback);
}

// The same step inside a run of steps holding the state as fixed point X on
// the float64 grid between launches (IN_FX / OUT_FX: X instead of float64),
// the undivided lattice's k_step_fxs: a cell outside the exact range records
// step j in *fail, later launches of the run return at once, and the host
// redoes the run from the last complete step with k_dom_step.
template <bool OM_GE1, bool IN_FX, bool OUT_FX>
__global__ void __launch_bounds__(kThreads, 5) k_dom_run(const BlockDev* __restrict__ blocks, int cur, FxConst c, int j,
                                                        int* __restrict__ fail)
{
    if (*fail < j) return;  // an earlier step of the run failed
    DomCell dc;
    if (!dom_cell(blocks, dc)) return;
    const auto* src = reinterpret_cast<const unsigned long long*>(blocks[blockIdx.y].buf[cur]);
    auto* dst = reinterpret_cast<unsigned long long*>(blocks[blockIdx.y].buf[1 - cur]);
    unsigned long long f[kQ];
    gather_pad(src, dc.g, dc.I, dc.J, dc.K, f);
    uint64_t in[kQ], out[kQ];
#pragma unroll
    for (int a = 0; a < kQ; ++a) in[a] = f[a];
    bool ok = true;
    fx::collide_cell_io<OM_GE1, IN_FX, OUT_FX>(in, out, c, ok);
    const size_t cell = pad_index(dc.g, dc.I, dc.J, dc.K);
#pragma unroll
    for (int a = 0; a < kQ; ++a) dst[(size_t)a * dc.g.plane + cell] = out[a];
    push_halo(blocks, blockIdx.y, 1 - cur, dc.g, dc.I - 1, dc.J - 1, dc.K - 1, out);
    if (!ok) atomicMin(fail, j);
}

// A block's f (pulled through the pending streaming when PULL) into the
// whole lattice's array out[a][x][y][z] at the block's offset.
template <bool PULL>
__global__ void __launch_bounds__(kThreads) k_dom_gather(const double* __restrict__ src, PadGeom b, int lo0, int lo1,
                                                        int lo2, int nx, int ny, int nz, double* __restrict__ out)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    if (k >= b.L[2]) return;
    double f[kQ];
    if (PULL) gather_pad(src, b, i + 1, j + 1, k + 1, f);
    else load_cell(src, b, i + 1, j + 1, k + 1, f);
    const size_t plane = (size_t)nx * ny * nz;
    const size_t c = ((size_t)(lo0 + i) * ny + (lo1 + j)) * nz + (lo2 + k);
#pragma unroll
    for (int a = 0; a < kQ; ++a) out[(size_t)a * plane + c] = f[a];
}

// Per-CTA partial sums of {mass, px, py, pz, ke} over a block's cells
// (src/lbm.cpp:271-294), pulled through the pending streaming when PULL.
template <bool PULL>
__global__ void __launch_bounds__(kThreads) k_dom_conserved(const double* __restrict__ src, PadGeom b,
                                                           double* __restrict__ partial)
{
    __shared__ double smem[32 * 5];
    const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, i = blockIdx.z;
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (k < b.L[2]) {
        double f[kQ];
        if (PULL) gather_pad(src, b, i + 1, j + 1, k + 1, f);
        else load_cell(src, b, i + 1, j + 1, k + 1, f);
        double pl = 0.0, ul = 0.0, vl = 0.0, wl = 0.0;
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
        v[0] = pl;
        v[1] = ul;
        v[2] = vl;
        v[3] = wl;
        v[4] = 0.5 * (ul * ul + vl * vl + wl * wl);
    }
    block_sum<5>(v, smem);
    if (threadIdx.x == 0) {
        const size_t q = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
#pragma unroll
        for (int r = 0; r < 5; ++r) partial[q * 5 + r] = v[r];
    }
}

dim3 block_grid(const BlockDev& b)
{
    return dim3((unsigned)((b.g.L[2] + kThreads - 1) / kThreads), (unsigned)b.g.L[1], (unsigned)b.g.L[0]);
}

// Grid of a launch over every block (dom_cell): the largest block's row
// segments by the block count.
dim3 domain_grid(const std::vector<BlockDev>& dev)
{
    size_t most = 0;
    for (const BlockDev& b : dev)
        most = std::max(most, (size_t)b.g.L[0] * b.g.L[1] * ((b.g.L[2] + kThreads - 1) / kThreads));
    return dim3((unsigned)most, (unsigned)dev.size(), 1);
}

}  // namespace
}  // namespace imex

using namespace imex;

struct imex_domain {
    Plan plan;
    std::vector<imex_block> blocks;
    std::vector<BlockDev> dev;     // host copy of the device table
    BlockDev* d_blocks = nullptr;
    unsigned long long halo_values = 0;  // values the halo exchange moves per step
    double* d_partial = nullptr;   // conserved partial sums, then 5 sums per block
    size_t partials = 0;           // partials per block region (largest block)
    unsigned long long* d_fallback = nullptr;
    int* d_fail = nullptr;         // first failing step of a fixed-point run
    int fx_skip = 0, fx_backoff = 0;  // after a failed run: calls that step one at a time
    double* d_field = nullptr;     // whole-lattice staging for imex_domain_get_f (lazily)
    cudaStream_t stream = nullptr;
    int device = 0;
    double tau0 = 0, rho0 = 0, u0 = 0;
    CollideF64 cf64{};
    FxParams fx{};
    bool fx_ok = false;
    int cur = 0;
    int tag = 0;  // 0 uninitialised, 1 exact, 2 streaming pending
    int64_t steps = 0, launches = 0;
    size_t bytes = 0;
    std::string err;
};

namespace {

int dfail(imex_domain* d, int code, const std::string& msg)
{
    if (d) d->err = msg;
    return set_thread_error(code, msg);
}

int dcuda(imex_domain* d, cudaError_t e, const char* what)
{
    cudaGetLastError();
    return dfail(d, IMEX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define D_CUDA(d, call, what)                             \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return dcuda(d, e_, what); \
    } while (0)

int ready(imex_domain* d, const char* what)
{
    if (!d) return set_thread_error(IMEX_ERR_ARG, std::string(what) + ": null domain");
    if (!d->tag) return dfail(d, IMEX_ERR_STATE, std::string(what) + ": domain not initialised");
    D_CUDA(d, cudaSetDevice(d->device), "cudaSetDevice");
    return IMEX_OK;
}

// First Collision of a run: in place, the streaming then pending (the
// undivided lattice's imex_collision on an exact state).
int collide_exact(imex_domain* d)
{
    const dim3 grid = domain_grid(d->dev);
    if (d->fx.om_ge1)
        k_dom_collide<true><<<grid, kThreads, 0, d->stream>>>(d->d_blocks, d->cur, d->fx.k, d->cf64, d->d_fallback);
    else
        k_dom_collide<false><<<grid, kThreads, 0, d->stream>>>(d->d_blocks, d->cur, d->fx.k, d->cf64, d->d_fallback);
    D_CUDA(d, cudaGetLastError(), "collision kernel launch");
    ++d->launches;
    d->tag = 2;
    ++d->steps;
    return IMEX_OK;
}

// One fused step, float64 in and out, cells outside the fixed-point range
// redone in native float64.
int fused_step(imex_domain* d)
{
    const dim3 grid = domain_grid(d->dev);
    if (d->fx.om_ge1)
        k_dom_step<true><<<grid, kThreads, 0, d->stream>>>(d->d_blocks, d->cur, d->fx.k, d->cf64, d->d_fallback);
    else
        k_dom_step<false><<<grid, kThreads, 0, d->stream>>>(d->d_blocks, d->cur, d->fx.k, d->cf64, d->d_fallback);
    D_CUDA(d, cudaGetLastError(), "step kernel launch");
    ++d->launches;
    d->cur = 1 - d->cur;
    ++d->steps;
    return IMEX_OK;
}

template <bool OM_GE1>
cudaError_t launch_run(imex_domain* d, int j, int n)
{
    const dim3 grid = domain_grid(d->dev);
    const bool in_fx = j > 1, out_fx = j < n;
    auto* b = d->d_blocks;
    if (in_fx && out_fx) k_dom_run<OM_GE1, true, true><<<grid, kThreads, 0, d->stream>>>(b, d->cur, d->fx.k, j, d->d_fail);
    else if (in_fx) k_dom_run<OM_GE1, true, false><<<grid, kThreads, 0, d->stream>>>(b, d->cur, d->fx.k, j, d->d_fail);
    else if (out_fx) k_dom_run<OM_GE1, false, true><<<grid, kThreads, 0, d->stream>>>(b, d->cur, d->fx.k, j, d->d_fail);
    else k_dom_run<OM_GE1, false, false><<<grid, kThreads, 0, d->stream>>>(b, d->cur, d->fx.k, j, d->d_fail);
    return cudaGetLastError();
}

// n fused steps as one run holding the state as fixed point between its
// launches (the undivided lattice's rule: float64 before and after, the
// same bits as n single steps).  A cell leaving the exact range stops the
// run at that step; the state before it is converted back to float64 and
// the rest is stepped one at a time with the native fallback, and the next
// 1, 2, 4 .. 64 calls (doubling per failure) step one at a time as well.
int fused_run(imex_domain* d, int n)
{
    if (n < 2 || d->fx_skip > 0) {
        if (n > 0 && d->fx_skip > 0) --d->fx_skip;
        for (int s = 0; s < n; ++s) {
            int rc = fused_step(d);
            if (rc) return rc;
        }
        return IMEX_OK;
    }
    const int64_t steps0 = d->steps;
    std::vector<int> src_of(n + 1);
    D_CUDA(d, cudaMemsetAsync(d->d_fail, 0x7f, sizeof(int), d->stream), "cudaMemset");
    for (int j = 1; j <= n; ++j) {
        D_CUDA(d, d->fx.om_ge1 ? launch_run<true>(d, j, n) : launch_run<false>(d, j, n), "step kernel launch");
        ++d->launches;
        src_of[j] = d->cur;
        d->cur = 1 - d->cur;
        ++d->steps;
    }
    int failed = 0;
    D_CUDA(d, cudaMemcpyAsync(&failed, d->d_fail, sizeof failed, cudaMemcpyDeviceToHost, d->stream), "cudaMemcpy");
    D_CUDA(d, cudaStreamSynchronize(d->stream), "fixed-point run");
    if (failed > n) {
        d->fx_backoff = 0;
        return IMEX_OK;
    }
    d->fx_backoff = d->fx_backoff ? std::min(64, 2 * d->fx_backoff) : 1;
    d->fx_skip = d->fx_backoff;
    d->cur = src_of[failed];
    d->steps = steps0 + failed - 1;
    if (failed > 1)
        for (const BlockDev& b : d->dev) {
            D_CUDA(d, launch_fx_to_f64(b.buf[d->cur], (size_t)kQ * b.g.plane, d->stream), "conversion");
            ++d->launches;
        }
    for (int s = failed; s <= n; ++s) {
        int rc = fused_step(d);
        if (rc) return rc;
    }
    return IMEX_OK;
}

}  // namespace

extern "C" {

int imex_decomp_grid(int nranks, int nx, int ny, int nz, int grid[3])
{
    if (!grid) return set_thread_error(IMEX_ERR_ARG, "imex_decomp_grid: null output");
    Plan p;
    int rc = check_plan_args(nranks, nx, ny, nz, "imex_decomp_grid", &p);
    if (rc) return rc;
    for (int d = 0; d < 3; ++d) grid[d] = p.grid[d];
    return IMEX_OK;
}

int imex_decomp_block(int nranks, int nx, int ny, int nz, int rank, imex_block* out)
{
    if (!out) return set_thread_error(IMEX_ERR_ARG, "imex_decomp_block: null output");
    Plan p;
    int rc = check_plan_args(nranks, nx, ny, nz, "imex_decomp_block", &p);
    if (rc) return rc;
    if (rank < 0 || rank >= nranks) return set_thread_error(IMEX_ERR_ARG, "imex_decomp_block: rank out of range");
    block_of(p, rank, out);
    return IMEX_OK;
}

int imex_decomp_halo(int nranks, int nx, int ny, int nz, int rank, int channel, imex_halo_msg* out)
{
    if (!out) return set_thread_error(IMEX_ERR_ARG, "imex_decomp_halo: null output");
    Plan p;
    int rc = check_plan_args(nranks, nx, ny, nz, "imex_decomp_halo", &p);
    if (rc) return rc;
    if (rank < 0 || rank >= nranks || channel < 0 || channel >= 26)
        return set_thread_error(IMEX_ERR_ARG, "imex_decomp_halo: rank or channel out of range");
    halo_msg(p, rank, channel, out);
    return IMEX_OK;
}

void imex_domain_destroy(imex_domain* d)
{
    if (!d) return;
    cudaSetDevice(d->device);
    if (d->stream) cudaStreamSynchronize(d->stream);
    for (BlockDev& b : d->dev)
        for (double* p : b.buf)
            if (p) cudaFree(p);
    if (d->d_blocks) cudaFree(d->d_blocks);
    if (d->d_partial) cudaFree(d->d_partial);
    if (d->d_fallback) cudaFree(d->d_fallback);
    if (d->d_fail) cudaFree(d->d_fail);
    if (d->d_field) cudaFree(d->d_field);
    if (d->stream) cudaStreamDestroy(d->stream);
    delete d;
}

int imex_domain_create(int nx, int ny, int nz, int nranks, double tau, double rho0, double u0, imex_domain** out)
{
    if (!out) return set_thread_error(IMEX_ERR_ARG, "imex_domain_create: null output");
    *out = nullptr;
    Plan p;
    int rc = check_plan_args(nranks, nx, ny, nz, "imex_domain_create", &p);
    if (rc) return rc;
    if (nranks > 512) return set_thread_error(IMEX_ERR_ARG, "imex_domain_create: at most 512 sub-domains");
    if (nx > 65535 || ny > 65535) return set_thread_error(IMEX_ERR_ARG, "imex_domain_create: nx and ny must be <= 65535");
    if (!std::isfinite(tau) || !std::isfinite(rho0) || !std::isfinite(u0) || !(tau + 0.5 > 0.0))
        return set_thread_error(IMEX_ERR_ARG, "imex_domain_create: tau, rho0, u0 must be finite with tau > -0.5");
    imex_domain* d = new imex_domain();
    d->plan = p;
    d->tau0 = tau;
    d->rho0 = rho0;
    d->u0 = u0;
    d->cf64 = make_collide_f64(tau);
    d->fx_ok = make_fx_params(tau, rho0, &d->fx);
    if (!d->fx_ok) {
        imex_domain_destroy(d);
        return set_thread_error(IMEX_ERR_ARG, "imex_domain_create: the sub-domain step uses the fixed-point engine, "
                                              "which needs 0.75 <= rho0 <= 1.25");
    }
    auto bail = [&](int code, const std::string& msg) {
        imex_domain_destroy(d);
        return set_thread_error(code, msg);
    };
    cudaError_t e = cudaGetDevice(&d->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(IMEX_ERR_CUDA, std::string("imex_domain_create: ") + cudaGetErrorString(e));
    // blocks, their padded boxes and the partial-sum room of the largest
    d->blocks.resize(nranks);
    d->dev.resize(nranks);
    size_t need = 0;
    for (int r = 0; r < nranks; ++r) {
        block_of(p, r, &d->blocks[r]);
        BlockDev& b = d->dev[r];
        for (int q = 0; q < 3; ++q) b.g.L[q] = d->blocks[r].len[q];
        b.g.P = pad_pitch(b.g.L[2]);
        b.g.plane = (size_t)(b.g.L[0] + 2) * (b.g.L[1] + 2) * b.g.P;
        need += 2 * (size_t)kQ * b.g.plane * sizeof(double);
        const dim3 g = block_grid(b);
        d->partials = std::max(d->partials, (size_t)g.x * g.y * g.z);
    }
    size_t free_b = 0, total_b = 0;
    e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) return bail(IMEX_ERR_CUDA, std::string("imex_domain_create: ") + cudaGetErrorString(e));
    if (need > free_b) return bail(IMEX_ERR_MEMORY, "imex_domain_create: not enough device memory");
    for (BlockDev& b : d->dev)
        for (double*& ptr : b.buf) {
            e = cudaMalloc(&ptr, (size_t)kQ * b.g.plane * sizeof(double));
            if (e == cudaSuccess) e = cudaMemsetAsync(ptr, 0, (size_t)kQ * b.g.plane * sizeof(double), d->stream);
            if (e != cudaSuccess) return bail(IMEX_ERR_MEMORY, "imex_domain_create: device allocation failed");
        }
    // each block's neighbours, and the values the halo moves per step: the
    // pruned directions of every channel's box
    unsigned long long total = 0;
    for (int r = 0; r < nranks; ++r) {
        for (int o = 0; o < 27; ++o) {
            const int off[3] = {o / 9 - 1, (o / 3) % 3 - 1, o % 3 - 1};
            d->dev[r].nb[o] = neighbour(p, d->blocks[r], off);
        }
        for (int c = 0; c < 26; ++c) {
            imex_halo_msg m;
            halo_msg(p, r, c, &m);
            total += (unsigned long long)m.ndir * m.ext[0] * m.ext[1] * m.ext[2];
        }
    }
    d->halo_values = total;
    e = cudaMalloc(&d->d_blocks, sizeof(BlockDev) * nranks);
    if (e == cudaSuccess) e = cudaMemcpy(d->d_blocks, d->dev.data(), sizeof(BlockDev) * nranks, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&d->d_partial, (d->partials + 1) * 5 * sizeof(double) * nranks);
    if (e == cudaSuccess) e = cudaMalloc(&d->d_fallback, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&d->d_fail, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(d->d_fallback, 0, sizeof(unsigned long long), d->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(d->stream);
    if (e != cudaSuccess) return bail(IMEX_ERR_CUDA, std::string("imex_domain_create: ") + cudaGetErrorString(e));
    d->bytes = need;
    *out = d;
    return IMEX_OK;
}

int imex_domain_initialize(imex_domain* d)
{
    if (!d) return set_thread_error(IMEX_ERR_ARG, "imex_domain_initialize: null domain");
    D_CUDA(d, cudaSetDevice(d->device), "cudaSetDevice");
    // the undivided lattice's per-axis tables (src/lbm.cpp:81-93)
    const int* n = d->plan.n;
    std::vector<double> table(3 * ((size_t)n[0] + n[1] + n[2]));
    size_t off = 0, offs[3];
    for (int q = 0; q < 3; ++q) {
        offs[q] = off;
        for (int i = 0; i < n[q]; ++i) {
            const double xx = (double)i / (double)n[q] * 2.0 * 3.1415926;
            table[off++] = std::sin(xx);
            table[off++] = std::cos(xx);
            table[off++] = std::cos(2.0 * xx);
        }
    }
    double* dt = nullptr;
    D_CUDA(d, cudaMallocAsync(&dt, table.size() * sizeof(double), d->stream), "cudaMallocAsync");
    cudaError_t e = cudaMemcpyAsync(dt, table.data(), table.size() * sizeof(double), cudaMemcpyHostToDevice, d->stream);
    for (size_t r = 0; r < d->dev.size() && e == cudaSuccess; ++r) {
        const imex_block& b = d->blocks[r];
        k_dom_init<<<block_grid(d->dev[r]), kThreads, 0, d->stream>>>(d->dev[r].buf[0], d->dev[r].g, b.lo[0], b.lo[1], b.lo[2],
                                                                     dt + offs[0], dt + offs[1], dt + offs[2], d->rho0,
                                                                     d->u0);
        e = cudaGetLastError();
        ++d->launches;
    }
    cudaError_t e2 = cudaFreeAsync(dt, d->stream);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaStreamSynchronize(d->stream);
    if (e != cudaSuccess) return dcuda(d, e, "imex_domain_initialize");
    d->cur = 0;
    d->tag = 1;
    d->steps = 0;
    return IMEX_OK;
}

int imex_domain_step(imex_domain* d, int nsteps)
{
    int rc = ready(d, "imex_domain_step");
    if (rc) return rc;
    if (nsteps < 0) return dfail(d, IMEX_ERR_ARG, "imex_domain_step: nsteps < 0");
    if (nsteps > 0 && d->tag == 1) {
        rc = collide_exact(d);
        if (rc) return rc;
        --nsteps;
    }
    return fused_run(d, nsteps);
}

int imex_domain_conserved_blocks(imex_domain* d, double* out)
{
    int rc = ready(d, "imex_domain_conserved");
    if (rc) return rc;
    if (!out) return dfail(d, IMEX_ERR_ARG, "imex_domain_conserved: null output");
    const bool pull = d->tag == 2;  // the ghost shells are current (the producers stored them)
    const size_t nb = d->dev.size();
    double* sums = d->d_partial + nb * d->partials * 5;
    for (size_t r = 0; r < nb; ++r) {
        const BlockDev& b = d->dev[r];
        double* part = d->d_partial + r * d->partials * 5;
        if (pull) k_dom_conserved<true><<<block_grid(b), kThreads, 0, d->stream>>>(b.buf[d->cur], b.g, part);
        else k_dom_conserved<false><<<block_grid(b), kThreads, 0, d->stream>>>(b.buf[d->cur], b.g, part);
        D_CUDA(d, cudaGetLastError(), "conserved kernel launch");
        const dim3 g = block_grid(b);
        D_CUDA(d, launch_reduce_partials(part, (size_t)g.x * g.y * g.z, sums + 5 * r, d->stream), "reduce launch");
        d->launches += 2;
    }
    D_CUDA(d, cudaMemcpyAsync(out, sums, nb * 5 * sizeof(double), cudaMemcpyDeviceToHost, d->stream), "cudaMemcpy");
    D_CUDA(d, cudaStreamSynchronize(d->stream), "imex_domain_conserved");
    return IMEX_OK;
}

int imex_domain_conserved(imex_domain* d, double out[5])
{
    if (!d || !out) return set_thread_error(IMEX_ERR_ARG, "imex_domain_conserved: null argument");
    std::vector<double> per(d->dev.size() * 5);
    int rc = imex_domain_conserved_blocks(d, per.data());
    if (rc) return rc;
    // the blocks' sums combined in rank order (the reference's MPI_Allreduce
    // of src/lbm.cpp:296-300)
    for (int q = 0; q < 5; ++q) {
        double s = 0.0;
        for (size_t r = 0; r < d->dev.size(); ++r) s += per[5 * r + q];
        out[q] = s;
    }
    for (int q = 0; q < 5; ++q)
        if (!std::isfinite(out[q])) return dfail(d, IMEX_ERR_NONFINITE, "imex_domain_conserved: non-finite diagnostics");
    return IMEX_OK;
}

int imex_domain_get_f(imex_domain* d, double* host, size_t n)
{
    int rc = ready(d, "imex_domain_get_f");
    if (rc) return rc;
    const size_t cells = (size_t)d->plan.n[0] * d->plan.n[1] * d->plan.n[2];
    if (!host || n != (size_t)kQ * cells) return dfail(d, IMEX_ERR_ARG, "imex_domain_get_f: buffer size must be 27*nx*ny*nz");
    const bool pull = d->tag == 2;  // the ghost shells are current (the producers stored them)
    if (!d->d_field) D_CUDA(d, cudaMalloc(&d->d_field, n * sizeof(double)), "cudaMalloc");
    for (size_t r = 0; r < d->dev.size(); ++r) {
        const imex_block& b = d->blocks[r];
        const BlockDev& bd = d->dev[r];
        const int* n3 = d->plan.n;
        if (pull)
            k_dom_gather<true><<<block_grid(bd), kThreads, 0, d->stream>>>(bd.buf[d->cur], bd.g, b.lo[0], b.lo[1],
                                                                          b.lo[2], n3[0], n3[1], n3[2], d->d_field);
        else
            k_dom_gather<false><<<block_grid(bd), kThreads, 0, d->stream>>>(bd.buf[d->cur], bd.g, b.lo[0], b.lo[1],
                                                                           b.lo[2], n3[0], n3[1], n3[2], d->d_field);
        D_CUDA(d, cudaGetLastError(), "gather kernel launch");
        ++d->launches;
    }
    D_CUDA(d, cudaMemcpyAsync(host, d->d_field, n * sizeof(double), cudaMemcpyDeviceToHost, d->stream), "cudaMemcpy");
    D_CUDA(d, cudaStreamSynchronize(d->stream), "imex_domain_get_f");
    return IMEX_OK;
}

int imex_domain_info(const imex_domain* d, imex_domain_stats* out)
{
    if (!d || !out) return set_thread_error(IMEX_ERR_ARG, "imex_domain_info: null argument");
    out->nranks = d->plan.nranks;
    for (int q = 0; q < 3; ++q) out->grid[q] = d->plan.grid[q];
    out->steps = d->steps;
    out->launches = d->launches;
    out->halo_values_per_step = (int64_t)d->halo_values;
    out->device_bytes = (int64_t)d->bytes;
    return IMEX_OK;
}

int imex_domain_fallback_cells(imex_domain* d, int64_t* out)
{
    if (!d || !out) return set_thread_error(IMEX_ERR_ARG, "imex_domain_fallback_cells: null argument");
    unsigned long long v = 0;
    D_CUDA(d, cudaMemcpyAsync(&v, d->d_fallback, sizeof v, cudaMemcpyDeviceToHost, d->stream), "cudaMemcpy");
    D_CUDA(d, cudaStreamSynchronize(d->stream), "imex_domain_fallback_cells");
    *out = (int64_t)v;
    return IMEX_OK;
}

int imex_domain_synchronize(imex_domain* d)
{
    if (!d) return set_thread_error(IMEX_ERR_ARG, "imex_domain_synchronize: null domain");
    D_CUDA(d, cudaStreamSynchronize(d->stream), "imex_domain_synchronize");
    return IMEX_OK;
}

const char* imex_domain_last_error(const imex_domain* d) { return d ? d->err.c_str() : thread_error(); }

}  // extern "C"
