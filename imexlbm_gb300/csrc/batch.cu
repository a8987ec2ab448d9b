// Batched step: many reduced-precision lattices of any sizes advance in one
// persistent launch over a packed cell index.
//
// A batch holds member lattice handles (float32 or float16-deviation
// storage).  Their cells are numbered consecutively - lattice after
// lattice, each in its own f[a][x][y][z] order - and every launch of the
// persistent kernel walks that packed index: a thread finds its lattice by
// binary search over the members' first-cell indices, decodes (x, y, z),
// pulls the 27 values from that lattice's buffer with periodic wrap,
// collides in float32 (lowp_math.cuh, the same arithmetic as the
// one-lattice kernels, so results are bit-identical) and writes the other
// buffer.  Lattices of different sizes, viscosities and storage formats mix
// in one launch; no launch is spent on a small lattice alone.
//
// The member table lives in device memory and the kernel reads it at every
// launch, so a CUDA graph of K launches (step index s = 0..K-1 baked in)
// stays valid while members join, leave or finish: a member runs at step s
// only while s < its step count for the tick, and within a tick it reads
// buf[cur ^ (s & 1)] and writes the other buffer.
//
// Members whose rows suit asynchronous bulk copies (nz * element size a
// multiple of 16 bytes) run instead in a second persistent kernel, the
// batched form of the row-staged step (rows.cuh): its work items are blocks
// of B consecutive y-rows of one member, B chosen per member so that an
// item's 27 source runs fill one stage of a shared-memory ring; the copies
// of later items are in flight while an item is collided, and the item's
// cells are spread over all threads of the CTA whatever the member's nz.
// Items of members whose step count for the tick is exhausted are armed
// with no bytes and skipped, keeping the ring's phases uniform.
//
// Launch shapes (cell kernel: threads per CTA, cells per thread, CTAs per
// SM; row kernel: stages, stage size, CTAs per SM) are chosen by an
// autotuner that times each candidate on the batch itself; timing writes
// only the members' spare buffers, so it changes no state.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "imexlbm.h"
#include "imexlbm_internal.hpp"
#include "lattice_internal.hpp"
#include "lowp_math.cuh"
#include "rows_lowp.cuh"

namespace imex {

namespace {

constexpr int kBatchMax = 2048;  // members per batch (shared-memory search table)

struct BatchEntry {
    unsigned long long begin;  // packed index of the member's first cell
    unsigned long long plane;  // cells of the member
    void* buf[2];
    int nx, ny, nz;
    int prec;   // IMEX_F32 or IMEX_F16DEV
    int cur;    // buffer holding the member's state at the start of the tick
    int steps;  // fused steps this tick
    float eps;      // 2 - omega
    int sr;         // float16 storage: stochastic rounding
    uint32_t seed;  // stochastic-rounding seed at the start of the tick
    int B;          // row kernel: y-rows per work item
    unsigned ibegin;  // row kernel: packed index of the member's first item
    int pad;
};

struct BatchHeader {
    unsigned long long total;  // cells of all members
    int count;
    int pad;
};

// Table header of the row kernel's members.
struct RowsHeader {
    unsigned total;  // work items of all its members
    int count;       // its members
};

// Fused step of cell (i, j, k) of member e - its index `local` within the
// member - at step s of the tick.
template <int P>
__device__ __forceinline__ void batch_cell_at(const BatchEntry& e, int i, int j, int k, unsigned local, int s,
                                              const CollideF32& base)
{
    using S = lowp::Storage<P>;
    using T = typename S::T;
    const int nz = e.nz, ny = e.ny, nx = e.nx;
    Geom g;
    g.nx = nx;
    g.ny = ny;
    g.nz = nz;
    g.plane = e.plane;
    const PullIndex pi(g, i, j, k, true);
    const T* src = static_cast<const T*>(e.buf[e.cur ^ (s & 1)]);
    T* dst = static_cast<T*>(e.buf[e.cur ^ (s & 1) ^ 1]);
    float h[kQ];
#pragma unroll
    for (int a = 0; a < kQ; ++a) h[a] = S::load(src + pi.at_dyn(g, a), a);
    CollideF32 cp = base;
    cp.eps = e.eps;
    lowp::collide_dev_f32<P>(h, cp);
    if constexpr (P == IMEX_F16DEV) {
        auto at = [&](int a) -> T& { return dst[(size_t)a * e.plane + local]; };
        lowp::store_f16_cell(h, e.sr, local, e.seed + (uint32_t)s, at);
    } else {
#pragma unroll
        for (int a = 0; a < kQ; ++a) dst[(size_t)a * e.plane + local] = S::store(h[a], a);
    }
}

template <int P>
__device__ __forceinline__ void batch_cell(const BatchEntry& e, unsigned local, int s, const CollideF32& base)
{
    const unsigned row = local / (unsigned)e.nz;  // members hold fewer than 2^32 cells
    const int k = (int)(local - row * (unsigned)e.nz);
    const int i = (int)(row / (unsigned)e.ny);
    const int j = (int)(row - (unsigned)i * (unsigned)e.ny);
    batch_cell_at<P>(e, i, j, k, local, s, base);
}

// Cells per row segment of the one-CTA-per-segment cell kernel.
constexpr int kUnitCells = kStepBlock;
constexpr int kUnitGroup = 256;  // row segments per entry of the member lookup table

// One CTA per row segment: the grid of the one-lattice kernel (k_step_lowp:
// 128 threads per CTA, each CTA kUnitCells consecutive z-cells of one (x, y)
// row), over every member of the cell kernel.  Segment u belongs to the
// member whose first segment index `begin` is the largest not above u; the
// member is found from group[u / kUnitGroup] (the member holding segment
// u - u mod kUnitGroup) by stepping forward, the same for every thread of
// the CTA, and the segment's (x, y, z block) is decoded once per CTA, so a
// thread's cell costs what it costs in the one-lattice kernel.  The grid
// covers the segments of the tick's members; a CUDA graph of these
// launches is captured again when that count changes.  The float32-only
// instantiation fits 48 registers (10 CTAs, 40 warps per SM, as the one-
// lattice kernel); with the float16 path too it needs 64.
template <int PF, int MINB = PF == IMEX_F32 ? 10 : 0>
__global__ void __launch_bounds__(kUnitCells, MINB) k_batch_units(const BatchHeader* __restrict__ hdr,
                                                            const BatchEntry* __restrict__ tab,
                                                            const int* __restrict__ group, int s, CollideF32 base)
{
    const unsigned u = blockIdx.x;
    const int count = hdr->count;
    int m = group[u / kUnitGroup];
    while (m + 1 < count && tab[m + 1].begin <= u) ++m;
    const BatchEntry& e = tab[m];
    if (s >= e.steps) return;
    const unsigned zbs = ((unsigned)e.nz + kUnitCells - 1) / kUnitCells;
    const unsigned seg = u - (unsigned)e.begin;
    const unsigned row = seg / zbs;
    const int k = (int)(seg - row * zbs) * kUnitCells + (int)threadIdx.x;
    if (k >= e.nz) return;
    const int i = (int)(row / (unsigned)e.ny);
    const int j = (int)(row - (unsigned)i * (unsigned)e.ny);
    const unsigned local = row * (unsigned)e.nz + (unsigned)k;
    if constexpr (PF == IMEX_F32) batch_cell_at<IMEX_F32>(e, i, j, k, local, s, base);
    else if (e.prec == IMEX_F32) batch_cell_at<IMEX_F32>(e, i, j, k, local, s, base);
    else batch_cell_at<IMEX_F16DEV>(e, i, j, k, local, s, base);
}

// CPT cells per thread, strided by blockDim within a chunk of CPT*blockDim.
// Every member starts on a chunk boundary of the packed index (upload_table
// pads the index), so a chunk holds cells of one member only: the member is
// looked up once per chunk, by a search all threads make on the same
// shared-memory entries, and the cells are numbered within the member in
// 32 bits.  (Searching per cell, 11 dependent shared-memory loads for 2048
// members, held the float32 kernel at 28.1-28.7 GLUPS on the 64-lattice
// workload.)  PF = IMEX_F32: every member of the packed index is float32,
// and only that path is compiled, held to 64 registers with one cell per
// thread (4 CTAs of 256 threads per SM).
//
// TPB / MINB: the launch bounds.  Threads 256 with 4 CTAs per SM (64
// registers) for the float32-only kernel with one cell per thread, the
// compiler's choice for the others; threads 128 with 9 CTAs per SM (56
// registers, 36 warps per SM) for the lean float32 kernel, near the
// occupancy of the one-lattice float32 kernel (48 registers, 128 threads,
// 40 warps).
template <int CPT, int PF, int TPB = 256, int MINB = (PF == IMEX_F32 && CPT == 1) ? 4 : 0>
__global__ void __launch_bounds__(TPB, MINB)
    k_batch(const BatchHeader* __restrict__ hdr, const BatchEntry* __restrict__ tab, int s, CollideF32 base)
{
    extern __shared__ unsigned long long sbegin[];  // count + 1 entries (the launch sizes it for the capacity)
    const int count = hdr->count;
    const unsigned long long total = hdr->total;
    for (int q = threadIdx.x; q < count; q += blockDim.x) sbegin[q] = tab[q].begin;
    if (threadIdx.x == 0) sbegin[count] = total;
    __syncthreads();
    const unsigned long long chunk = (unsigned long long)blockDim.x * CPT;
    for (unsigned long long c0 = (unsigned long long)blockIdx.x * chunk; c0 < total; c0 += (unsigned long long)gridDim.x * chunk) {
        int lo = 0, hi = count;  // largest lo with sbegin[lo] <= c0 (the same for every thread)
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (sbegin[mid] <= c0) lo = mid;
            else hi = mid;
        }
        const BatchEntry& e = tab[lo];
        if (s >= e.steps) continue;
        const unsigned first = (unsigned)(c0 - sbegin[lo]) + threadIdx.x;
        const unsigned cells = (unsigned)e.plane;
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            const unsigned local = first + (unsigned)c * blockDim.x;
            if (local >= cells) break;
            if constexpr (PF == IMEX_F32) batch_cell<IMEX_F32>(e, local, s, base);
            else if (e.prec == IMEX_F32) batch_cell<IMEX_F32>(e, local, s, base);
            else batch_cell<IMEX_F16DEV>(e, local, s, base);
        }
    }
}

// Bytes of the row kernel's table of first items for `members` members.
__host__ __device__ inline size_t rows_table_bytes(int members)
{
    return (sizeof(unsigned) * (size_t)(members + 1) + 15) & ~(size_t)15;
}

// Row-staged batched step (rows_lowp.cuh): work items of every member in
// one persistent loop; an item's member is found by binary search over the
// members' first-item indices, kept in shared memory after the ring, and
// its entry is copied next to them.  Thread 0 describes every item (it arms
// the stage), ahead of the CTA barrier that ends the item before it; a
// CTA's consecutive items usually belong to one member, so the entry is
// looked up and loaded from global memory only when the member changes.
template <int kDirBytes, int kMinBlocks>
__global__ void __launch_bounds__(rowslp::kThreads, kMinBlocks)
    k_batch_rows(const RowsHeader* __restrict__ hdr, const BatchEntry* __restrict__ tab, int s, CollideF32 base,
                 int stages, int table_cap, WaitCtl wc)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int count = hdr->count;
    if (count > table_cap) {  // the table would not fit the shared memory the launch has
        if (threadIdx.x == 0) atomicOr(wc.err, 2u);
        return;
    }
    const unsigned total = hdr->total;
    unsigned* sbegin = reinterpret_cast<unsigned*>(smem + rowslp::smem_bytes(kDirBytes, stages));
    BatchEntry* sentry = reinterpret_cast<BatchEntry*>(reinterpret_cast<unsigned char*>(sbegin) +
                                                       rows_table_bytes(table_cap));
    for (int q = threadIdx.x; q < count; q += blockDim.x) sbegin[q] = tab[q].ibegin;
    if (threadIdx.x == 0) sbegin[count] = total;
    __syncthreads();
    const unsigned G = gridDim.x;
    const int my = blockIdx.x < total ? (int)((total - 1 - blockIdx.x) / G) + 1 : 0;
    int cached = -1;  // member whose entry sentry holds (thread 0, the only caller)
    auto item_of = [&](int t) {
        const unsigned itx = blockIdx.x + (unsigned)t * G;
        if (cached < 0 || itx < sbegin[cached] || itx >= sbegin[cached + 1]) {
            int lo = 0, hi = count;  // largest lo with sbegin[lo] <= itx
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (sbegin[mid] <= itx) lo = mid;
                else hi = mid;
            }
            *sentry = tab[lo];
            cached = lo;
        }
        const BatchEntry& e = *sentry;
        const int lo = cached;
        rowslp::Item it;
        const int cur = e.cur ^ (s & 1);
        it.src = static_cast<const unsigned char*>(e.buf[cur]);
        it.dst = static_cast<unsigned char*>(e.buf[cur ^ 1]);
        it.plane = e.plane;
        it.nx = e.nx;
        it.ny = e.ny;
        it.nz = e.nz;
        it.B = e.B;
        const unsigned local = itx - sbegin[lo];
        const unsigned yblocks = (unsigned)rowslp::y_blocks(e.ny, e.B);
        it.x = (int)(local / yblocks);
        it.y0 = (int)(local - (unsigned)it.x * yblocks) * e.B;
        if (e.ny - it.y0 < it.B) it.B = e.ny - it.y0;  // the last block of a plane may be shorter
        it.prec = e.prec;
        it.eps = e.eps;
        it.sr = e.sr;
        it.seed = e.seed + (uint32_t)s;
        it.active = s < e.steps;
        return it;
    };
    rowslp::run_items<kDirBytes, lowp::F2, true>(item_of, my, stages, base, smem, wc);
}

}  // namespace

}  // namespace imex

using namespace imex;

// Row-kernel launch shape: ring depth, KiB per direction in a stage (1, 2
// or 4), resident CTAs per SM (stages 0: not chosen yet; -1: row kernel
// off, every member in the cell kernel) and whether float32 members join
// it (float16-deviation members always do when their rows allow).
struct RowShape {
    int stages = 0, dir_kb = 0, ctas_per_sm = 0, f32 = 1;
};

struct BatchShape {
    int threads = 0, cpt = 0, ctas_per_sm = 0;  // 0: not chosen yet
};

struct imex_batch {
    std::vector<imex_lattice*> members;
    std::vector<int64_t> limit;  // total reference steps after which a member stops (-1: none)
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    BatchHeader* d_hdr = nullptr;  // cell kernel's members
    BatchEntry* d_tab = nullptr;
    BatchHeader* h_hdr = nullptr;  // pinned staging
    BatchEntry* h_tab = nullptr;
    RowsHeader* d_rhdr = nullptr;  // row kernel's members
    BatchEntry* d_rtab = nullptr;
    RowsHeader* h_rhdr = nullptr;
    BatchEntry* h_rtab = nullptr;
    int* d_group = nullptr;     // one-CTA-per-segment cell kernel: member of every kUnitGroup-th segment
    int* h_group = nullptr;
    size_t group_cap = 0;
    unsigned* d_err = nullptr;  // set by the row kernel when a bounded wait runs out
    int capacity = 0;
    int device = 0;
    int sms = 0;
    BatchShape shape;
    RowShape rshape;
    int n_cell = 0, n_row = 0;  // members in each kernel (last uploaded table)
    int n_cell_f16 = 0;         // float16-deviation members in the cell kernel
    int graph_steps = 0;  // K of the captured graph (0: no graph)
    cudaGraphExec_t graph = nullptr;
    int graph_k = 0;
    BatchShape graph_shape;
    unsigned long long graph_units = 0;  // segments the captured cell-kernel launches cover
    const int* graph_group = nullptr;    // the group table the captured segment-kernel launches read
    RowShape graph_rshape;
    int graph_kinds = 0;  // bit 0: cell kernel, bit 1: row kernel, bit 2: cell kernel with float16 members
    int64_t launches = 0;
    std::string err;
};

namespace {

int bfail(imex_batch* b, int code, const std::string& msg)
{
    if (b) b->err = msg;
    return set_thread_error(code, msg);
}

int bcuda(imex_batch* b, cudaError_t e, const char* what)
{
    cudaGetLastError();
    return bfail(b, IMEX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define B_CUDA(b, call, what)                            \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return bcuda(b, e_, what); \
    } while (0)

CollideF32 base_constants()
{
    // eps is per member; w and the e.u coefficients are shared.
    return make_collide_f32(0.0);
}

// Shared memory of a row-kernel CTA: barriers, ring, the table of the
// members' first items (sized for the batch's capacity - a CUDA graph keeps
// the size it was captured with while members join) and a copy of the
// member entry last looked up.
size_t rows_smem(const RowShape& rs, int members)
{
    return rowslp::smem_bytes(rs.dir_kb * 1024, rs.stages) + rows_table_bytes(members) + sizeof(BatchEntry);
}

// Whether the row shape's CTAs fit an SM's shared memory.
bool rows_fit(const RowShape& rs, int members)
{
    const size_t smem = rows_smem(rs, members);
    return smem <= 227 * 1024 && (size_t)rs.ctas_per_sm * (smem + 1024) <= 228 * 1024;
}

int kinds(const imex_batch* b)
{
    return (b->n_cell > 0 ? 1 : 0) | (b->n_row > 0 ? 2 : 0) | (b->n_cell_f16 > 0 ? 4 : 0);
}

// One step (index s of the tick) of every member: the cell kernel over its
// members, then the row kernel over its members.
// Persistent grid of the cell kernel `fn` for shape sh: sh.ctas_per_sm CTAs
// per SM, but no more than can be resident at once.  CTAs beyond the
// resident ones would run their whole strided loop after the first wave,
// reading rows whose neighbours the first wave has already evicted from L2.
unsigned cell_grid(const imex_batch* b, const void* fn, const BatchShape& sh)
{
    static std::mutex lock;
    static std::map<std::tuple<int, const void*, int>, int> cache;
    const auto key = std::make_tuple(b->device * 4096 + b->capacity, fn, sh.threads);
    int resident = 0;
    {
        std::lock_guard<std::mutex> guard(lock);
        auto it = cache.find(key);
        if (it != cache.end()) resident = it->second;
    }
    if (!resident) {
        const size_t smem = sizeof(unsigned long long) * ((size_t)b->capacity + 1);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, fn, sh.threads, smem) != cudaSuccess ||
            resident < 1) {
            cudaGetLastError();
            resident = 1;
        }
        std::lock_guard<std::mutex> guard(lock);
        cache[key] = resident;
    }
    return (unsigned)(b->sms * std::min(sh.ctas_per_sm, resident));
}

template <int C, int PF, int TPB = 256, int MINB = (PF == IMEX_F32 && C == 1) ? 4 : 0>
cudaError_t launch_cells(imex_batch* b, const BatchShape& sh, int s, const CollideF32& base)
{
    auto* fn = k_batch<C, PF, TPB, MINB>;
    const size_t smem = sizeof(unsigned long long) * ((size_t)b->capacity + 1);
    fn<<<cell_grid(b, (const void*)fn, sh), sh.threads, smem, b->stream>>>(b->d_hdr, b->d_tab, s, base);
    return cudaGetLastError();
}

cudaError_t launch_step(imex_batch* b, const BatchShape& sh, const RowShape& rs, int s)
{
    const CollideF32 base = base_constants();
    if (b->n_cell > 0) {
        const bool f32 = b->n_cell_f16 == 0;
        cudaError_t e;
        if (sh.cpt == 0) {  // one CTA per row segment
            const unsigned long long units = b->h_hdr->total;
            if (units == 0 || units > 0x7fffffffull) return cudaErrorInvalidValue;
            if (f32)
                k_batch_units<IMEX_F32><<<(unsigned)units, kUnitCells, 0, b->stream>>>(b->d_hdr, b->d_tab, b->d_group, s,
                                                                                     base);
            else
                k_batch_units<0><<<(unsigned)units, kUnitCells, 0, b->stream>>>(b->d_hdr, b->d_tab, b->d_group, s, base);
            e = cudaGetLastError();
        } else if (f32 && sh.cpt == 1 && sh.threads == 128) e = launch_cells<1, IMEX_F32, 128, 9>(b, sh, s, base);
        else if (sh.cpt == 1) e = f32 ? launch_cells<1, IMEX_F32>(b, sh, s, base) : launch_cells<1, 0>(b, sh, s, base);
        else if (sh.cpt == 2) e = f32 ? launch_cells<2, IMEX_F32>(b, sh, s, base) : launch_cells<2, 0>(b, sh, s, base);
        else if (sh.cpt == 4) e = f32 ? launch_cells<4, IMEX_F32>(b, sh, s, base) : launch_cells<4, 0>(b, sh, s, base);
        else e = cudaErrorInvalidValue;
        if (e != cudaSuccess) return e;
    }
    if (b->n_row > 0) {
        const unsigned items = b->h_rhdr->total;
        unsigned grid = (unsigned)(b->sms * rs.ctas_per_sm);
        if (grid > items) grid = items;
        if (!rows_fit(rs, b->capacity)) return cudaErrorInvalidValue;
        const size_t smem = rows_smem(rs, b->capacity);
        const bool one = rs.ctas_per_sm <= 1;  // one resident CTA: the full register file
        // the test hook IMEX_TEST_FAULT_BATCH_TABLE hands the kernel a table
        // capacity below the member count, so that its refusal fires
        const int cap = test_fault_kind() == IMEX_TEST_FAULT_BATCH_TABLE ? b->n_row - 1 : b->capacity;
        const WaitCtl wc = make_wait_ctl(b->d_err);
#define IMEX_BATCH_ROWS(D, M) \
    k_batch_rows<D, M><<<grid, rowslp::kThreads, smem, b->stream>>>(b->d_rhdr, b->d_rtab, s, base, rs.stages, cap, wc)
        switch (rs.dir_kb) {
        case 1:
            if (one) IMEX_BATCH_ROWS(1024, 1);
            else IMEX_BATCH_ROWS(1024, 2);
            break;
        case 2:
            if (one) IMEX_BATCH_ROWS(2048, 1);
            else IMEX_BATCH_ROWS(2048, 2);
            break;
        case 4: IMEX_BATCH_ROWS(4096, 1); break;
        default: return cudaErrorInvalidValue;
        }
#undef IMEX_BATCH_ROWS
        return cudaGetLastError();
    }
    return cudaSuccess;
}

// Steps a member still owes before its limit.
int64_t owed(const imex_batch* b, size_t m, int64_t want)
{
    if (b->limit[m] < 0) return want;
    const int64_t left = b->limit[m] - b->members[m]->steps;
    return left < 0 ? 0 : (left < want ? left : want);
}

// Rows per work item of a member in the row kernel under shape rs
// (rowslp::item_rows); 0 if the member stays in the cell kernel.
int rows_per_item(const imex_lattice* h, const RowShape& rs)
{
    if (rs.stages <= 0 || (h->precision == IMEX_F32 && !rs.f32)) return 0;
    const size_t row_bytes = (size_t)h->g.nz * lattice_elem_size(h->precision);
    const size_t cap = (size_t)rs.dir_kb * 1024;
    if (row_bytes % 16 || row_bytes > cap) return 0;
    if ((size_t)h->g.nx * h->g.ny >= 0x7fffffffu) return 0;
    return rowslp::item_rows(h->g.ny, h->g.nz, (int)lattice_elem_size(h->precision), (int)cap);
}

// Write the member tables for a tick where member m runs steps[m] fused
// steps under row shape rs and cell-kernel shape sh, and upload them
// (stream-ordered).  In the cell kernel's packed index every member starts
// on a boundary of sh's chunk (threads x cells per thread).
int upload_table(imex_batch* b, const std::vector<int>& steps, const RowShape& rs, const BatchShape& sh)
{
    const bool units = sh.cpt == 0;  // one CTA per row segment: the index counts segments
    const unsigned long long chunk = (unsigned long long)(sh.threads > 0 ? sh.threads : 256) * (sh.cpt > 0 ? sh.cpt : 1);
    unsigned long long begin = 0;
    unsigned ibegin = 0;
    int n = 0, nr = 0, n16 = 0;
    for (size_t m = 0; m < b->members.size(); ++m) {
        imex_lattice* h = b->members[m];
        const int B = rows_per_item(h, rs);
        if (!B && h->precision != IMEX_F32) ++n16;
        BatchEntry& e = B ? b->h_rtab[nr++] : b->h_tab[n++];
        e.plane = h->ncells;
        e.buf[0] = h->buf[0];
        e.buf[1] = h->buf[1];
        e.nx = h->g.nx;
        e.ny = h->g.ny;
        e.nz = h->g.nz;
        e.prec = h->precision;
        e.cur = h->cur;
        e.steps = steps[m];
        e.eps = h->cf32.eps;
        e.sr = h->cf32.sr;
        e.seed = (uint32_t)h->steps;
        e.B = B;
        e.pad = 0;
        if (B) {
            e.begin = 0;
            e.ibegin = ibegin;
            ibegin += (unsigned)((size_t)h->g.nx * rowslp::y_blocks(h->g.ny, B));
        } else {
            e.begin = begin;
            e.ibegin = 0;
            if (units)
                begin += (unsigned long long)h->g.nx * h->g.ny * ((h->g.nz + kUnitCells - 1) / kUnitCells);
            else
                begin += (h->ncells + chunk - 1) / chunk * chunk;
        }
    }
    b->h_hdr->total = begin;
    b->h_hdr->count = n;
    if (units && n > 0) {
        if (begin > 0x7fffffffull) return bfail(b, IMEX_ERR_ARG, "imex_batch_step: too many row segments for one launch");
        const size_t groups = (size_t)((begin + kUnitGroup - 1) / kUnitGroup);
        if (groups > b->group_cap) {
            if (b->d_group) cudaFreeAsync(b->d_group, b->stream);
            if (b->h_group) cudaFreeHost(b->h_group);
            b->d_group = nullptr;
            b->h_group = nullptr;
            b->group_cap = 0;
            const size_t cap = groups * 2;
            B_CUDA(b, cudaMallocAsync((void**)&b->d_group, cap * sizeof(int), b->stream), "cudaMallocAsync");
            B_CUDA(b, cudaMallocHost((void**)&b->h_group, cap * sizeof(int)), "cudaMallocHost");
            b->group_cap = cap;
        }
        int m = 0;
        for (size_t q = 0; q < groups; ++q) {
            const unsigned long long u = (unsigned long long)q * kUnitGroup;
            while (m + 1 < n && b->h_tab[m + 1].begin <= u) ++m;
            b->h_group[q] = m;
        }
        B_CUDA(b, cudaMemcpyAsync(b->d_group, b->h_group, groups * sizeof(int), cudaMemcpyHostToDevice, b->stream),
               "cudaMemcpyAsync");
    }
    b->h_rhdr->total = ibegin;
    b->h_rhdr->count = nr;
    b->n_cell = n;
    b->n_row = nr;
    b->n_cell_f16 = n16;
    B_CUDA(b, cudaMemcpyAsync(b->d_tab, b->h_tab, sizeof(BatchEntry) * (n ? n : 1), cudaMemcpyHostToDevice, b->stream),
           "cudaMemcpyAsync");
    B_CUDA(b, cudaMemcpyAsync(b->d_hdr, b->h_hdr, sizeof(BatchHeader), cudaMemcpyHostToDevice, b->stream),
           "cudaMemcpyAsync");
    B_CUDA(b, cudaMemcpyAsync(b->d_rtab, b->h_rtab, sizeof(BatchEntry) * (nr ? nr : 1), cudaMemcpyHostToDevice,
                              b->stream),
           "cudaMemcpyAsync");
    B_CUDA(b, cudaMemcpyAsync(b->d_rhdr, b->h_rhdr, sizeof(RowsHeader), cudaMemcpyHostToDevice, b->stream),
           "cudaMemcpyAsync");
    // the pinned staging is reused next tick: wait until the copies are done
    B_CUDA(b, cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    return IMEX_OK;
}

// Make the batch stream wait for every member's queued work.
int join_members(imex_batch* b)
{
    for (imex_lattice* h : b->members) {
        B_CUDA(b, cudaEventRecord(b->done, h->stream), "cudaEventRecord");
        B_CUDA(b, cudaStreamWaitEvent(b->stream, b->done, 0), "cudaStreamWaitEvent");
    }
    return IMEX_OK;
}

// Make every member stream wait for the batch stream.
int release_members(imex_batch* b)
{
    B_CUDA(b, cudaEventRecord(b->done, b->stream), "cudaEventRecord");
    for (imex_lattice* h : b->members) B_CUDA(b, cudaStreamWaitEvent(h->stream, b->done, 0), "cudaStreamWaitEvent");
    return IMEX_OK;
}

std::vector<BatchShape> candidates()
{
    std::vector<BatchShape> out;
    out.push_back(BatchShape{kUnitCells, 0, 0});  // one CTA per row segment
    const int threads[2] = {128, 256};
    const int cpts[3] = {1, 2, 4};
    const int ctas[4] = {2, 4, 8, 9};
    for (int t : threads)
        for (int c : cpts)
            for (int k : ctas) {
                if (t * k > 2048 || (k == 9 && (t != 128 || c != 1))) continue;  // 9: the lean kernel's residency
                BatchShape s;
                s.threads = t;
                s.cpt = c;
                s.ctas_per_sm = k;
                out.push_back(s);
            }
    return out;
}

// Row-kernel shapes (stages, KiB per direction, CTAs per SM); those whose
// CTAs do not fit an SM's shared memory with the batch's table are skipped.
std::vector<RowShape> row_candidates()
{
    const int shapes[][3] = {{2, 2, 2}, {2, 1, 2}, {3, 1, 2}, {2, 2, 1}, {3, 2, 1}, {2, 4, 1}};
    std::vector<RowShape> out;
    for (const auto& x : shapes) {
        RowShape r;
        r.stages = x[0];
        r.dir_kb = x[1];
        r.ctas_per_sm = x[2];
        out.push_back(r);
    }
    return out;
}

// Milliseconds per step of shapes (sh, rs) on the current members: step 0
// of a one-step tick reads buf[cur] and writes the other buffer, leaving
// every member's state as it was.
int time_step(imex_batch* b, const BatchShape& sh, const RowShape& rs, float* ms)
{
    std::vector<int> one(b->members.size(), 1);
    int rc = upload_table(b, one, rs, sh);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    B_CUDA(b, cudaEventCreate(&e0), "cudaEventCreate");
    B_CUDA(b, cudaEventCreate(&e1), "cudaEventCreate");
    cudaError_t e = launch_step(b, sh, rs, 0);  // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(e0, b->stream);
    for (int r = 0; r < 3 && e == cudaSuccess; ++r) e = launch_step(b, sh, rs, 0);
    if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return bcuda(b, e, "batch autotune");
    b->launches += 4 * ((b->n_cell > 0) + (b->n_row > 0));
    *ms = t / 3;
    return IMEX_OK;
}

// Pick the launch shapes.  First the row kernel's: each shape, with and
// without the float32 members, against the row kernel off, the members it
// leaves in the cell kernel at the cell kernel's current (or default)
// shape; then the cell kernel's shapes - only if the chosen split leaves it
// members, and timed on that split.  Shapes pinned by imex_batch_set_launch
// / imex_batch_set_row_launch are kept.  Each timing is one warm-up and
// three steps of the whole batch, so the order matters for a large batch:
// float16-deviation members usually go to the row kernel and float32 ones
// to the one-CTA-per-segment cell kernel, and the cell kernel's other
// shapes are timed only on what is left to it.
int tune_batch(imex_batch* b, bool tune_cells, bool tune_rows)
{
    const RowShape off{-1, 0, 0, 1};
    // the row kernel's shapes are weighed against the cell kernel's usual
    // best, one CTA per row segment
    if (!b->shape.threads) b->shape = BatchShape{kUnitCells, 0, 0};
    if (tune_rows) {
        float best = 0.f;
        int rc = time_step(b, b->shape, off, &best);
        if (rc) return rc;
        RowShape best_rs = off;
        for (RowShape rs : row_candidates()) {
            if (!rows_fit(rs, b->capacity)) continue;
            for (int f32 = 1; f32 >= 0; --f32) {
                rs.f32 = f32;
                float ms = 0.f;
                rc = time_step(b, b->shape, rs, &ms);
                if (rc) return rc;
                if (b->n_row > 0 && ms < best) {
                    best = ms;
                    best_rs = rs;
                }
            }
        }
        b->rshape = best_rs;
    }
    if (tune_cells) {
        std::vector<int> one(b->members.size(), 1);
        int rc = upload_table(b, one, b->rshape, b->shape);
        if (rc) return rc;
        if (b->n_cell > 0) {
            float best = 0.f;
            BatchShape best_shape;
            for (const BatchShape& sh : candidates()) {
                float ms = 0.f;
                rc = time_step(b, sh, b->rshape, &ms);
                if (rc) return rc;
                if (!best_shape.threads || ms < best) {
                    best = ms;
                    best_shape = sh;
                }
            }
            b->shape = best_shape;
        }
    }
    return IMEX_OK;
}

// Capture K steps (s = 0..K-1) of the current shapes into a graph.
int capture_graph(imex_batch* b, int K)
{
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    cudaGraph_t g = nullptr;
    B_CUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    cudaError_t e = cudaSuccess;
    for (int s = 0; s < K && e == cudaSuccess; ++s) e = launch_step(b, b->shape, b->rshape, s);
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) return bcuda(b, e, "batch graph capture");
    b->graph_k = K;
    b->graph_shape = b->shape;
    b->graph_rshape = b->rshape;
    b->graph_kinds = kinds(b);
    b->graph_units = b->h_hdr->total;
    b->graph_group = b->d_group;
    return IMEX_OK;
}

// Whether the captured graph still describes the launches: the same shapes
// and kernels, and for the segment kernel the same segment count (its grid)
// and the same group table (a pointer baked into the graph; upload_table
// moves the table when a tick or a tuning candidate needs a larger one).
bool graph_valid(const imex_batch* b, int K)
{
    return b->graph && b->graph_k == K && b->graph_shape.threads == b->shape.threads &&
           b->graph_shape.cpt == b->shape.cpt && b->graph_shape.ctas_per_sm == b->shape.ctas_per_sm &&
           b->graph_rshape.stages == b->rshape.stages && b->graph_rshape.dir_kb == b->rshape.dir_kb &&
           b->graph_rshape.f32 == b->rshape.f32 &&
           b->graph_rshape.ctas_per_sm == b->rshape.ctas_per_sm && b->graph_kinds == kinds(b) &&
           (b->shape.cpt != 0 || b->n_cell == 0 || (b->graph_units == b->h_hdr->total && b->graph_group == b->d_group));
}

}  // namespace

extern "C" {

int imex_batch_create(int max_members, imex_batch** out)
{
    if (!out) return set_thread_error(IMEX_ERR_ARG, "imex_batch_create: null output");
    *out = nullptr;
    if (max_members < 1 || max_members > kBatchMax)
        return set_thread_error(IMEX_ERR_ARG, "imex_batch_create: max_members must be in [1, 2048]");
    imex_batch* b = new imex_batch();
    b->capacity = max_members;
    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_hdr, sizeof(BatchHeader));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_tab, sizeof(BatchEntry) * max_members);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_hdr, sizeof(BatchHeader));
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_tab, sizeof(BatchEntry) * max_members);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_rhdr, sizeof(RowsHeader));
    if (e == cudaSuccess) e = cudaMalloc(&b->d_rtab, sizeof(BatchEntry) * max_members);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_rhdr, sizeof(RowsHeader));
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_rtab, sizeof(BatchEntry) * max_members);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_err, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(b->d_err, 0, sizeof(unsigned));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_batch_rows<1024, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_batch_rows<1024, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_batch_rows<2048, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_batch_rows<2048, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_batch_rows<4096, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e != cudaSuccess) {
        imex_batch_destroy(b);
        cudaGetLastError();
        return set_thread_error(IMEX_ERR_CUDA, std::string("imex_batch_create: ") + cudaGetErrorString(e));
    }
    b->graph_steps = 16;
    *out = b;
    return IMEX_OK;
}

void imex_batch_destroy(imex_batch* b)
{
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->d_hdr) cudaFree(b->d_hdr);
    if (b->d_tab) cudaFree(b->d_tab);
    if (b->h_hdr) cudaFreeHost(b->h_hdr);
    if (b->h_tab) cudaFreeHost(b->h_tab);
    if (b->d_rhdr) cudaFree(b->d_rhdr);
    if (b->d_rtab) cudaFree(b->d_rtab);
    if (b->h_rhdr) cudaFreeHost(b->h_rhdr);
    if (b->h_rtab) cudaFreeHost(b->h_rtab);
    if (b->d_err) cudaFree(b->d_err);
    if (b->d_group) cudaFree(b->d_group);
    if (b->h_group) cudaFreeHost(b->h_group);
    if (b->done) cudaEventDestroy(b->done);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

int imex_batch_add(imex_batch* b, imex_lattice* h, int64_t max_steps)
{
    if (!b || !h) return set_thread_error(IMEX_ERR_ARG, "imex_batch_add: null argument");
    if (h->precision == IMEX_F64)
        return bfail(b, IMEX_ERR_ARG, "imex_batch_add: members must use float32 or float16-deviation storage");
    if (h->tag == kUninit) return bfail(b, IMEX_ERR_STATE, "imex_batch_add: lattice not initialised");
    if (h->device != b->device) return bfail(b, IMEX_ERR_ARG, "imex_batch_add: lattice is on another device");
    if (h->ncells >= 0xffffffffull) return bfail(b, IMEX_ERR_ARG, "imex_batch_add: members need fewer than 2^32 cells");
    if ((int)b->members.size() >= b->capacity) return bfail(b, IMEX_ERR_MEMORY, "imex_batch_add: batch is full");
    for (imex_lattice* m : b->members)
        if (m == h) return bfail(b, IMEX_ERR_ARG, "imex_batch_add: lattice already in the batch");
    b->members.push_back(h);
    b->limit.push_back(max_steps);
    return IMEX_OK;
}

int imex_batch_remove(imex_batch* b, imex_lattice* h)
{
    if (!b || !h) return set_thread_error(IMEX_ERR_ARG, "imex_batch_remove: null argument");
    for (size_t m = 0; m < b->members.size(); ++m)
        if (b->members[m] == h) {
            B_CUDA(b, cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
            b->members.erase(b->members.begin() + m);
            b->limit.erase(b->limit.begin() + m);
            return IMEX_OK;
        }
    return bfail(b, IMEX_ERR_ARG, "imex_batch_remove: lattice not in the batch");
}

int imex_batch_size(const imex_batch* b) { return b ? (int)b->members.size() : -1; }

int imex_batch_step(imex_batch* b, int nsteps)
{
    if (!b) return set_thread_error(IMEX_ERR_ARG, "imex_batch_step: null batch");
    if (nsteps < 0) return bfail(b, IMEX_ERR_ARG, "imex_batch_step: nsteps < 0");
    if (b->members.empty() || nsteps == 0) return IMEX_OK;
    B_CUDA(b, cudaSetDevice(b->device), "cudaSetDevice");
    // Members whose reference f sits in the buffer (just initialised, or
    // after get_f) take their first Collision alone (in place), then mark
    // the streaming pending; every further step is a fused batched step.
    std::vector<int64_t> left(b->members.size());
    for (size_t m = 0; m < b->members.size(); ++m) {
        imex_lattice* h = b->members[m];
        left[m] = owed(b, m, nsteps);
        if (left[m] > 0 && h->tag == kExact) {
            int rc = imex_collision(h);
            if (!rc) rc = imex_streaming(h);
            if (rc) return bfail(b, rc, std::string("imex_batch_step: ") + imex_last_error(h));
            --left[m];
        }
    }
    int rc = join_members(b);
    if (rc) return rc;
    if (!b->shape.threads || !b->rshape.stages) {
        rc = tune_batch(b, !b->shape.threads, !b->rshape.stages);
        if (rc) return rc;
    }
    std::vector<int> tick(b->members.size());
    for (;;) {
        int64_t most = 0;
        for (size_t m = 0; m < left.size(); ++m) most = std::max(most, left[m]);
        if (most == 0) break;
        const int K = b->graph_steps > 0 ? b->graph_steps : 1;
        const int k = (int)std::min<int64_t>(most, K);
        for (size_t m = 0; m < left.size(); ++m) tick[m] = (int)std::min<int64_t>(left[m], k);
        rc = upload_table(b, tick, b->rshape, b->shape);
        if (rc) return rc;
        if (b->graph_steps > 0 && k == b->graph_steps) {
            if (!graph_valid(b, k)) {
                rc = capture_graph(b, k);
                if (rc) return rc;
            }
            B_CUDA(b, cudaGraphLaunch(b->graph, b->stream), "cudaGraphLaunch");
        } else {
            for (int s = 0; s < k; ++s) B_CUDA(b, launch_step(b, b->shape, b->rshape, s), "batch kernel launch");
        }
        b->launches += (int64_t)k * ((b->n_cell > 0) + (b->n_row > 0));
        for (size_t m = 0; m < left.size(); ++m) {
            imex_lattice* h = b->members[m];
            h->cur ^= tick[m] & 1;
            h->steps += tick[m];
            h->launches += tick[m];
            left[m] -= tick[m];
        }
    }
    return release_members(b);
}

int imex_batch_synchronize(imex_batch* b)
{
    if (!b) return set_thread_error(IMEX_ERR_ARG, "imex_batch_synchronize: null batch");
    unsigned v = 0;
    B_CUDA(b, cudaMemcpyAsync(&v, b->d_err, sizeof v, cudaMemcpyDeviceToHost, b->stream), "cudaMemcpyAsync");
    B_CUDA(b, cudaStreamSynchronize(b->stream), "imex_batch_synchronize");
    if (v) {
        B_CUDA(b, cudaMemset(b->d_err, 0, sizeof v), "cudaMemset");
        return bfail(b, IMEX_ERR_CUDA, (v & 2u) ? "imex_batch_synchronize: the row kernel's member table exceeded "
                                                  "its shared memory; the members' results are invalid"
                                                : "imex_batch_synchronize: a row kernel's asynchronous copy did not "
                                                  "complete in time; the members' results are invalid");
    }
    return IMEX_OK;
}

int imex_batch_set_launch(imex_batch* b, int threads, int cells_per_thread, int ctas_per_sm)
{
    if (!b) return set_thread_error(IMEX_ERR_ARG, "imex_batch_set_launch: null batch");
    if (threads == 0) {
        b->shape = BatchShape{};
        return IMEX_OK;
    }
    if (cells_per_thread == 0) {  // one CTA of 128 threads per row segment
        if (threads != kUnitCells)
            return bfail(b, IMEX_ERR_ARG, "imex_batch_set_launch: cells_per_thread 0 (one CTA per row segment) "
                                          "takes 128 threads");
        b->shape = BatchShape{kUnitCells, 0, 0};
        return IMEX_OK;
    }
    if ((threads != 128 && threads != 256) || (cells_per_thread != 1 && cells_per_thread != 2 && cells_per_thread != 4) ||
        ctas_per_sm < 1 || ctas_per_sm * threads > 2048)
        return bfail(b, IMEX_ERR_ARG, "imex_batch_set_launch: threads 128|256, cells_per_thread 0|1|2|4, "
                                      "ctas_per_sm*threads <= 2048");
    b->shape.threads = threads;
    b->shape.cpt = cells_per_thread;
    b->shape.ctas_per_sm = ctas_per_sm;
    return IMEX_OK;
}

int imex_batch_get_launch(imex_batch* b, int out[3])
{
    if (!b || !out) return set_thread_error(IMEX_ERR_ARG, "imex_batch_get_launch: null argument");
    out[0] = b->shape.threads;
    out[1] = b->shape.cpt;
    out[2] = b->shape.ctas_per_sm;
    return IMEX_OK;
}

int imex_batch_set_row_launch(imex_batch* b, int stages, int dir_kb, int ctas_per_sm, int float32_members)
{
    if (!b) return set_thread_error(IMEX_ERR_ARG, "imex_batch_set_row_launch: null batch");
    if (stages == 0 || stages == -1) {  // 0: autotune, -1: row kernel off
        b->rshape = RowShape{stages, 0, 0, 1};
        return IMEX_OK;
    }
    const RowShape rs{stages, dir_kb, ctas_per_sm, float32_members ? 1 : 0};
    if (stages < 2 || stages > 8 || (dir_kb != 1 && dir_kb != 2 && dir_kb != 4) || ctas_per_sm < 1 ||
        ctas_per_sm > 4 || !rows_fit(rs, b->capacity))
        return bfail(b, IMEX_ERR_ARG, "imex_batch_set_row_launch: 2 <= stages <= 8, dir_kb 1, 2 or 4, 1 <= "
                                      "ctas_per_sm <= 4, and the CTAs' rings must fit an SM's shared memory");
    b->rshape = rs;
    return IMEX_OK;
}

int imex_batch_get_row_launch(imex_batch* b, int out[4])
{
    if (!b || !out) return set_thread_error(IMEX_ERR_ARG, "imex_batch_get_row_launch: null argument");
    out[0] = b->rshape.stages;
    out[1] = b->rshape.dir_kb;
    out[2] = b->rshape.ctas_per_sm;
    out[3] = b->rshape.f32;
    return IMEX_OK;
}

int imex_batch_set_graph(imex_batch* b, int steps_per_graph)
{
    if (!b || steps_per_graph < 0) return set_thread_error(IMEX_ERR_ARG, "imex_batch_set_graph: bad argument");
    b->graph_steps = steps_per_graph;
    return IMEX_OK;
}

int64_t imex_batch_kernel_launches(const imex_batch* b) { return b ? b->launches : -1; }

const char* imex_batch_last_error(const imex_batch* b) { return b ? b->err.c_str() : imex::thread_error(); }

}  // extern "C"
