// Row-staged step of the reduced-precision formats, for one lattice
// (k_rows_lowp) and for a batch of lattices (k_batch_rows, batch.cu).
//
// Work item: B consecutive y-rows (x, y0 .. y0+B-1) of one lattice.  As in
// rows.cuh, the 27 source runs of an item (one per direction: B rows of the
// plane, two runs at the periodic y-wrap) arrive in a ring stage of shared
// memory by bulk copies completing on an mbarrier, the copies of item
// t + S - 1 in flight while item t is collided.  What differs from the
// float64 row kernel cuts instructions per cell, which bound the first
// version of this kernel (75% of issue slots busy, ~600 thread instructions
// per float16 cell):
//   - each thread takes two neighbouring z cells and collides them in lock
//     step with the packed f32x2 instructions (lowp_math.cuh, collide_dev
//     with F2): one instruction for both cells' arithmetic;
//   - a direction's block in a stage sits at a compile-time offset
//     (kDirBytes per direction), so shared-memory addressing is immediate;
//   - the pair's two results of a direction leave as one 32-bit (float16)
//     or 64-bit (float32) store, coalesced along z across the warp.
// Items of 2 KB per direction (B = 4 rows of 256 float16 values) measured
// 296 us per 256^3 float16 step (57 GLUPS, 91% of the copy bandwidth);
// 1 KB items 369 us; staging the outputs in shared memory for bulk stores
// instead of storing them directly, 403 us; 4 KB items (B = 8), 283 us
// (59.3 GLUPS).  Float16 results go through round_f16_conserving (each
// cell's momentum kept); stochastic rounding packs the pair with
// cvt.rs.f16x2.f32 and the pair's random words (sr_word), the same bits the
// one-cell kernels use.
//
// Requirements: nz * element size a multiple of 16 bytes (so nz is even and
// every run is 16-byte aligned), B * nz * element size <= kDirBytes.  B
// need not divide ny: the last item of each x plane takes the rows left.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "bulk.cuh"
#include "kernels_common.cuh"
#include "lowp_math.cuh"

namespace imex {
namespace rowslp {

constexpr int kThreads = 256;
constexpr int kMaxStages = 16;
constexpr int kBarBytes = 128;  // kMaxStages mbarriers

// One work item.
struct Item {
    const unsigned char* src;  // the lattice's source and destination buffers
    unsigned char* dst;
    size_t plane;  // cells per direction plane
    int nx, ny, nz, B, x, y0;
    int prec;  // IMEX_F32 or IMEX_F16DEV
    float eps;
    int sr;
    uint32_t seed;
    bool active;  // false: skip (member done for this tick)
};

__device__ __forceinline__ uint32_t elem_bytes(int prec) { return prec == IMEX_F32 ? 4u : 2u; }

// Descriptors of the items in flight: one slot more than the stages, so
// that an item's slot is rewritten only after every thread has finished
// the item (128-byte aligned).
constexpr int kSlotBytes = (int)(((kMaxStages + 1) * sizeof(Item) + 127) / 128 * 128);

// Shared memory of a CTA: barriers, item descriptors and `stages` ring stages.
__host__ __device__ inline size_t smem_bytes(int dir_bytes, int stages)
{
    return kBarBytes + kSlotBytes + (size_t)stages * kQ * dir_bytes;
}

// Rows per work item for a lattice of ny rows of nz cells of es bytes in a
// stage with dir_bytes per direction: the B (B * nz * es <= dir_bytes) whose
// items - ceil(ny / B) per x plane, the last one ny mod B rows when B does
// not divide ny - keep the CTA's threads busiest, counting half a round of
// kThreads pairs per item for its barrier and copies: the score
// pairs / (sum over items of (rounds + 1/2) kThreads).  A 96-wide float16
// lattice, for one, takes B = 10 in a 2 KB block (9 items of 480 pairs and
// one of 288 per plane) rather than the largest divisor 8 (384 pairs, a half
// idle second round).  0 if a single row does not fit.
inline int item_rows(int ny, int nz, int es, int dir_bytes)
{
    const long long row = (long long)nz * es;
    if (row > dir_bytes) return 0;
    auto rounds = [](long long pairs) { return (pairs + kThreads - 1) / kThreads; };
    const long long total = (long long)ny * nz / 2;
    int best = 0;
    double best_score = -1.0;
    for (int B = 1; B <= ny && (long long)B * row <= dir_bytes; ++B) {
        const int full = ny / B, last = ny % B;
        double cost = full * (rounds((long long)B * nz / 2) + 0.5);
        if (last) cost += rounds((long long)last * nz / 2) + 0.5;
        const double score = (double)total / (cost * kThreads);
        if (score >= best_score) {
            best_score = score;
            best = B;
        }
    }
    return best;
}

// Number of y-blocks of a plane with items of B rows.
__host__ __device__ inline int y_blocks(int ny, int B) { return (ny + B - 1) / B; }

// Collide the item staged at `in` into the lattice's destination buffer;
// Ar is the two-cell arithmetic (lowp::F2).
template <int P, int kDirBytes, class Ar>
__device__ __forceinline__ void compute_item(const unsigned char* __restrict__ in, const Item& it,
                                             const CollideF32& base)
{
    using S = lowp::Storage<P>;
    using T = typename S::T;
    constexpr int kDir = kDirBytes / (int)sizeof(T);
    const T* st = reinterpret_cast<const T*>(in);
    CollideF32 cp = base;
    cp.eps = it.eps;
    cp.sr = it.sr;
    cp.seed = it.seed;
    const int nz = it.nz, half = nz >> 1, npairs = it.B * half;
    const unsigned long long row0 = ((unsigned long long)it.x * it.ny + it.y0) * nz;  // item's first cell
    // (b, zp): row and z pair of pair q; advanced by kThreads pairs a step
    int b = threadIdx.x / half, zp = threadIdx.x - b * half;
    const int db = kThreads / half, dz = kThreads - db * half;
    for (int q = threadIdx.x; q < npairs; q += kThreads) {
        const int z = 2 * zp;
        const int zm = z == 0 ? nz - 1 : z - 1;    // source of cell z along ez = +1
        const int z2 = z + 2 == nz ? 0 : z + 2;    // source of cell z + 1 along ez = -1
        const T* r = st + b * nz;
        float2 h[kQ];
#pragma unroll
        for (int a = 0; a < kQ; ++a) {
            const T* ra = r + a * kDir;
            const int e = ex(a, 2);
            T v0, v1;
            if (e == 0) {  // the pair itself: one aligned 2-element load
                if constexpr (P == IMEX_F16DEV) {
                    const __half2 v = *reinterpret_cast<const __half2*>(ra + z);
                    v0 = __low2half(v);
                    v1 = __high2half(v);
                } else {
                    const float2 v = *reinterpret_cast<const float2*>(ra + z);
                    v0 = v.x;
                    v1 = v.y;
                }
            } else {
                v0 = e == 1 ? ra[zm] : ra[z + 1];
                v1 = e == 1 ? ra[z] : ra[z2];
            }
            h[a] = make_float2(S::dev(v0, a), S::dev(v1, a));
        }
        lowp::collide_dev<P, Ar>(h, cp);
        T* o = reinterpret_cast<T*>(it.dst) + row0 + (size_t)b * nz + z;
        if constexpr (P == IMEX_F16DEV) {
            // one rounding loop per mode (a branch per direction costs
            // issue slots in this instruction-heavy loop)
            if (cp.sr) {
                const uint32_t ph = lowp::sr_hash((row0 + (unsigned long long)b * nz + z) >> 1, cp.seed);
                const uint32_t pc = lowp::sr_corner_hash(ph);
                lowp::round_f16_conserving<Ar>(h, [&](int a, float2 v) -> float2 {
                    const uint32_t w = lowp::cvt_rs_f16x2(v.y, v.x, lowp::sr_word(ph, pc, a));
                    const __half2 r = *reinterpret_cast<const __half2*>(&w);
                    *reinterpret_cast<__half2*>(o + (size_t)a * it.plane) = r;
                    return make_float2(lowp::sub_f16_f32(__low2half(r), v.x), lowp::sub_f16_f32(__high2half(r), v.y));
                });
            } else {
                lowp::round_f16_conserving<Ar>(h, [&](int a, float2 v) -> float2 {
                    const __half2 r = __floats2half2_rn(v.x, v.y);
                    *reinterpret_cast<__half2*>(o + (size_t)a * it.plane) = r;
                    return make_float2(lowp::sub_f16_f32(__low2half(r), v.x), lowp::sub_f16_f32(__high2half(r), v.y));
                });
            }
        } else {
#pragma unroll
            for (int a = 0; a < kQ; ++a) {
                const float wa = (float)weight(a);
                *reinterpret_cast<float2*>(o + (size_t)a * it.plane) = make_float2(wa + h[a].x, wa + h[a].y);
            }
        }
        zp += dz;
        b += db;
        if (zp >= half) {
            zp -= half;
            ++b;
        }
    }
}

// The persistent loop of one CTA over its items t = 0 .. my-1 (item_of(t)
// describes item t).  smem: kBarBytes of mbarriers, stages + 1 descriptor
// slots, then `stages` stages of 27 * kDirBytes.  Thread 0 describes each
// item once, when it arms the item's stage, into slot t % (stages + 1);
// the other threads read the slot (a member lookup per item per thread - a
// binary search and a table read for a batch - would sit in front of every
// item's loads and arithmetic).  Slot t is rewritten by arm(t + stages + 1)
// at the end of iteration t + 1, after the barrier that ends item t.
//
// kSlots false: every thread describes the items itself (one lattice: a
// division, cheaper than the shared-memory reads).
template <int kDirBytes, class Ar, bool kSlots, class ItemOf>
__device__ __forceinline__ void run_items(const ItemOf& item_of, int my, int stages, const CollideF32& base,
                                          unsigned char* smem, const WaitCtl& wc)
{
    constexpr uint32_t kStage = (uint32_t)kQ * kDirBytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem);
    Item* slots = reinterpret_cast<Item*>(smem + kBarBytes);
    unsigned char* ring = smem + kBarBytes + kSlotBytes;
    constexpr int nwarps = kThreads / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int my_dir = warp + nwarps * lane;  // copies of direction my_dir are issued by this lane
    const bool issuer = my_dir < kQ;

    const int nslots = stages + 1;
    // Thread 0 describes item t and arms its stage's next phase.  An item
    // with no bytes (a batch member done for the tick) completes that phase
    // at its arrival; with defer_empty the arrival is left to the caller
    // (returns true), who makes it only once every thread has passed its
    // wait on the stage's previous phase - completed early, the phase would
    // flip the stage's parity back under a thread still waiting on it, and
    // that thread's parity wait would run out.
    auto arm = [&](int t, bool defer_empty) -> bool {
        const Item it = item_of(t);
        if (kSlots) slots[t % nslots] = it;
        if (!it.active && defer_empty) return true;
        const uint32_t bytes = it.active ? (uint32_t)kQ * it.B * it.nz * elem_bytes(it.prec) : 0u;
        bulk::mbar_arrive_expect_tx(&full[t % stages], bytes);
        return false;
    };
    auto issue = [&](int t) {  // after the barrier that follows arm(t)
        const Item it = kSlots ? slots[t % nslots] : item_of(t);
        if (!it.active) return;
        if (t == 0 && (int)blockIdx.x == wc.starve_cta) return;  // test hook: stage 0 never fills
        const uint32_t es = elem_bytes(it.prec);
        const uint32_t row_bytes = (uint32_t)it.nz * es;
        const int a = my_dir, B = it.B, ny = it.ny;
        int xs = it.x - ex(a, 0);
        xs = xs < 0 ? xs + it.nx : xs >= it.nx ? xs - it.nx : xs;
        const unsigned char* pl = it.src + ((size_t)a * it.plane + (size_t)xs * ny * it.nz) * es;
        unsigned char* s = ring + (size_t)(t % stages) * kStage + (size_t)a * kDirBytes;
        uint64_t* bar = &full[t % stages];
        const int lo = it.y0 - ex(a, 1);  // source row of the item's first row
        if (lo < 0) {
            bulk::copy_g2s(s, pl + (size_t)(ny - 1) * row_bytes, row_bytes, bar);
            if (B > 1) bulk::copy_g2s(s + row_bytes, pl, (uint32_t)(B - 1) * row_bytes, bar);
        } else if (lo + B > ny) {
            if (B > 1) bulk::copy_g2s(s, pl + (size_t)lo * row_bytes, (uint32_t)(B - 1) * row_bytes, bar);
            bulk::copy_g2s(s + (size_t)(B - 1) * row_bytes, pl, row_bytes, bar);
        } else {
            bulk::copy_g2s(s, pl + (size_t)lo * row_bytes, (uint32_t)B * row_bytes, bar);
        }
    };

    if (threadIdx.x == 0) {
        for (int q = 0; q < stages; ++q) bulk::mbar_init(&full[q], 1);
        bulk::fence_mbar_init();
        for (int t = 0; t < stages && t < my; ++t) arm(t, false);  // first item of every stage (no waits yet)
    }
    __syncthreads();
    if (issuer)
        for (int t = 0; t < stages - 1 && t < my; ++t) issue(t);

    // A copy did not complete: record it, wait (bounded) for the copies
    // this CTA still has in flight (items t .. t + stages - 1), and stop.
    auto fail_at = [&](int t) {
        if (threadIdx.x == 0) {
            atomicOr(wc.err, 1u);
            const int last = t + stages - 1 < my ? t + stages - 1 : my - 1;
            for (int q = t; q <= last; ++q)
                bulk::mbar_wait(&full[q % stages], (uint32_t)((q / stages) & 1), wc.cycles);
        }
        __syncthreads();
    };
    for (int t = 0; t < my; ++t) {
        const int s = t % stages;
        if (issuer && t + stages - 1 < my) issue(t + stages - 1);
        const int ok = bulk::mbar_wait(&full[s], (uint32_t)((t / stages) & 1), wc.cycles);
        // One lattice: every thread starts on the item together (measured
        // faster: 59.0 against 55.7 GLUPS at 256^3 float16).  A batch: each
        // warp starts once it sees the stage full, a thread whose wait ran
        // out skips the item, and the barrier that ends the item tells every
        // thread (62.3 against 58.5 GLUPS on four 256^3 float16 lattices).
        if (!kSlots && __syncthreads_or(!ok)) {
            fail_at(t);
            return;
        }
        const Item& it = kSlots ? slots[t % nslots] : item_of(t);
        if (ok && it.active) {
            if (it.prec == IMEX_F32) compute_item<IMEX_F32, kDirBytes, Ar>(ring + (size_t)s * kStage, it, base);
            else compute_item<IMEX_F16DEV, kDirBytes, Ar>(ring + (size_t)s * kStage, it, base);
        }
        // stage s, next use: armed only on a phase thread 0 saw complete
        // (an arrival on a phase still pending would be one too many); in a
        // batch other warps may still be waiting on stage s, so an item with
        // no bytes arrives after the barrier
        bool owed = false;
        if (threadIdx.x == 0 && ok && t + stages < my) owed = arm(t + stages, kSlots);
        if (kSlots) {
            if (__syncthreads_or(!ok)) {  // stage s may be refilled - unless a copy did not complete
                fail_at(t);
                return;
            }
            if (owed) bulk::mbar_arrive_expect_tx(&full[s], 0u);
        } else {
            __syncthreads();  // stage s may be refilled
        }
    }
}

// One lattice: items are the nx * ceil(ny / B) row blocks in x-major order.
// kMinBlocks: resident CTAs per SM the register budget is cut for (1: up to
// 255 registers; 2: 128).
template <int kDirBytes, int kMinBlocks, class Ar = lowp::F2>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
    k_rows_lowp(const void* __restrict__ src, void* __restrict__ dst, Geom g, int prec, int B, CollideF32 cp,
                int stages, WaitCtl wc)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int yblocks = y_blocks(g.ny, B);
    const int items = g.nx * yblocks;
    const int G = gridDim.x;
    const int my = (int)blockIdx.x < items ? (items - 1 - (int)blockIdx.x) / G + 1 : 0;
    auto item_of = [&](int t) {
        Item it;
        const int item = (int)blockIdx.x + t * G;
        it.src = static_cast<const unsigned char*>(src);
        it.dst = static_cast<unsigned char*>(dst);
        it.plane = g.plane;
        it.nx = g.nx;
        it.ny = g.ny;
        it.nz = g.nz;
        it.x = item / yblocks;
        it.y0 = (item - it.x * yblocks) * B;
        it.B = g.ny - it.y0 < B ? g.ny - it.y0 : B;  // the last block of a plane may be shorter
        it.prec = prec;
        it.eps = cp.eps;
        it.sr = cp.sr;
        it.seed = cp.seed;
        it.active = true;
        return it;
    };
    run_items<kDirBytes, Ar, false>(item_of, my, stages, cp, smem, wc);
}

}  // namespace rowslp
}  // namespace imex
