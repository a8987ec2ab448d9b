// Row-kernel engine of the reduced-precision formats: the float32 collision
// of one staged cell (used by the one-lattice row kernel, rows.cuh, and the
// batched row kernel, batch.cu).
#pragma once

#include "lowp_math.cuh"
#include "rows.cuh"

namespace imex {

// Row-kernel engine: float32 collision of one staged cell.
template <int P>
struct EngLowp {
    using T = typename lowp::Storage<P>::T;
    static constexpr int kMinBlocks = 4;
    CollideF32 cp;

    __device__ __forceinline__ void run(const T* __restrict__ st, int astride, int nz, int z, T* __restrict__ dst,
                                        size_t plane, size_t rowoff) const
    {
        const int zm = z == 0 ? nz - 1 : z - 1, zp = z == nz - 1 ? 0 : z + 1;
        float h[kQ];
#pragma unroll
        for (int a = 0; a < kQ; ++a) h[a] = lowp::Storage<P>::load_plain(st + a * astride + pull_z(ex(a, 2), z, zm, zp), a);
        lowp::collide_dev_f32<P>(h, cp);
        if constexpr (P == IMEX_F16DEV) {
            auto at = [&](int a) -> T& { return dst[(size_t)a * plane + rowoff + z]; };
            if (cp.sr) lowp::store_f16_cell_sr(h, lowp::sr_hash(rowoff + z, cp.seed), at);
            else lowp::store_f16_cell(h, at);
            return;
        }
#pragma unroll
        for (int a = 0; a < kQ; ++a) dst[(size_t)a * plane + rowoff + z] = lowp::Storage<P>::store(h[a], a);
    }
};

}  // namespace imex
