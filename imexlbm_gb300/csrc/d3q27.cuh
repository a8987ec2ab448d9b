// D3Q27 lattice: velocities, weights and the pair structure used by every
// kernel.  The direction ORDER is the reference's (src/lbm.cpp:20-30) because
// distributions cross the C ABI in that order; weights are src/lbm.cpp:9-19.
//
// Direction a = 0 is the rest particle.  For a = 1..26 the directions come in
// opposite pairs (2k-1, 2k), k = 1..13, with e[2k] = -e[2k-1]
// (src/lbm.cpp:32-35).  Kernels work pair-wise: both members share |e.u|,
// the quadratic equilibrium term and the weight.
#pragma once

#include <cstdint>

#ifndef IMEX_HD
#if defined(__CUDACC__)
#define IMEX_HD __host__ __device__ __forceinline__
#else
#define IMEX_HD inline
#endif
#endif

namespace imex {

constexpr int kQ = 27;
constexpr int kPairs = 13;

// Velocity of the first member of pair k (k = 1..13) packed as three base-3
// digits (component + 1): x digit * 9 + y digit * 3 + z digit.
//   k:  1 +x, 2 +y, 3 +z, 4 (+,+,0), 5 (+,-,0), 6 (+,0,+), 7 (+,0,-),
//       8 (0,+,+), 9 (0,+,-), 10 (+,+,+), 11 (+,-,+), 12 (+,+,-), 13 (+,-,-)
IMEX_HD constexpr int pair_code(int k)
{
    return k == 1 ? 2 * 9 + 1 * 3 + 1
         : k == 2 ? 1 * 9 + 2 * 3 + 1
         : k == 3 ? 1 * 9 + 1 * 3 + 2
         : k == 4 ? 2 * 9 + 2 * 3 + 1
         : k == 5 ? 2 * 9 + 0 * 3 + 1
         : k == 6 ? 2 * 9 + 1 * 3 + 2
         : k == 7 ? 2 * 9 + 1 * 3 + 0
         : k == 8 ? 1 * 9 + 2 * 3 + 2
         : k == 9 ? 1 * 9 + 2 * 3 + 0
         : k == 10 ? 2 * 9 + 2 * 3 + 2
         : k == 11 ? 2 * 9 + 0 * 3 + 2
         : k == 12 ? 2 * 9 + 2 * 3 + 0
         : 2 * 9 + 0 * 3 + 0;
}

// Component d (0 = x, 1 = y, 2 = z) of direction a.
IMEX_HD constexpr int ex(int a, int d)
{
    return a == 0 ? 0
         : ((pair_code((a + 1) / 2) / (d == 0 ? 9 : d == 1 ? 3 : 1)) % 3 - 1) * ((a & 1) ? 1 : -1);
}

IMEX_HD constexpr int opposite(int a) { return a == 0 ? 0 : ((a & 1) ? a + 1 : a - 1); }

// Weight times 216: 64 (rest), 16 (axis), 4 (face diagonal), 1 (corner).
IMEX_HD constexpr int weight216(int a)
{
    return (ex(a, 0) != 0) + (ex(a, 1) != 0) + (ex(a, 2) != 0) == 0 ? 64
         : (ex(a, 0) != 0) + (ex(a, 1) != 0) + (ex(a, 2) != 0) == 1 ? 16
         : (ex(a, 0) != 0) + (ex(a, 1) != 0) + (ex(a, 2) != 0) == 2 ? 4
         : 1;
}

// Weight as the reference writes it (8/27, 2/27, 1/54, 1/216), so the
// double constant rounds exactly like the reference's literal division.
IMEX_HD constexpr double weight(int a)
{
    return weight216(a) == 64 ? 8.0 / 27.0
         : weight216(a) == 16 ? 2.0 / 27.0
         : weight216(a) == 4 ? 1.0 / 54.0
         : 1.0 / 216.0;
}

// Compile-time self-checks of the table against its defining properties.
constexpr bool table_ok()
{
    int sw = 0, s[3] = {0, 0, 0}, sxx = 0;
    for (int a = 0; a < kQ; ++a) {
        sw += weight216(a);
        for (int d = 0; d < 3; ++d) {
            s[d] += weight216(a) * ex(a, d);
            if (ex(opposite(a), d) != -ex(a, d)) return false;
        }
        sxx += weight216(a) * ex(a, 0) * ex(a, 0);
        for (int b = 0; b < a; ++b)
            if (ex(a, 0) == ex(b, 0) && ex(a, 1) == ex(b, 1) && ex(a, 2) == ex(b, 2)) return false;
    }
    return sw == 216 && s[0] == 0 && s[1] == 0 && s[2] == 0 && sxx == 72;
}
static_assert(table_ok(), "D3Q27 table is inconsistent");
// Spot checks of the reference ordering (src/lbm.cpp:22-28).
static_assert(ex(1, 0) == 1 && ex(2, 0) == -1 && ex(3, 1) == 1 && ex(6, 2) == -1, "axis order");
static_assert(ex(9, 0) == 1 && ex(9, 1) == -1 && ex(13, 2) == -1 && ex(17, 1) == 1 && ex(17, 2) == -1, "edge order");
static_assert(ex(21, 0) == 1 && ex(21, 1) == -1 && ex(21, 2) == 1, "corner order");
static_assert(ex(25, 0) == 1 && ex(25, 1) == -1 && ex(25, 2) == -1 && ex(26, 0) == -1 && ex(26, 1) == 1 && ex(26, 2) == 1, "corner order");

}  // namespace imex
