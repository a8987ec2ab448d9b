// Exact 64-bit fixed-point arithmetic of the fixed-point float64 engine,
// and the per-cell collision built from it.  Host and device compile the
// same code (the host branch of each intrinsic is a portable restatement),
// so the arithmetic can be checked bit for bit on a CPU.
//
// Representation.  A distribution f is held as X = f * 2^61 in a 64-bit
// integer.  A float64 in [2^-9, 1) converts exactly (its 53-bit mantissa is
// shifted left by 0..8 bits); sums of X are exact, so 3p = sum f and
// u = sum f e are exact.  Products with the collision constants use a 64x64
// high product (error < 2 units of 2^-61, ~1e-18 absolute), the quadratic
// terms drop a < 36-unit low part, and each output is rounded once to
// float64: per value ~0.5 ulp + 1e-17 absolute.
//
// Collision, per opposite pair (a, a') with V = e_a . u (exact integer):
//   B    = 3p - 1.5 u.u + 4.5 V^2
//   f_a  <- (1 - w) f_a  + (w w_a) B + (3 w w_a) V
//   f_a' <- (1 - w) f_a' + (w w_a) B - (3 w w_a) V          (w = omega)
// which is src/lbm.cpp:153-163 with feq expanded (3 pp = sum f).
//
// Exact range: f_0 in [2^-9, 1), other f in [2^-9, 1/8), |e.u| < 1/2,
// 3p < 2, 3p - 1.5 u.u >= 0, every output in [2^-9, 4).  Outside it (a
// negative, tiny or huge value, NaN/Inf) `ok` is cleared and the caller must
// redo the cell in native float64.
#pragma once

#include <cstdint>
#include <cstring>

#include "d3q27.cuh"

namespace imex {

// Kernel constants of the exact fixed-point collision, each a real number
// in [0, 1) times 2^64: omega * w and 3 * omega * w per weight class
// (0 rest, 1 axis, 2 face diagonal, 3 corner) and |omega - 1|.
struct FxConst {
    unsigned long long c_ow[4];
    unsigned long long c_3ow[4];
    unsigned long long c_om1;
};

namespace fx {

constexpr int kFrac = 61;                      // X = f * 2^61
constexpr uint32_t kInShift = 1075 - kFrac;    // s = biased exponent - kInShift
constexpr uint32_t kOutExp = (uint32_t)(1074 - kFrac) << 20;

// ---- portable intrinsics -------------------------------------------------
IMEX_HD uint32_t fshl(uint32_t lo, uint32_t hi, uint32_t s)  // high word of (hi:lo) << (s & 31)
{
#if defined(__CUDA_ARCH__)
    return __funnelshift_l(lo, hi, s);
#else
    s &= 31u;
    return s ? (hi << s) | (lo >> (32u - s)) : hi;
#endif
}

IMEX_HD uint32_t fshr(uint32_t lo, uint32_t hi, uint32_t s)  // low word of (hi:lo) >> (s & 31)
{
#if defined(__CUDA_ARCH__)
    return __funnelshift_r(lo, hi, s);
#else
    s &= 31u;
    return s ? (lo >> s) | (hi << (32u - s)) : lo;
#endif
}

IMEX_HD uint32_t clz32(uint32_t x)
{
#if defined(__CUDA_ARCH__)
    return (uint32_t)__clz((int)x);
#else
    return x ? (uint32_t)__builtin_clz(x) : 32u;
#endif
}

IMEX_HD uint64_t bits_of(double v)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(v);
#else
    uint64_t b;
    std::memcpy(&b, &v, 8);
    return b;
#endif
}

IMEX_HD double double_of(uint32_t hi, uint32_t lo)
{
#if defined(__CUDA_ARCH__)
    return __hiloint2double((int)hi, (int)lo);
#else
    const uint64_t b = ((uint64_t)hi << 32) | lo;
    double v;
    std::memcpy(&v, &b, 8);
    return v;
#endif
}

// ---- conversions ---------------------------------------------------------
// float64 (bit pattern b) -> X for values whose shift s is in [0, smax];
// clears ok otherwise.  The sign bit is part of (hi >> 20), so negatives
// fail.
IMEX_HD uint64_t to_fixed_bits(uint64_t b, uint32_t smax, bool& ok)
{
    const uint32_t lo = (uint32_t)b, hi = (uint32_t)(b >> 32);
    const uint32_t s = (hi >> 20) - kInShift;
    ok = ok && (s <= smax);
    const uint32_t mh = (hi & 0x000FFFFFu) | 0x00100000u;
    return ((uint64_t)fshl(lo, mh, s) << 32) | fshl(0u, lo, s);
}

IMEX_HD uint64_t to_fixed(double v, uint32_t smax, bool& ok) { return to_fixed_bits(bits_of(v), smax, ok); }

// A value already held as X (float64 precision, see round_fixed): the range
// check to_fixed makes on the float64 it stands for, 2^52 <= X < 2^(53 +
// smax), i.e. f in [2^-9, 2^(smax - 8)).
IMEX_HD uint64_t check_fixed(uint64_t x, uint32_t smax, bool& ok)
{
    const uint32_t hi = (uint32_t)(x >> 32);
    ok = ok && (hi - 0x00100000u) < ((0x00200000u << smax) - 0x00100000u);
    return x;
}

// X -> float64 rounded to nearest (ties away from zero) for
// 2^52 <= X < 2^63; clears ok otherwise.
IMEX_HD double from_fixed(uint64_t y, bool& ok)
{
    const uint32_t yh = (uint32_t)(y >> 32);
    const uint32_t r = 11u - clz32(yh);  // bits below the 53-bit mantissa
    ok = ok && (r <= 10u);
    const uint32_t half = fshl(0u, 1u, r) >> 1;
    const uint64_t t = y + half;
    const uint32_t tl = (uint32_t)t, th = (uint32_t)(t >> 32);
    return double_of(fshr(th, 0u, r) + (r << 20) + kOutExp, fshr(tl, th, r));
}

// X -> X rounded to the float64 grid, to nearest with ties away from zero
// (the value from_fixed would return, still in fixed point: the low r bits,
// those below the 53-bit mantissa, cleared after adding half of their
// weight); clears ok outside 2^52 <= X < 2^63.  to_fixed(from_fixed(y)) ==
// round_fixed(y) for every y whose result is in range.
IMEX_HD uint64_t round_fixed(uint64_t y, bool& ok)
{
    const uint32_t yh = (uint32_t)(y >> 32);
    const uint32_t r = 11u - clz32(yh);
    ok = ok && (r <= 10u);
    const uint32_t unit = fshl(0u, 1u, r);  // 2^r (r <= 10)
    const uint64_t t = y + (unit >> 1);
    return t & ~(uint64_t)(unit - 1u);
}

// ---- products ------------------------------------------------------------
// floor(x * c / 2^64) - e with e in {0, 1}, for x < 2^63:
//   x c / 2^64 = xh ch + (xh cl + xl ch) / 2^32 + xl cl / 2^64
// with the two middle products summed without overflow (m1 < 2^63 because
// xh < 2^31; m2 <= (2^32 - 1)^2 + 2^32 - 1 < 2^64) and xl cl dropped.
IMEX_HD uint64_t mulhi(uint64_t x, uint64_t c)
{
    const uint32_t xl = (uint32_t)x, xh = (uint32_t)(x >> 32);
    const uint32_t cl = (uint32_t)c, ch = (uint32_t)(c >> 32);
    const uint64_t m1 = (uint64_t)xh * cl;
    const uint64_t m2 = (uint64_t)xl * ch + (uint32_t)m1;
    return (uint64_t)xh * ch + (m1 >> 32) + (m2 >> 32);
}

// Quadratic terms in units of 2^-61 for |V| = v < 2^60.  With v = h 2^32 + l:
//   4.5 v^2 / 2^61 = 36 h^2 + 9 h l / 2^29 + 4.5 l^2 / 2^61
//   1.5 v^2 / 2^61 = 12 h^2 + 3 h l / 2^29 + 1.5 l^2 / 2^61
// The l^2 terms are dropped; on average they cancel between the 4.5 (e.u)^2
// and 1.5 u.u terms that B combines.
IMEX_HD uint64_t quad45(uint64_t v)
{
    const uint32_t l = (uint32_t)v, h = (uint32_t)(v >> 32);
    const uint32_t a = 9u * h;
    return (uint64_t)a * (4u * h) + (((uint64_t)a * l) >> 29);
}

IMEX_HD uint64_t quad15(uint64_t v)
{
    const uint32_t l = (uint32_t)v, h = (uint32_t)(v >> 32);
    const uint32_t a = 3u * h;
    return (uint64_t)a * (4u * h) + (((uint64_t)a * l) >> 29);
}

IMEX_HD uint64_t absval(int64_t v, uint64_t& signmask)
{
    signmask = (uint64_t)(v >> 63);
    return ((uint64_t)v ^ signmask) - signmask;
}

// Weight class of direction a: 0 rest, 1 axis, 2 face diagonal, 3 corner.
IMEX_HD constexpr int wclass(int a)
{
    return weight216(a) == 64 ? 0 : weight216(a) == 16 ? 1 : weight216(a) == 4 ? 2 : 3;
}

// ---- one cell ------------------------------------------------------------
// BGK collision of the 27 values in `in` (reference direction order) into
// out.  OM_GE1: omega >= 1, so (1 - omega) f is subtracted.  IN_FX / OUT_FX:
// the values are held as X on the float64 grid (round_fixed), otherwise as
// float64 bit patterns; both hold the same numbers, so the four encodings
// give the same results.  Clears ok when the cell leaves the exact range
// (out is then meaningless).
template <bool OM_GE1, bool IN_FX, bool OUT_FX>
IMEX_HD void collide_cell_io(const uint64_t (&in)[kQ], uint64_t (&out)[kQ], const FxConst& c, bool& ok)
{
    uint64_t X[kQ];
#pragma unroll
    for (int a = 0; a < kQ; ++a)
        X[a] = IN_FX ? check_fixed(in[a], a == 0 ? 8u : 5u, ok) : to_fixed_bits(in[a], a == 0 ? 8u : 5u, ok);

    // Exact moments.  G[x][y] sums the z-members of each (ex, ey) column;
    // every unsigned sum stays below 2^64 in the exact range.
    uint64_t G[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
    for (int a = 0; a < kQ; ++a) G[ex(a, 0) + 1][ex(a, 1) + 1] += X[a];
    const uint64_t sxm = G[0][0] + G[0][1] + G[0][2];
    const uint64_t sx0 = G[1][0] + G[1][1] + G[1][2];
    const uint64_t sxp = G[2][0] + G[2][1] + G[2][2];
    const uint64_t sym = G[0][0] + G[1][0] + G[2][0];
    const uint64_t syp = G[0][2] + G[1][2] + G[2][2];
    uint64_t zp = 0, zm = 0;
#pragma unroll
    for (int a = 0; a < kQ; ++a) {
        if (ex(a, 2) == 1) zp += X[a];
        if (ex(a, 2) == -1) zm += X[a];
    }
    const uint64_t S = sxm + sx0 + sxp;  // 3p * 2^61
    const int64_t U[3] = {(int64_t)(sxp - sxm), (int64_t)(syp - sym), (int64_t)(zp - zm)};
    ok = ok && (S >> 62) == 0;

    uint64_t P15 = 0;  // 1.5 u.u
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        uint64_t m;
        P15 += quad15(absval(U[d], m));
    }
    const int64_t base = (int64_t)(S - P15);  // 3p - 1.5 u.u
    ok = ok && base >= 0;

    uint64_t o[kQ];
    {
        const uint64_t T = mulhi((uint64_t)base, c.c_ow[0]);
        const uint64_t M = mulhi(X[0], c.c_om1);
        o[0] = OM_GE1 ? T - M : T + M;
    }
#pragma unroll
    for (int kk = 1; kk <= kPairs; ++kk) {
        const int a = 2 * kk - 1;
        const int cls = wclass(a);
        int64_t V = 0;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (ex(a, d) == 1) V += U[d];
            if (ex(a, d) == -1) V -= U[d];
        }
        uint64_t m;
        const uint64_t av = absval(V, m);
        ok = ok && (av >> 60) == 0;
        const uint64_t B = (uint64_t)base + quad45(av);
        const uint64_t T = mulhi(B, c.c_ow[cls]);
        const uint64_t R = (mulhi(av, c.c_3ow[cls]) ^ m) - m;  // sign of V restored
        const uint64_t M1 = mulhi(X[a], c.c_om1);
        const uint64_t M2 = mulhi(X[a + 1], c.c_om1);
        o[a] = OM_GE1 ? T + R - M1 : T + R + M1;
        o[a + 1] = OM_GE1 ? T - R - M2 : T - R + M2;
    }
#pragma unroll
    for (int a = 0; a < kQ; ++a) out[a] = OUT_FX ? round_fixed(o[a], ok) : bits_of(from_fixed(o[a], ok));
}

template <bool OM_GE1>
IMEX_HD void collide_cell(const double (&f)[kQ], double (&out)[kQ], const FxConst& c, bool& ok)
{
    uint64_t in[kQ], o[kQ];
#pragma unroll
    for (int a = 0; a < kQ; ++a) in[a] = bits_of(f[a]);
    collide_cell_io<OM_GE1, false, false>(in, o, c, ok);
#pragma unroll
    for (int a = 0; a < kQ; ++a) out[a] = double_of((uint32_t)(o[a] >> 32), (uint32_t)o[a]);
}

}  // namespace fx
}  // namespace imex
