"""The fixed-point float64 arithmetic (csrc/fx_math.cuh) compiled for the
host: its four value encodings agree bit for bit.

A run of fused steps holds the state as X = f 2^61 on the float64 grid
between launches (round_fixed) instead of as float64; the step's results
must be the same numbers either way.  The header's host branches are
portable restatements of the device intrinsics, so the check runs here on
random values and random near-equilibrium cells."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "imexlbm_gb300", "csrc")

HARNESS = r"""
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <cmath>
#include <random>
#include "fx_math.cuh"
#include "fx_params.hpp"
using namespace imex;

static double dbl(uint64_t b) { double v; std::memcpy(&v, &b, 8); return v; }

template <bool OM>
static long check_cells(const FxConst& c, std::mt19937_64& rng, int ncells, long* ran)
{
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    long bad = 0;
    for (int t = 0; t < ncells; ++t) {
        const double u[3] = {0.08 * U(rng), 0.08 * U(rng), 0.08 * U(rng)};
        const double p = 1.0 / 3.0 + 1e-3 * U(rng);
        uint64_t fb[kQ], X[kQ];
        bool ok = true;
        for (int a = 0; a < kQ; ++a) {
            const double edu = ex(a, 0) * u[0] + ex(a, 1) * u[1] + ex(a, 2) * u[2];
            const double udu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
            double f = weight216(a) / 216.0 * (3 * p + 3 * edu + 4.5 * edu * edu - 1.5 * udu);
            f *= 1.0 + 1e-3 * U(rng);
            fb[a] = fx::bits_of(f);
            X[a] = fx::to_fixed(f, a == 0 ? 8u : 5u, ok);
        }
        if (!ok) continue;
        uint64_t o_ff[kQ], o_fx[kQ], o_xf[kQ], o_xx[kQ];
        bool k1 = true, k2 = true, k3 = true, k4 = true;
        fx::collide_cell_io<OM, false, false>(fb, o_ff, c, k1);
        fx::collide_cell_io<OM, false, true>(fb, o_fx, c, k2);
        fx::collide_cell_io<OM, true, false>(X, o_xf, c, k3);
        fx::collide_cell_io<OM, true, true>(X, o_xx, c, k4);
        if (!(k1 && k2 && k3 && k4)) { ++bad; continue; }
        ++*ran;
        for (int a = 0; a < kQ; ++a) {
            bool okc = true;
            const uint64_t back = fx::to_fixed_bits(o_ff[a], 10u, okc);
            if (o_xf[a] != o_ff[a] || o_fx[a] != back || o_xx[a] != back || !okc) { ++bad; break; }
        }
    }
    return bad;
}

int main()
{
    std::mt19937_64 rng(20261203);
    long bad = 0, n = 0;
    // round_fixed(y) == to_fixed(from_fixed(y)) on random y and at the
    // rounding boundaries
    for (int t = 0; t < 2000000; ++t) {
        const int e = 52 + (int)(rng() % 11);
        uint64_t y = (rng() >> (63 - e)) | (1ull << e);
        if (t % 4 == 1) y = (y >> 10 << 10) | 0x1ff;   // just below a half
        if (t % 4 == 2) y = (y >> 10 << 10) | 0x200;   // a tie
        if (t % 4 == 3) y = (1ull << e) - 1 + (1ull << 52);
        bool a = true, b = true, c = true;
        const double d = fx::from_fixed(y, a);
        const uint64_t want = fx::to_fixed(d, 10u, b);
        const uint64_t got = fx::round_fixed(y, c);
        if (a != c || (a && (!b || want != got))) ++bad;
        ++n;
    }
    std::printf("values %ld bad %ld\n", n, bad);
    long ran = 0, badc = 0;
    FxParams fp;
    for (double tau : {0.003, 0.02, 0.4, 0.9}) {
        if (!make_fx_params(tau, 1.0, &fp)) { std::printf("params failed\n"); return 2; }
        badc += fp.om_ge1 ? check_cells<true>(fp.k, rng, 20000, &ran) : check_cells<false>(fp.k, rng, 20000, &ran);
    }
    std::printf("cells %ld bad %ld\n", ran, badc);
    return (bad || badc || ran < 60000) ? 1 : 0;
}
"""


def test_fixed_point_encodings_agree(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "fx_host.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "fx_host"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC, "-I", os.path.join(ROOT, "include"),
                    str(src), os.path.join(CSRC, "fx_params.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
