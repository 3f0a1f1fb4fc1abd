"""div_rn (saras_gb300/csrc/df64.cuh): x / d correctly rounded from y = RN(1/d) by
Markstein's correction step, q = RN(x y), r = x - q d (exact, FMA), RN(q + r y).
The reference-form smoother and Crank-Nicolson kernels divide by level or launch
constants this way instead of by a division, and must keep the division's bits
(the drop-in's parity is bit for bit).  The step is IEEE arithmetic, so the
host's FMA gives the device's results: a C++ program checks it against the
division on random pairs over many binades, divisors with all-ones and
power-of-two significands included."""
import os
import subprocess

import pytest

SRC = r"""
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
static double div_rn(double x, double d, double y) { double q = x * y; return std::fma(std::fma(-q, d, x), y, q); }
int main(int argc, char **argv) {
    long n = std::atol(argv[1]);
    std::mt19937_64 rng(20250101);
    long bad = 0, done = 0;
    for (long t = 0; done < n; ++t) {
        uint64_t db = rng();
        if (t % 10 == 0) db |= 0x000fffffffffffffULL;
        if (t % 10 == 1) db &= 0xfff0000000000000ULL;
        double d = std::ldexp(1.0 + (double)(db & 0x000fffffffffffffULL) * std::ldexp(1.0, -52), (int)(rng() % 200) - 100);
        if (t % 2) d = -d;
        double y = 1.0 / d;
        for (int k = 0; k < 1000; ++k, ++done) {
            uint64_t xb = rng();
            double x = std::ldexp(1.0 + (double)(xb & 0x000fffffffffffffULL) * std::ldexp(1.0, -52), (int)(rng() % 120) - 60);
            if (xb >> 63) x = -x;
            double a = x / d, b = div_rn(x, d, y);
            if (std::memcmp(&a, &b, 8)) ++bad;
        }
    }
    std::printf("%ld %ld\n", done, bad);
    return 0;
}
"""


def test_markstein_division_matches_ieee_division(tmp_path):
    src = tmp_path / "div.cc"
    src.write_text(SRC)
    exe = tmp_path / "div"
    r = subprocess.run(["g++", "-O2", "-ffp-contract=off", "-o", str(exe), str(src)], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("no C++ compiler: " + r.stderr[:200])
    out = subprocess.run([str(exe), "5000000"], capture_output=True, text=True, timeout=300)
    done, bad = map(int, out.stdout.split())
    assert done == 5000000
    assert bad == 0
