"""The bit-level helpers of csrc/bitsplit.h return what the FP64 expressions
they replace return (decide_num_to_spawn's split, threshold tests on |C|,
the Bernoulli threshold floor(p 2^64) and the compares of the death step),
for random signs over many magnitudes and for the edge cases: integers,
values just above and below integers and 1e-12, signed zeros, tiny and
subnormal values, and the 2^31 limit."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>
#include "bitsplit.h"
using namespace neci;

static unsigned long long prob_thresh(double p) {
    if (!(p > 0.0)) return 0ull;
    if (p >= 1.0) return ~0ull;
    return (unsigned long long)(p * 18446744073709551616.0);
}
static int check(double c) {
    // the FP64 form (fcimc_helper.F90:2160-2174 with AvMCExcits = 1)
    const double pa = c * 1.0;
    const int ns = std::abs((int)pa);
    const bool extra = std::fabs(std::fabs(pa) - (double)ns) > 1e-12;
    const unsigned long long thr = extra ? prob_thresh(std::fabs(pa) - (double)ns) : 0ull;
    uint32_t w; bool e; uint64_t t;
    if (!split_count(c, w, e, t)) return std::fabs(c) >= 2147483648.0 ? 0 : 1;
    if (std::fabs(c) >= 2147483648.0) return 1;
    if (w != (uint32_t)ns || e != extra || (extra && t != thr)) return 1;
    // threshold tests on |c|
    const double ys[] = {1e-12, 3.0, 1.0, 0.95, 0.5, 1e-300, 0.0};
    for (double y : ys) if ((std::fabs(c) > y) != (abs_bits(c) > dbl_bits(y))) return 1;
    if ((std::fabs(c) >= 1e-12) != (abs_bits(c) >= dbl_bits(1e-12))) return 1;
    if ((c < 0.0) != is_negative(c)) return 1;
    if ((c > 0.0) != is_positive(c)) return 1;
    const double bs[] = {1.0, -1.0, -2.3283064365386963e-10, 5e-300, -5e-300, 0.0, -0.0, -4.9e-324, 1e300, -7.5};
    for (double b : bs) if ((c * b < 0.0) != prod_negative(c, b)) return 1;
    // Bernoulli thresholds (bern) and the compares of the death step
    for (double pp : {c, std::fabs(c), std::fabs(c) - std::floor(std::fabs(c)), 1.0 - std::fabs(c), c * 1e-3,
                      std::fabs(c) * 0.5})
        if (prob_thresh_bits(pp) != prob_thresh(pp)) return 1;
    for (double b : {std::fabs(c), 0.0, 1.0, 0.5, 3.0, 1e-300})
        for (double a : {c, -c, c * 0.999, c * 1.001, 0.0, -0.0})
            if ((a <= b) != le_nonneg(a, b)) return 1;
    for (double y : {2.0, 1.0, 1e-12})
        if ((c > y) != gt_pos(c, y)) return 1;
    // the spawn amplitude's fixed point: llrint(c 2^32) and its overflow rule
    for (double x : {c, c * 2.3283064365386963e-10, c * 1e-9, c * 3.0e9}) {
        const double sc = x * 4294967296.0;
        const bool ovf = !(std::fabs(sc) < 9.2e18);
        int64_t q = 12345;
        const bool ok = fixed32_from_double(x, q);
        if (ok == ovf) return 1;
        if (ok && q != (int64_t)std::llrint(sc)) return 1;
    }
    return 0;
}
int main() {
    std::vector<double> v = {0.0, -0.0, 1e-12, -1e-12, std::nextafter(1e-12, 1.0), std::nextafter(1e-12, 0.0),
                             4.9e-324, 2.2e-308, 1.0, -1.0, 2.0, 3.0, 0.5, 0.95, 2147483647.0, 2147483647.5,
                             2147483648.0, -2147483648.0, 1e9, 1e15, 1e300};
    // (NaN and infinities are appended below for the fixed point only)
    for (int k = 1; k < 40; ++k) {
        const double b = (double)k;
        v.push_back(b + 1e-12); v.push_back(b + 2e-12); v.push_back(b - 1e-13);
        v.push_back(std::nextafter(b, 0.0)); v.push_back(std::nextafter(b, 1e9));
        v.push_back(-(b + 1e-12)); v.push_back(b + 0.5);
    }
    // ties of the fixed point's rounding: x 2^32 = k + 1/2
    for (int k = -40; k < 40; ++k) v.push_back(((double)k + 0.5) * 2.3283064365386963e-10);
    v.push_back(std::nan("")); v.push_back(INFINITY); v.push_back(-INFINITY);
    v.push_back(2142047537.0); v.push_back(-2142047538.5); v.push_back(4294967296.0);
    std::mt19937_64 g(7);
    std::uniform_real_distribution<double> u(-36.0, 10.0);
    for (int i = 0; i < 2000000; ++i) {
        const double mag = std::pow(10.0, u(g));
        v.push_back((g() & 1) ? mag : -mag);
        v.push_back((double)(long long)(g() % 1000) * 0.015625 * ((g() & 1) ? 1 : -1));
    }
    int bad = 0;
    for (double c : v) {
        if (!std::isfinite(c)) {
            int64_t q;
            if (fixed32_from_double(c, q)) ++bad;
            if (prob_thresh_bits(c) != prob_thresh(c) || prob_thresh_bits(-c) != prob_thresh(-c)) ++bad;
            continue;
        }
        const int b = check(c);
        if (b && bad < 5) std::printf("mismatch at %.17g\n", c);
        bad += b;
    }
    std::printf("%d\n", bad);
    return bad != 0;
}
"""


def test_bitsplit_matches_fp64_expressions(tmp_path):
    src = tmp_path / "h.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "h"
    r = subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", f"-I{ROOT / 'neci_stable_gb300' / 'csrc'}",
                        str(src), "-o", str(exe)], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
