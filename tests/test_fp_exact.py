"""mul_float_by_double (lighthouse2_gb300/csrc/fp_exact.h) against real double arithmetic.

The SVGF kernels use it in place of the reference's float * double-literal product (an FP64 instruction on the
GPU). The host instantiation of the same source is compiled here with g++ and compared bit for bit with
(float)((double)w * 0.0001) over every float class: zero, denormals (where the float result rounds at the fixed
2^-149 quantum or underflows to zero), normals across the whole exponent range, the largest finite value,
infinity, and dense random samples; and against other double constants."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r'''
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <cmath>
#include "fp_exact.h"
using namespace lh2g;
static uint32_t bitsof(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static float fromb(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint64_t st = 0x9E3779B97F4A7C15ull;
static uint64_t rnd() { st ^= st << 13; st ^= st >> 7; st ^= st << 17; return st; }
int main() {
    long long bad = 0, n = 0;
    struct C { double c; } consts[] = {{0.0001}, {0.1}, {1.0 / 3.0}, {3.14159265358979}, {1e-30}, {7.5e20}};
    for (const C& cc : consts) {
        int ex;
        const double fr = frexp(cc.c, &ex);                 /* c = fr * 2^ex, fr in [0.5, 1) */
        const uint64_t mc = (uint64_t)ldexp(fr, 53);
        const int ec = ex - 53;
        auto check = [&](uint32_t b) {
            const float w = fromb(b);
            const float want = (float)((double)w * cc.c);
            const float got = mul_float_by_double(w, mc, ec);
            n++;
            if (bitsof(want) != bitsof(got)) {
                if (bad < 10) printf("c=%.17g w=%08x want %08x got %08x\n", cc.c, b, bitsof(want), bitsof(got));
                bad++;
            }
        };
        for (uint32_t b = 0; b < 0x00100000u; b++) check(b);                    /* zero and small denormals */
        for (uint32_t b = 0x007f0000u; b < 0x00900000u; b++) check(b);          /* the denormal / normal boundary */
        for (uint32_t b = 0x7f700000u; b <= 0x7f800000u; b++) check(b);         /* the largest values and +inf */
        for (uint32_t e = 0; e < 255; e++)
            for (int k = 0; k < 4096; k++) check((e << 23) | (uint32_t)(rnd() & 0x7fffffu));
        for (int k = 0; k < 2000000; k++) check((uint32_t)(rnd() % 0x7f800001u));
    }
    /* the constant the filter uses, as stored */
    if (mul_float_by_double(1.0f, DBL_1EM4_MANT, DBL_1EM4_EXP) != (float)(1.0 * 0.0001)) bad++;
    printf("%lld of %lld differ\n", bad, n);
    return bad != 0;
}
'''


def test_mul_float_by_double_matches_fp64(tmp_path):
    src = tmp_path / "probe.cpp"
    src.write_text(PROBE)
    exe = tmp_path / "probe"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "lighthouse2_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
