"""The integer FP32 <-> FP64 conversions of schnellfmm_gb300/csrc/fp_convert.cuh,
compiled for the host (the CUDA bit-cast intrinsics replaced by memcpy) and
checked against the host's own conversions, which round to nearest even as
the GPU's do: the widening on every 7th FP32 bit pattern, the narrowing on
random doubles (a third of them in the FP32 exponent range, some exactly
half-way between two floats) and on the edges (zeros, the largest float and
the value that rounds up past it, the smallest normal and subnormals,
infinities, NaN)."""
import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parents[1] / "schnellfmm_gb300" / "csrc"

PROGRAM = r"""
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#define __device__
#define __forceinline__ inline
static inline uint32_t __float_as_uint(float x) { uint32_t u; std::memcpy(&u, &x, 4); return u; }
static inline float __uint_as_float(uint32_t u) { float x; std::memcpy(&x, &u, 4); return x; }
static inline long long __double_as_longlong(double x) { long long u; std::memcpy(&u, &x, 8); return u; }
static inline double __longlong_as_double(long long u) { double x; std::memcpy(&x, &u, 8); return x; }
#include "fp_convert.cuh"

static bool same32(float a, float b) {
    if (std::isnan(a) && std::isnan(b)) return true;
    return __float_as_uint(a) == __float_as_uint(b);
}
static bool same64(double a, double b) {
    if (std::isnan(a) && std::isnan(b)) return true;
    return __double_as_longlong(a) == __double_as_longlong(b);
}

int main() {
    unsigned long long bad = 0, n = 0;
    for (uint64_t i = 0; i < (1ull << 32); i += 7, ++n) {
        const float x = __uint_as_float((uint32_t)i);
        if (!same64(slfmm::f64_of_f32(x), (double)x)) ++bad;
    }
    std::mt19937_64 g(12345);
    for (int i = 0; i < 20000000; ++i, ++n) {
        uint64_t b = g();
        if (i % 3 == 0) {
            const int e = 1023 + (int)(g() % 300) - 150;
            b = (b & 0x800fffffffffffffull) | ((uint64_t)e << 52);
            if (i % 7 == 0) b = (b & ~0x1fffffffull) | 0x10000000ull;  // half-way
        }
        const double x = __longlong_as_double((long long)b);
        if (!same32(slfmm::f32_of_f64(x), (float)x)) ++bad;
    }
    const double edge[] = {0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38,
                           -3.4028235677973366e38, 1.1754943508222875e-38, 1.1754942e-38, 1e-45, 1e-300,
                           INFINITY, -INFINITY, NAN, 65504.0, 0.1, 1.0 / 3.0};
    for (double x : edge) {
        ++n;
        if (!same32(slfmm::f32_of_f64(x), (float)x)) ++bad;
        const float f = (float)x;
        if (!same64(slfmm::f64_of_f32(f), (double)f)) ++bad;
    }
    std::printf("%llu %llu\n", n, bad);
    return bad != 0;
}
"""


def test_fp_convert_matches_host_conversions(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "fp_convert_check.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "fp_convert_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(CSRC), str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    n, bad = map(int, r.stdout.split())
    assert n > 600_000_000 and bad == 0, r.stdout
