"""CPU unit test of the compensated-pair -> FP64 rounding used by the kernels' write-out
(ferrite.jl_gb300/csrc/dfloat.h): the exact path and the kernels' branch-free forms (with their
flagged sums redone exactly) are bitwise equal to the correctly rounded double sum, for low
words smaller and larger than the high word."""
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r'''
#include "dfloat.h"
#include <cstdio>
#include <cmath>
#include <random>
#include <cstring>
#include <utility>
int main() {
    std::mt19937_64 g(12345);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    long bad = 0, n = 0, nrare = 0;
    for (int it = 0; it < 2000000; ++it) {
        const int ex = (int)(g() % 120) - 60;
        float hi = (float)std::ldexp(U(g), ex);
        if (it % 7 == 0) hi = std::ldexp(1.0f, ex) * ((it & 8) ? -1.f : 1.f);  // powers of two
        const int k = (int)(g() % 40);
        float lo = (float)std::ldexp(U(g), ex - 24 - k);
        if (it % 11 == 0) lo = 0.0f;
        if (it % 13 == 0) lo = std::ldexp(std::nextafter(std::ldexp(hi, 0), 2 * hi) - hi, -1);  // exact half ulp
        if (it % 17 == 0) std::swap(hi, lo);  // low word larger than the high word (cancellation)
        const double want = (double)hi + (double)lo;
        const double got = fe::pair_to_double(hi, lo);
        // the kernels' branch-free forms, with the flagged sums redone exactly
        bool rare1 = false, rare2 = false;
        double got1 = fe::pair1_to_double(hi, lo, rare1);
        if (rare1) got1 = fe::pair_to_double(hi, lo);
        double got2, other;
        fe::pair2_to_double(fe::float2{hi, 1.5f}, fe::float2{lo, 0.0f}, got2, other, rare2);
        if (rare2) got2 = fe::pair_to_double(hi, lo);
        uint64_t a, b, c1, c2;
        std::memcpy(&a, &want, 8);
        std::memcpy(&b, &got, 8);
        std::memcpy(&c1, &got1, 8);
        std::memcpy(&c2, &got2, 8);
        ++n;
        nrare += rare1;
        if (a != b || a != c1 || a != c2 || rare1 != rare2 || other != 1.5) {
            if (bad < 5) std::printf("hi=%a lo=%a want=%a got=%a p1=%a p2=%a\n", hi, lo, want, got, got1, got2);
            ++bad;
        }
    }
    for (int it = 0; it < 1000000; ++it) {
        const float v = (float)std::ldexp(U(g), (int)(g() % 200) - 100);
        const double w = (double)v, z = fe::float_to_double(v);
        if (std::memcmp(&w, &z, 8) != 0) { ++bad; if (bad < 5) std::printf("f2d %a\n", v); }
    }
    // every exponent field (zero, subnormal, normal, inf, quiet NaN) with random mantissas
    for (uint32_t e = 0; e < 256; ++e)
        for (int k = 0; k < 4000; ++k) {
            uint32_t m = (uint32_t)(g() & 0x7FFFFF);
            if (k == 0) m = 0;
            if (e == 255 && m) m |= 0x400000;  // quiet NaNs (the integer path keeps payloads exactly)
            const uint32_t bits = ((uint32_t)(g() & 1) << 31) | (e << 23) | m;
            float v;
            std::memcpy(&v, &bits, 4);
            const double w = (double)v, z = fe::float_to_double(v);
            if (std::memcmp(&w, &z, 8) != 0) { ++bad; if (bad < 10) std::printf("f2d bits %08x\n", bits); }
        }
    std::printf("%ld %ld %ld\n", bad, n, nrare);
    if (nrare > n / 4) { std::printf("too many flagged sums\n"); return 1; }
    return bad != 0;
}
'''


def test_pair_to_double_bitwise():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.cpp")
        exe = os.path.join(d, "t")
        open(src, "w").write(SRC)
        subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "ferrite.jl_gb300", "csrc"), src, "-o", exe],
                       check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
