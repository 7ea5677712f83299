"""The arclength's division and square root (div_fast, sqrt_fast in
csrc/sevc_device.cuh), compiled for the host from the device header's own
source and compared bit for bit with the native binary64 operations.

Those routines refine a binary32 seed to a float-float approximation, then
correct and certify the result on 64-bit integer significands (128-bit
remainders): a certified result must be the correctly rounded one, and an
uncertified candidate falls back to the native operation.  On the host the
two seed instructions (rcp.approx, rsqrt.approx) become the correctly
rounded binary32 reciprocal and reciprocal square root, and the CUDA integer
intrinsics their exact host equivalents; the seeds only bound how often the
fallback runs, so the check of every certified result is the same one the
device makes.  The GPU test of sevc_selftest_arith runs the same comparison
on the device.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "se-grain-growth-gpu_gb300", "csrc", "sevc_device.cuh")
START = "/* binary32 -> binary64 by bit manipulation"
END = "/* vector2_mag (src/geometry.h:217)"

SHIM = r"""
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#define __device__
#define __forceinline__ inline
static inline long long dbits(double x) { long long b; std::memcpy(&b, &x, 8); return b; }
static inline double __longlong_as_double(long long b) { double x; std::memcpy(&x, &b, 8); return x; }
static inline unsigned __float_as_uint(float x) { unsigned u; std::memcpy(&u, &x, 4); return u; }
static inline float __uint_as_float(unsigned u) { float x; std::memcpy(&x, &u, 4); return x; }
static inline float __uint2float_rn(unsigned u) { return (float)u; }
static inline float __int2float_rn(int u) { return (float)u; }
static inline int __float2int_rn(float x) { return (int)std::lrintf(x); }
static inline unsigned long long __umul64hi(unsigned long long a, unsigned long long b)
{
    return (unsigned long long)(((unsigned __int128)a * b) >> 64);
}
"""

HARNESS = r"""
static unsigned long long mix64(unsigned long long z)
{
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static double unit_pow2(unsigned long long u, int k)
{
    return __longlong_as_double((long long)((u & 0x000FFFFFFFFFFFFFULL) | ((unsigned long long)(1023 + k) << 52)));
}
int main(int argc, char **argv)
{
    long long n = atoll(argv[1]);
    unsigned long long seed = strtoull(argv[2], 0, 10);
    long long c[6] = {0, 0, 0, 0, 0, 0}, plain_uncert = 0;
    for (long long i = 0; i < n; i++) {
        unsigned long long a = mix64(seed ^ (2 * i)), b = mix64(seed ^ (2 * i + 1)), kind = (a >> 60) & 7;
        /* q / p, 0 <= q <= p: general ratios, quotients next to a rounding
         * midpoint (and one ulp either side), q = p, q = 0, subnormal q */
        int kp = (int)((b >> 56) % 121) - 60;
        double p = unit_pow2(b, kp), q;
        if (kind < 4) {
            q = p * unit_pow2(a, -1 - (int)((a >> 52) & 7));
        } else if (kind < 7) {
            double kd = __longlong_as_double((long long)((a & 0x000FFFFFFFFFFFFFULL) | (1022ULL << 52)));
            q = std::fma(p, kd, p * 0x1p-54);
            if (kind == 6) q = __longlong_as_double(dbits(q) + (((a >> 59) & 1) ? 1 : -1));
            if (dbits(q) > dbits(p)) q = p;
        } else {
            int w = (int)((a >> 40) & 3);
            q = w == 0 ? p : (w == 1 ? 0.0 : p * 0x1p-1040);
        }
        double r;
        c[0]++;
        if (div_fast(q, p, r)) { if (dbits(r) != dbits(q / p)) c[1]++; }
        else { c[2]++; if (kind < 7) plain_uncert++; }
        /* sqrt(t), t in [1, 2): general, next to the square of a midpoint */
        double t;
        if (kind < 4) {
            t = unit_pow2(a, 0);
        } else {
            double s = unit_pow2(a, 0);
            if (s > 1.4142135623730950) s = s - 0.4142135623730950;
            t = std::fma(s, s, s * 0x1p-52);
            if (kind == 6) t = __longlong_as_double(dbits(t) + (((a >> 59) & 1) ? 1 : -1));
            if ((dbits(t) >> 52) != 1023) t = 1.5;
        }
        c[3]++;
        if (sqrt_fast(t, r)) { if (dbits(r) != dbits(std::sqrt(t))) c[4]++; }
        else c[5]++;
    }
    /* edges: t = 1 and the largest t below 2, q = p at extreme exponents */
    double edges_t[] = {1.0, 0x1.fffffffffffffp0, 0x1.0000000000001p0};
    for (double t : edges_t) { double r; if (sqrt_fast(t, r) && dbits(r) != dbits(std::sqrt(t))) c[4]++; }
    printf("%lld %lld %lld %lld %lld %lld %lld\n", c[0], c[1], c[2], c[3], c[4], c[5], plain_uncert);
    return 0;
}
"""


def _source():
    text = open(HEADER).read()
    i, j = text.index(START), text.index(END)
    block = text[i:j]
    # the two seed instructions, as host functions
    for name, expr in (("rcp_seed", "1.0f / x"), ("rsqrt_seed", "1.0f / std::sqrt(x)")):
        k = block.index("__device__ __forceinline__ float %s(float x)" % name)
        e = block.index("}\n", k) + 2
        block = block[:k] + "static inline float %s(float x) { return %s; }\n" % (name, expr) + block[e:]
    assert "asm(" not in block, "an inline-asm helper needs a host stand-in"
    return SHIM + block + HARNESS


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
@pytest.mark.parametrize("seed", [1, 20240611])
def test_integer_certified_division_and_sqrt_match_native(tmp_path, seed):
    src = tmp_path / "intcert.cpp"
    exe = tmp_path / "intcert"
    src.write_text(_source())
    subprocess.run(["g++", "-O2", "-std=c++17", "-o", str(exe), str(src)], check=True, capture_output=True)
    n = 1 << 21
    out = subprocess.run([str(exe), str(n), str(seed)], check=True, capture_output=True, text=True).stdout.split()
    div, div_bad, div_unc, sq, sq_bad, sq_unc, plain_unc = map(int, out)
    assert div == sq == n
    assert div_bad == 0 and sq_bad == 0, out
    # the fallback is for special operands (subnormal q), never for ordinary ones
    assert plain_unc == 0, out
    assert sq_unc == 0, out
    assert div_unc < n // 8, out
