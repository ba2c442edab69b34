"""cmfeed::angle32, the FP32 search's draw of an Euler angle (csrc/cm_feed.h),
against cmfeed::angle, the FP64 draw that the oracle restates
(src/rigid_body.jl:122-125): compiled for the host with g++.

* The same stream: after every draw both leave the generator in the same
  state (the same rejections of points outside the unit disk).
* cos and sin within 3.01 u (u = 2^-24) of the FP64 values, the bound the
  guard band of the FP32 placement is built on.
* Points on the unit circle's edge, where the integer test hands over to
  the FP64 test: the same accept / reject as the FP64 test.
* u128_to_f32 is the correctly rounded FP32 value (ties to even) of a
  128-bit integer, checked against exact rational rounding.
"""
import os
import shutil
import struct
import subprocess
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FEED = os.path.join(ROOT, "complexmixtures.jl_gb300", "csrc", "cm_feed.h")

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include "cm_feed.h"
using namespace cmfeed;
int main(int argc, char **argv) {
    if (argc > 1 && !strcmp(argv[1], "u128")) {
        unsigned long long hi, lo;
        while (scanf("%llu %llu", &hi, &lo) == 2) {
            const float f = u128_to_f32(hi, lo);
            uint32_t b;
            memcpy(&b, &f, 4);
            printf("%u\n", b);
        }
        return 0;
    }
    const long n = atol(argv[1]);
    double wc = 0, ws = 0;
    long mism = 0;
    for (long i = 0; i < n; ++i) {
        uint64_t s0 = key(20261204, kTagSlot, (uint64_t)i, (uint64_t)i * 7, (uint64_t)i * 13), s1 = s0;
        double c64, s64;
        float c32, s32;
        angle(s0, c64, s64);
        angle32(s1, c32, s32);
        if (s0 != s1) { ++mism; continue; }
        wc = fmax(wc, fabs((double)c32 - c64));
        ws = fmax(ws, fabs((double)s32 - s64));
    }
    long bad = 0, tested = 0;
    for (long i = 0; i < n / 10; ++i) {
        uint64_t st = key(91, 9, (uint64_t)i, 0, 0);
        const int64_t a = ((int64_t)(next(st) >> 11) - (int64_t(1) << 52)) * 2;
        const long double rem = ldexpl(1.0L, 106) - (long double)a * (long double)a;
        const int64_t b0 = (int64_t)floorl(sqrtl(rem));
        for (int d = -3; d <= 3; ++d) {
            const int64_t b = b0 + d;
            if (b > (int64_t(1) << 53)) continue;
            uint64_t sq[4];
            const double u = (double)a * 0x1.0p-53, v = (double)b * 0x1.0p-53;
            const double r2 = add(mul(u, u), mul(v, v));
            ++tested;
            if (disk_accept(a, b, sq) != (r2 > 0.0 && r2 < 1.0)) ++bad;
        }
    }
    printf("%ld %.6f %.6f %ld %ld\n", mism, wc / 0x1.0p-24, ws / 0x1.0p-24, tested, bad);
    return 0;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("angle32")
    shutil.copy(FEED, d / "cm_feed.h")
    (d / "h.cpp").write_text(HARNESS)
    exe = d / "h"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", str(exe), str(d / "h.cpp")], check=True)
    return str(exe)


def test_angle32_follows_the_fp64_stream_within_the_bound(harness):
    out = subprocess.run([harness, "400000"], capture_output=True, text=True, check=True).stdout.split()
    mism, wc, ws, tested, bad = int(out[0]), float(out[1]), float(out[2]), int(out[3]), int(out[4])
    assert mism == 0
    assert wc <= 3.01 and ws <= 3.01
    assert tested > 200000 and bad == 0


def test_u128_to_f32_rounds_to_nearest_even(harness):
    rng = np.random.default_rng(12)
    vals = [0, 1, (1 << 24) + 1, (1 << 25) + 3, (1 << 107), (1 << 127) - 1]
    for _ in range(20000):
        bits = int(rng.integers(1, 127))
        x = int.from_bytes(rng.bytes(16), "little") >> (128 - bits)
        if x.bit_length() > 25 and rng.random() < 0.4:
            # a tie or a near-tie at the 24-bit rounding position
            sh = x.bit_length() - 24
            x = (x >> sh << sh) | (1 << (sh - 1)) | int(rng.integers(0, 2))
        vals.append(x)
    inp = "\n".join(f"{x >> 64} {x & ((1 << 64) - 1)}" for x in vals)
    out = subprocess.run([harness, "u128"], input=inp, capture_output=True, text=True, check=True).stdout.split()
    assert len(out) == len(vals)
    for x, o in zip(vals, out):
        got = struct.unpack("<f", struct.pack("<I", int(o)))[0]
        if x == 0:
            assert got == 0.0
            continue
        e = x.bit_length() - 1
        m = round(Fraction(x, 1 << (e - 23))) if e >= 23 else x << (23 - e)
        want = m * 2.0 ** (e - 23)
        assert got == want, x
