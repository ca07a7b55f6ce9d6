"""Integer recombination arithmetic of the split-precision GEMM epilogue
(csrc/dcg_fixed.cuh), compiled for the host with g++ and checked against exact rational
arithmetic: FP32 values to 2^-28 fixed point (exact on multiples of 2^-28, nearest with
halves away from zero otherwise) and 64-bit integers times a power of two to correctly
rounded doubles."""
import os
import random
import struct
import subprocess
from fractions import Fraction

import pytest

from conftest import ROOT

DRIVER = r"""
#include <cstdio>
#include <cinttypes>
#include <cstring>
#include "dcg_fixed.cuh"
int main() {
    char op[8];
    while (std::scanf("%7s", op) == 1) {
        if (op[0] == 'f') {
            unsigned b;
            std::scanf("%u", &b);
            std::printf("%" PRId64 "\n", dcg::fx28_from_float_bits(b));
        } else {
            long long x;
            int s;
            std::scanf("%lld %d", &x, &s);
            double d = dcg::fx_to_double((int64_t)x, s);
            unsigned long long u;
            std::memcpy(&u, &d, 8);
            std::printf("%llu\n", u);
        }
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    d = tmp_path_factory.mktemp("fx")
    (d / "drv.cpp").write_text(DRIVER)
    exe = d / "drv"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "dirac_caspt2_gb300", "csrc"),
                        str(d / "drv.cpp"), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(exe)


def _run(exe, lines):
    out = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True).stdout
    return [int(x) for x in out.split()]


def _round_half_away(q: Fraction) -> int:
    n = abs(q)
    r = int(n + Fraction(1, 2)) if n.denominator != 1 else int(n)
    return r if q >= 0 else -r


def _f32(x: float) -> int:
    return struct.unpack("<I", struct.pack("<f", x))[0]


def test_fx28_from_float(driver):
    rng = random.Random(7)
    vals = [0.0, -0.0, 1.0, -1.0, 2.0 ** -28, -(2.0 ** -28), 3 * 2.0 ** -29, 2.0 ** -29, 2.0 ** -30,
            1e-40, 2.0 ** 24 - 1, -(2.0 ** 25), 16777215.0 * 2.0 ** -14]
    for _ in range(3000):
        e = rng.randint(-40, 33)
        vals.append(rng.choice([-1, 1]) * rng.randint(1, 2 ** 24 - 1) * 2.0 ** (e - 24))
    bits = [_f32(v) for v in vals]
    got = _run(driver, [f"f {b}" for b in bits])
    for b, g in zip(bits, got):
        f = struct.unpack("<f", struct.pack("<I", b))[0]
        assert g == _round_half_away(Fraction(f) * 2 ** 28), (f, g)


def test_fx_to_double(driver):
    rng = random.Random(11)
    cases = [(1, 0), (-1, 0), (2 ** 53 + 1, 0), (2 ** 53 + 3, 0), (2 ** 62 - 1, -10), (-(2 ** 61) - 5, 7),
             (3, -1074 + 60), (12345, 900)]
    for _ in range(4000):
        x = rng.choice([-1, 1]) * rng.randint(1, 2 ** rng.randint(1, 62) - 1)
        cases.append((x, rng.randint(-300, 300)))
    got = _run(driver, [f"d {x} {s}" for x, s in cases])
    for (x, s), g in zip(cases, got):
        want = float(Fraction(x) * (Fraction(2) ** s))
        assert struct.unpack("<d", struct.pack("<Q", g))[0] == want, (x, s)
    assert _run(driver, ["d 0 5"]) == [0]
