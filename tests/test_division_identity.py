"""The Jacobi kernels divide by the stored reciprocal with one remainder correction:
q = RN(a y), q' = RN(q + RN_exact(a - b q) y) with y = RN(1/b) (Markstein, IBM J. Res. Dev.
34(1), 1990).  This checks on the CPU, in IEEE double with a correctly rounded fma (the
operations the kernels use), that q' equals the correctly rounded a / b on random operands,
on divisors with all-ones and near-zero mantissas and on a ~ b."""
import os
import shutil
import subprocess

import pytest

SRC = r"""
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
static uint64_t s = 0x243F6A8885A308D3ull;
static uint64_t next(void) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double make(uint64_t mant, int e) {
  uint64_t b = ((uint64_t)(1023 + e) << 52) | (mant & ((1ull << 52) - 1));
  double d;
  memcpy(&d, &b, 8);
  return d;
}
int main(int argc, char** argv) {
  long n = atol(argv[1]), bad = 0;
  for (long i = 0; i < n; ++i) {
    uint64_t ma = next(), mb = next();
    switch (i % 4) {
      case 1: mb |= ((1ull << 52) - 1) ^ (next() & 0xff); break;
      case 2: mb &= 0xff; break;
      case 3: ma = (ma & 0xffffffffull) | (mb & 0xfffff00000000ull); break;
    }
    volatile double a = make(ma, (int)(next() % 40) - 20), b = make(mb, (int)(next() % 12));
    double y = 1.0 / b;
    double q = a * y;
    double q1 = fma(fma(-q, b, a), y, q);
    if (q1 != a / b) ++bad;
  }
  printf("%ld\n", bad);
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_remainder_corrected_quotient_is_correctly_rounded(tmp_path):
    src = tmp_path / "q.c"
    src.write_text(SRC.replace("#include <string.h>", "#include <string.h>\n#include <stdlib.h>"))
    exe = tmp_path / "q"
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-o", str(exe), str(src), "-lm"], check=True)
    out = subprocess.run([str(exe), "20000000"], check=True, capture_output=True, text=True).stdout
    assert int(out.strip()) == 0
