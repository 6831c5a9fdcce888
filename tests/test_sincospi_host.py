"""Accuracy of the lobe-mean sine/cosine (csrc/mixture.cuh: sincospi_poly
and sincospi_tab) and of the series of the mixture-only kernels' vMF
normaliser (bernoulli_gen).

The mixture kernels evaluate sin(pi t) and cos(pi t) of the logistic lobe
angles with their own functions instead of the hardware approximation: the
plain FP32 path with a folded polynomial, the mixture-only kernels from a
128-entry table of sin/cos(pi k/32) and short polynomials of the remainder.
An error e in a lobe mean becomes a relative pdf error of about e * kappa,
so both must stay within ~1e-7 of the exact value. The functions are
__host__ __device__, so this test compiles a small host program against the
header with nvcc and compares them with long-double sin/cos on a dense grid
of float arguments -- on the CPU, no GPU needed.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "neural-mixture-guiding_gb300", "csrc")

PROGRAM = r"""
#include <cmath>
#include <cstdio>
#include "mixture.cuh"

int main() {
  const long n = 2000000;
  const long double pi = 3.141592653589793238462643383279502884L;
  static const float2 tab[128] = NMG_SINCOSPI32_TABLE;
  double e2 = 0.0, e1 = 0.0, et = 0.0;
  for (long i = 0; i <= n; ++i) {
    // t over [0, 2] (the azimuth argument 2 sp) and over [0, 1] (theta's)
    const float t2 = float(2.0 * double(i) / double(n));
    const float t1 = float(double(i) / double(n));
    float s, c;
    nmg::sincospi_poly<true>(t2, &s, &c);
    long double x = (long double)t2 * pi;
    e2 = fmax(e2, double(fabsl((long double)s - sinl(x))));
    e2 = fmax(e2, double(fabsl((long double)c - cosl(x))));
    nmg::sincospi_tab(tab, t2, &s, &c);
    et = fmax(et, double(fabsl((long double)s - sinl(x))));
    et = fmax(et, double(fabsl((long double)c - cosl(x))));
    nmg::sincospi_poly<false>(t1, &s, &c);
    x = (long double)t1 * pi;
    e1 = fmax(e1, double(fabsl((long double)s - sinl(x))));
    e1 = fmax(e1, double(fabsl((long double)c - cosl(x))));
  }
  double ee = 0.0;  // the table entries themselves
  for (int k = 0; k < 128; ++k) {
    const long double x = pi * (long double)k / 32.0L;
    ee = fmax(ee, double(fabsl((long double)tab[k].x - sinl(x))));
    ee = fmax(ee, double(fabsl((long double)tab[k].y - cosl(x))));
  }
  printf("%.6e %.6e %.6e %.6e\n", e2, e1, et, ee);
  return 0;
}
"""


def test_sincospi_poly_and_table_within_1e7(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "sincospi.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "sincospi"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", CSRC, str(src), "-o", str(exe)], check=True,
                   capture_output=True, timeout=600)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=600).stdout.split()
    e_two, e_one, e_tab, e_entry = (float(v) for v in out[:4])
    # within 1e-7 of exact over [0, 2] and, without the [1, 2] fold, over [0, 1]
    assert e_two <= 1e-7, e_two
    assert e_one <= 1e-7, e_one
    # the table form over [0, 2] (its argument range: theta's t in [0, 1], phi's 2 t in [0, 2])
    assert e_tab <= 1e-7, e_tab
    # every entry rounded correctly: within half an FP32 ulp of values below 1 (2^-25)
    assert e_entry <= 2.0 ** -25, e_entry


BERNOULLI = r"""
#include <cmath>
#include <cstdio>
#include "mixture.cuh"

int main() {
  // B(x) = x / (1 - e^{-x}) on [0, 0.5], the range where the mixture-only
  // kernels' vMF normaliser takes the series (1/4pi) B(2 kappa)
  const long n = 1000000;
  double er = 0.0;
  for (long i = 0; i <= n; ++i) {
    const float x = float(0.5 * double(i) / double(n));
    const long double xl = x;
    const long double exact = xl > 0 ? xl / -expm1l(-xl) : 1.0L;
    er = fmax(er, double(fabsl((long double)nmg::bernoulli_gen(x) / exact - 1.0L)));
  }
  // the sampler's 1 - e^{-2k} = 2k / B(2k), relative
  double ed = 0.0;
  for (long i = 1; i <= n; ++i) {
    const float x = float(0.5 * double(i) / double(n));
    const long double exact = -expm1l(-(long double)x);
    ed = fmax(ed, double(fabsl((long double)(x / nmg::bernoulli_gen(x)) / exact - 1.0L)));
  }
  printf("%.6e %.6e\n", er, ed);
  return 0;
}
"""


def test_bernoulli_series_within_2e7(tmp_path):
    """bernoulli_gen (csrc/mixture.cuh) against long double: the normaliser's series below
    2 kappa = 0.5 and the sampler's 1 - e^{-2 kappa} derived from it, both within 2e-7 relative
    (a few FP32 roundings; the truncation is below 3.3e-9)."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "bern.cu"
    src.write_text(BERNOULLI)
    exe = tmp_path / "bern"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", CSRC, str(src), "-o", str(exe)], check=True,
                   capture_output=True, timeout=600)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=600).stdout.split()
    e_series, e_den = float(out[0]), float(out[1])
    assert e_series <= 2e-7, e_series
    assert e_den <= 2e-7, e_den
