"""The copy engine's index decoding (mps_gb300/csrc/copy_decode.hpp) on the CPU, compiled with g++:
the magic-number division the kernel runs equals plain division for every position of random
tasks, every decoded address lies inside the task span, the span is reached, and the comparison
the device-checked library makes catches a planted wrong division constant or extent."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "mps_gb300", "csrc")

HARNESS = r"""
#include <cstdio>
#include <cstdlib>
#include <random>
#include "copy_decode.hpp"
using namespace mpsg;

// decodes every position of a random task both ways; returns mismatches (and span misses)
static long run_task(std::mt19937_64& g, int plant, long& positions) {
  const int nd = 1 + (int)(g() % 6);
  int64_t ext[6], sstr[6], dstr[6];
  uint32_t mag[6], shf[6];
  int ax[6];
  int64_t n = 1;
  for (int i = 0; i < nd; ++i) {
    ext[i] = 1 + (int64_t)(g() % 40);
    if (g() % 8 == 0) ext[i] = 1 + (int64_t)(g() % 3000);
    if (n * ext[i] > 200000) ext[i] = 1;
    n *= ext[i];
    ax[i] = i;
  }
  for (int i = nd - 1; i > 0; --i) std::swap(ax[i], ax[(int)(g() % (i + 1))]);
  // destination dense in the decode order, source strided with padding between axes
  int64_t s = 1, d = 1;
  for (int j = 0; j < nd; ++j) {
    dstr[ax[j]] = d;
    d *= ext[ax[j]];
  }
  for (int i = 0; i < nd; ++i) {
    sstr[i] = s;
    s *= ext[i] + (int64_t)(g() % 3);
  }
  for (int i = 0; i < nd; ++i) magic_u31((uint32_t)ext[i], mag[i], shf[i]);
  if (plant == 1) {  // the division constants of a wrong extent, on an axis that is not last
    for (int j = 0; j < nd - 1; ++j)
      if (ext[ax[j]] > 1) { magic_u31((uint32_t)ext[ax[j]] + 1, mag[ax[j]], shf[ax[j]]); break; }
  }
  int64_t ext_fast[6];
  for (int i = 0; i < nd; ++i) ext_fast[i] = ext[i];
  if (plant == 2) {  // a wrong extent in the fast decode
    for (int i = 0; i < nd - 1; ++i)
      if (ext[ax[i]] > 1) { ext_fast[ax[i]] += 1; break; }
  }
  const int64_t soff = (int64_t)(g() % 1000), doff = (int64_t)(g() % 1000);
  int64_t slo, shi, dlo, dhi;
  task_span(ext, sstr, nd, soff, slo, shi);
  task_span(ext, dstr, nd, doff, dlo, dhi);
  long bad = 0;
  int64_t smax = soff, dmax = doff;
  for (int64_t q = 0; q < n; ++q) {
    int64_t rs = soff, rd = doff, fs = soff, fd = doff;
    ref_decode(ext, sstr, dstr, ax, nd, q, rs, rd);
    fast_decode(ext_fast, sstr, dstr, mag, shf, ax, nd, (uint32_t)q, fs, fd);
    if (rs != fs || rd != fd) ++bad;
    if (rs < slo || rs > shi || rd < dlo || rd > dhi) ++bad;
    if (rs > smax) smax = rs;
    if (rd > dmax) dmax = rd;
  }
  if (plant == 0 && (smax != shi || dmax != dhi || slo != soff || dlo != doff)) ++bad;
  positions += n;
  return bad;
}

int main(int argc, char** argv) {
  const int plant = argc > 1 ? atoi(argv[1]) : 0;
  std::mt19937_64 g(1911);
  long positions = 0, bad_tasks = 0, tasks = 0;
  for (int t = 0; t < 400; ++t) {
    const long b = run_task(g, plant, positions);
    ++tasks;
    if (b) ++bad_tasks;
  }
  // the magic-number division itself at the top of its range
  long bad_div = 0;
  for (uint32_t d = 1; d < 5000; d += 7) {
    uint32_t m, s;
    magic_u31(d, m, s);
    for (uint32_t n : {0u, 1u, d - 1, d, d + 1, 0x7fffffffu, 0x7ffffffeu, 0x40000000u})
      if (fdiv(n, m, s) != n / d) ++bad_div;
  }
  printf("%ld %ld %ld %ld\n", tasks, bad_tasks, positions, bad_div);
  return 0;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("decode")
    src = d / "h.cpp"
    src.write_text(HARNESS)
    exe = d / "h"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    return str(exe)


def _run(exe, plant):
    out = subprocess.run([exe, str(plant)], check=True, capture_output=True, text=True).stdout
    return [int(x) for x in out.split()]


def test_fast_decode_equals_plain_division_and_stays_in_span(harness):
    tasks, bad_tasks, positions, bad_div = _run(harness, 0)
    assert tasks == 400 and positions > 100000
    assert bad_tasks == 0 and bad_div == 0


@pytest.mark.parametrize("plant", [1, 2])
def test_planted_decode_mistakes_are_caught(harness, plant):
    tasks, bad_tasks, positions, _ = _run(harness, plant)
    assert bad_tasks > tasks // 4


def test_normal_library_has_no_device_checks():
    import mps_gb300 as mg
    assert not mg.checked_library()
    with pytest.raises(mg.MPSGError) as e:
        mg.device_checks()
    assert e.value.code == 5
