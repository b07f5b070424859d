"""The row table of the TMA-staged copy path (mps_gb300/csrc/copy_decode.hpp) on the CPU, compiled
with g++: for random tasks, with a unit-stride axis shared by source and destination or with a
strided row axis, the rows ``append_bulk_rows`` emits move exactly the task's (source,
destination) element pairs, each row holds 1..max elements, and the 16-byte-aligned interior
``row_interior`` gives the bulk copy (aligned start, a multiple of 16 bytes, inside the row, at
most one element left at each end) covers every other element of a unit-stride row. A planted
off-by-one in the row lengths is caught."""
import shutil
import subprocess

import pytest

from test_copy_decode_cpu import CSRC

HARNESS = r"""
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <utility>
#include <vector>
#include "copy_decode.hpp"
using namespace mpsg;

// one random task; returns the number of violations found
static long run_task(std::mt19937_64& g, int plant, int maxe, long& elems, long& rows_out) {
  const int nd = 1 + (int)(g() % 5);
  const int a = (int)(g() % nd);
  int64_t ext[6], sstr[6], dstr[6];
  int64_t n = 1;
  for (int i = 0; i < nd; ++i) {
    ext[i] = 1 + (int64_t)(g() % 12);
    if (i == a) ext[i] = 32 + (int64_t)(g() % 1500);
    if (n * ext[i] > 300000) ext[i] = i == a ? ext[i] : 1;
    n *= ext[i];
  }
  // unit stride along a on both sides (or, one task in four, strides 2..4 on one side), the
  // other axes strided in random orders with padding
  int perm_s[6], perm_d[6], k = 0;
  for (int i = 0; i < nd; ++i) if (i != a) { perm_s[k] = i; perm_d[k] = i; ++k; }
  std::shuffle(perm_s, perm_s + k, g);
  std::shuffle(perm_d, perm_d + k, g);
  sstr[a] = dstr[a] = 1;
  if (g() % 4 == 0) (g() % 2 ? sstr[a] : dstr[a]) = 2 + (int64_t)(g() % 3);
  int64_t s = ext[a] * sstr[a] + (int64_t)(g() % 3), d = ext[a] * dstr[a];
  for (int j = 0; j < k; ++j) {
    sstr[perm_s[j]] = s;
    s *= ext[perm_s[j]] + (int64_t)(g() % 2);
    dstr[perm_d[j]] = d;
    d *= ext[perm_d[j]];
  }
  const int64_t soff = (int64_t)(g() % 1000), doff = (int64_t)(g() % 1000);
  std::vector<BulkRow> rows;
  append_bulk_rows(nd, ext, sstr, dstr, soff, doff, a, maxe, rows);
  if (plant && !rows.empty()) rows[rows.size() / 2].len -= 1;
  long bad = 0;
  std::vector<std::pair<int64_t, int64_t>> got, want;
  for (const BulkRow& r : rows) {
    if (r.len < 1 || r.len > maxe || r.sstr != sstr[a] || r.dstr != dstr[a]) ++bad;
    for (int32_t i = 0; i < r.len; ++i)
      got.push_back({r.soff + (int64_t)i * r.sstr, r.doff + (int64_t)i * r.dstr});
    // the bulk part of the row at a random 8-byte-aligned base address
    const uint64_t a0 = 4096 + 8 * (g() % 64) + 8 * (uint64_t)r.soff;
    uint64_t i0, i1;
    row_interior(a0, r.len, i0, i1);
    if (i0 % 16 || i1 % 16 || (i1 - i0) % 16 || i0 < a0 || i1 > a0 + 8 * (uint64_t)r.len) ++bad;
    if (i1 - i0 > 8 * (uint64_t)maxe) ++bad;
    if (i0 - a0 > 8 || a0 + 8 * (uint64_t)r.len - i1 > 8) ++bad;
  }
  int ax[6], nax = 0;
  for (int i = 0; i < nd; ++i) ax[nax++] = i;
  for (int64_t q = 0; q < n; ++q) {
    int64_t so = soff, dof = doff;
    ref_decode(ext, sstr, dstr, ax, nax, q, so, dof);
    want.push_back({so, dof});
  }
  std::sort(got.begin(), got.end());
  std::sort(want.begin(), want.end());
  if (got != want) ++bad;
  elems += n;
  rows_out += (long)rows.size();
  return bad;
}

int main(int argc, char** argv) {
  const int plant = argc > 1 ? atoi(argv[1]) : 0;
  std::mt19937_64 g(7);
  long elems = 0, rows = 0, bad_tasks = 0;
  const int tasks = 300;
  for (int t = 0; t < tasks; ++t) {
    const int maxe = t % 3 == 0 ? 512 : (t % 3 == 1 ? 64 : 33);
    if (run_task(g, plant, maxe, elems, rows)) ++bad_tasks;
  }
  printf("%d %ld %ld %ld\n", tasks, bad_tasks, elems, rows);
  return 0;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("rows")
    src = d / "h.cpp"
    src.write_text(HARNESS)
    exe = d / "h"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    return str(exe)


def _run(exe, plant):
    out = subprocess.run([exe, str(plant)], check=True, capture_output=True, text=True).stdout
    return [int(x) for x in out.split()]


def test_rows_cover_each_task_exactly(harness):
    tasks, bad, elems, rows = _run(harness, 0)
    assert tasks == 300 and elems > 100000 and rows > 1000
    assert bad == 0


def test_planted_row_length_mistake_is_caught(harness):
    tasks, bad, _, _ = _run(harness, 1)
    assert bad == tasks
