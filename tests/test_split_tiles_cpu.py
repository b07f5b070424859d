"""The split-K tile list of the exact split GEMM (``split_k_tiles`` in
mps_gb300/csrc/split.hpp) on the CPU, compiled with g++: for random problem lists, every output
tile is covered once (whole K) or by exactly two halves that meet at a multiple of the exact
chunk, only problems with halves are marked for zeroing, no tile is split twice, and splitting
stops once the list reaches the target count."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "mps_gb300", "csrc")
CUDA_INC = "/usr/local/cuda/include"

HARNESS = r"""
#include <cstdio>
#include <map>
#include <random>
#include <tuple>
#include "split.hpp"
using namespace mpsg;
using namespace mpsg::split;

int main() {
  std::mt19937_64 g(7);
  long bad = 0, splits = 0;
  for (int trial = 0; trial < 400; ++trial) {
    const int nprob = 1 + (int)(g() % 30), c64 = 1 + (int)(g() % 16);
    std::vector<Problem> probs(nprob);
    std::vector<int4> tl;
    for (int p = 0; p < nprob; ++p) {
      probs[p].nks = (int)(g() % 200);
      probs[p].mt = 1 + (int)(g() % 5);
      probs[p].nt = 1 + (int)(g() % 5);
      for (int ni = 0; ni < probs[p].nt; ++ni)
        for (int mi = 0; mi < probs[p].mt; ++mi)
          tl.push_back(make_int4(p, mi, ni, probs[p].nks << 16));
    }
    const size_t n0 = tl.size();
    const int64_t target = 1 + (int64_t)(g() % (2 * n0 + 2));
    std::vector<char> zero(nprob, 0);
    const int64_t n = split_k_tiles(tl, probs, c64, target, zero);
    splits += n;
    if ((int64_t)tl.size() != (int64_t)n0 + n) ++bad;
    if (n > 0 && (int64_t)tl.size() > std::max<int64_t>(target, (int64_t)n0)) ++bad;
    std::map<std::tuple<int, int, int>, std::vector<std::pair<int, int>>> cover;
    for (const int4& t : tl)
      cover[{t.x, t.y, t.z}].push_back({t.w & 0xffff, (int)((unsigned)t.w >> 16)});
    std::vector<char> has_half(nprob, 0);
    for (auto& e : cover) {
      const int p = std::get<0>(e.first), nks = probs[p].nks;
      auto v = e.second;
      std::sort(v.begin(), v.end());
      if (v.size() == 1) {
        if (v[0].first != 0 || v[0].second != nks) ++bad;
      } else if (v.size() == 2) {
        has_half[p] = 1;
        const int mid = v[0].second;
        if (v[0].first != 0 || v[1].first != mid || v[1].second != nks) ++bad;
        if (mid <= 0 || mid >= nks || mid % c64 != 0) ++bad;
      } else {
        ++bad;
      }
    }
    for (int p = 0; p < nprob; ++p)
      if ((bool)has_half[p] != (bool)zero[p]) ++bad;
  }
  printf("%ld %ld\n", bad, splits);
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None or not os.path.isdir(CUDA_INC),
                    reason="g++ and the CUDA headers are needed")
def test_split_k_tiles_cover_every_tile_once(tmp_path):
    src = tmp_path / "h.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "h"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", CSRC, "-I", CUDA_INC, str(src), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    bad, splits = int(out[0]), int(out[1])
    assert bad == 0
    assert splits > 100  # the random lists do exercise the splitting
