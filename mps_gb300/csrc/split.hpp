// Split-precision (bf16 slices on tcgen05) grouped block GEMM: host plan and launcher.
#pragma once

#include <cuda.h>
#include <vector_types.h>

#include <algorithm>
#include <vector>

#include "runtime.hpp"

namespace mpsg {
namespace split {

constexpr int BM = 128, BN = 64, BK = 64;
constexpr int kSliceBits = 7;  // beta: bits per bf16 slice digit
constexpr int kMaxSlices = 7;  // 49 bits: the FP64-class setting

// Accumulators of the exact mode. The products of slice pair (p, q) form group g = p + q, of
// relative weight 2^(-7 g). Groups g <= S - 3 keep one accumulator each, summed exactly within a
// chunk; the two smallest groups (S - 2 and S - 1) share one FP32 accumulator. Its rounding
// (2^-24 of a sum of weight 2^(-7(S-2))) stays about 2^-10 below the 2^(-7 S) slicing error
// even after a few thousand K indices, and it frees one accumulator of TMEM per tile.
constexpr int exact_accs(int S) { return S >= 2 ? S - 1 : 1; }

// K chunk of the exact mode: the longest K range whose exact group sums stay FP32 integers.
// Balanced digits satisfy |t_0| <= 2^7 and |t_p| <= 2^6 (p >= 1), so one K index adds at most
// 2^14 to group 0 and 2 * 2^13 + (g - 1) * 2^12 = 2^12 (g + 3) to group g >= 1; with exact
// groups g <= S - 3 the chunk is 2^24 / (2^12 max(4, S)), rounded down to a multiple of 64 (one
// packed row): 1024 up to S = 4, 576 at S = 7.
constexpr int exact_chunk(int S) { return ((4096 / (S > 4 ? S : 4)) / 64) * 64; }

// N tile of the exact mode: exact_accs(S) accumulators of exact_bn columns must fit the 512
// TMEM columns; 128-column MMAs halve the shared-memory operand traffic per MAC of 64-column
// ones.
constexpr int exact_bn(int S) { return exact_accs(S) * 128 <= 512 ? 128 : 64; }

// Kernel configuration of one grouped GEMM, chosen by the tuner (batch.cu) or left at the
// defaults: the N tile of the exact mode (0 = exact_bn(S); else 64 or exact_bn(S)), and the
// order in which output tiles are dealt to the persistent CTAs (kOrderK: decreasing K, which
// balances ragged sectors; kOrderProblem: problem by problem, N tile by N tile, which keeps the
// CTAs of one wave on the same operands).
enum { kOrderK = 0, kOrderProblem = 1 };
// splitk: cut the output tiles with the longest K loops into two halves at a chunk boundary
// while that leaves fewer than two waves of tiles on the GPU (exact mode only). Each half adds
// its FP64 partial result into the zeroed output with one atomic add; with exactly two terms
// the sum does not depend on their order, so results stay deterministic.
struct Tuning {
  int bn = 0;
  int order = kOrderK;
  int splitk = 0;
};

// One sector GEMM as the split kernels see it (column-major A: M x K, B: K x N, C: M x N).
struct Problem {
  int64_t M, N, K;
  int64_t offA, offB, offC, lda, ldb, ldc;
  int32_t mt, nt, nks, nch;  // M tiles, N tiles, K steps of 64, K chunks
  int64_t tA, tB;            // first packed tile of A / of B
  int64_t rA, rB;            // first row in the per-row exponent arrays (A rows, B columns)
  int64_t eA, eB;            // first entry in the per-(row, chunk) exponent arrays
};

// Device tables, packed-slice scratch and TMA descriptors of one grouped GEMM at S slices.
struct SplitPlan {
  int S = 0;
  cudaStream_t stream = nullptr;  // storage is allocated and freed in this stream's order
  bool fast = false;   // one FP32 accumulator, 128 x 256 tiles (S <= 3); else exact chunked mode
  int bn = 64;         // rows of a packed B tile = N of an output tile
  int order = kOrderK; // output tile order (Tuning)
  int64_t nsplit = 0;  // tiles cut in two by split-K
  int nzero = 0;       // problems whose output is zeroed before the GEMM (split tiles)
  int* d_zero = nullptr;
  int chunk = 0;       // K columns per exact chunk (whole K in fast mode)
  int seg = 0;         // K columns per exponent-pass work item
  int nprob = 0;
  int64_t ntiles = 0, tilesA = 0, tilesB = 0, rowsA = 0, rowsB = 0, nrowsA = 0, nrowsB = 0;
  int64_t rowsRA = 0, rowsCB = 0;  // entries of the row-reference exponent arrays
  double flops = 0;
  std::vector<Problem> probs;
  Problem* d_probs = nullptr;
  int64_t *d_tile_prefix = nullptr, *d_packA_prefix = nullptr, *d_packB_prefix = nullptr;
  int64_t *d_rowA_prefix = nullptr, *d_rowB_prefix = nullptr;
  int32_t *d_RA = nullptr, *d_CB = nullptr;
  int16_t *d_EA = nullptr, *d_EB = nullptr;
  void *d_packA = nullptr, *d_packB = nullptr;
  int* d_err = nullptr;
  int4* d_tiles = nullptr;  // output tiles (problem, M tile, N tile, K steps), descending K
  alignas(64) CUtensorMap tmA;
  alignas(64) CUtensorMap tmB;
  void build(Context* ctx, const std::vector<GemmTask>& g, int S, Tuning t = Tuning());
  void release();
  ~SplitPlan() { release(); }
};

int chunk_for(int S);

// Split-K of a tile list (host): tiles are (problem, M tile, N tile, kb | ke << 16) with K steps
// [kb, ke) of 64 columns. The tiles with the longest K loops (stable order) are halved at a
// multiple of c64 K steps (one exact chunk) while the list has fewer than `target` tiles; each
// halved tile's problem is marked in `zero_prob` (its output is zeroed, the halves add into
// it). Returns the number of tiles halved. Pure host code (checked on the CPU).
inline int64_t split_k_tiles(std::vector<int4>& tl, const std::vector<Problem>& probs, int c64,
                             int64_t target, std::vector<char>& zero_prob) {
  auto work = [](const int4& t) { return (int)((unsigned)t.w >> 16) - (t.w & 0xffff); };
  std::stable_sort(tl.begin(), tl.end(),
                   [&](const int4& a, const int4& b) { return work(a) > work(b); });
  int64_t n = 0;
  const size_t n0 = tl.size();
  for (size_t i = 0; i < n0 && (int64_t)tl.size() < target; ++i) {
    const int4 t = tl[i];  // a copy: push_back below may move the list
    const int nks = probs[t.x].nks;
    const int mid = c64 > 0 ? ((nks / c64) / 2) * c64 : 0;
    if (mid <= 0 || mid >= nks || work(t) != nks) continue;  // short, or already a half
    tl[i].w = mid << 16;
    tl.push_back(make_int4(t.x, t.y, t.z, mid | (nks << 16)));
    zero_prob[t.x] = 1;
    ++n;
  }
  return n;
}
// what: bit 0 = pack A, bit 1 = pack B, bit 2 = run the GEMM (an operand packed by an earlier
// call stays valid in the plan's scratch until the plan is packed again).
enum { kPackA = 1, kPackB = 2, kRunGemm = 4, kAll = 7 };
void launch_split_gemm(Context* ctx, SplitPlan& sp, const double* A, const double* B, double* C,
                       int what = kAll);
// Error code recorded by the kernel (0 = none; nonzero = a bounded wait timed out).
int read_error(Context* ctx, SplitPlan& sp);

}  // namespace split
}  // namespace mpsg
