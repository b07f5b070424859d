// Block-permute engine: executes a list of strided N-d copy tasks (permutelegs, fuselegs,
// splitleg, SymMatrix fusion and the split+permute of contraction outputs are all such lists).
//
// Work is dealt out per warp (no block-wide barriers): a persistent grid walks a global unit
// index, each warp finds its task by binary search in the per-task unit prefix sums and keeps
// the task's extents, strides and division constants in a per-warp slot of shared memory.
// One of three unit shapes is chosen per task on the host:
//   * row    : source and destination share their unit-stride axis a and it holds at least 32
//              elements; a unit is a group of rows along a, each row's multi-index is decoded
//              once (magic-number division) and the lanes stream it, coalesced on both sides;
//   * tile   : the unit-stride axes differ (a transpose) and both hold at least 16 elements; a
//              unit is a 32 x 32 tile staged in the warp's shared-memory slot, read coalesced
//              along the source axis and written coalesced along the destination axis;
//   * gather : everything else (short runs, e.g. the MPO and physical legs of size 1..12); a
//              unit is 256 consecutive destination positions in destination-stride order, one
//              per lane and step, each decoded to its source address. Writes stay coalesced and
//              reads follow the source's short runs through the caches.
//
// Tasks whose source and destination share a unit-stride axis of at least 32 elements (the
// bulk of every fusion and split of the contraction path) do not go through the warp units:
// the host cuts them into rows of at most 512 elements and copy_rows_bulk_kernel moves them.
// Each warp keeps a ring of kBulkStages row slots in shared memory; one lane stages the
// 16-byte-aligned interior of each row with a bulk asynchronous copy (cp.async.bulk, completion
// counted on the slot's mbarrier) several rows ahead, and the warp writes the row out with
// coalesced stores, reading the at most two unaligned end elements straight from global memory.
// A few KB per warp in flight keep HBM busy with one load instruction per row.
//
// Built with MPSG_DEVICE_CHECKS (the device-checked debug library), the kernel also recomputes
// every decoded offset by plain division, checks every address against its task's span, records
// the first violation and a count in device memory (read_device_checks) and skips the access.
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "copy_decode.hpp"
#include "runtime.hpp"

namespace mpsg {

namespace {

#ifdef MPSG_DEVICE_CHECKS
enum CheckKind { kChkTask = 1, kChkDecode = 2, kChkSpan = 3 };
__device__ unsigned long long g_chk_count;
__device__ long long g_chk_first[4];  // kind, task, index, detail

__device__ __noinline__ void chk_fail(int kind, long long task, long long index,
                                      long long detail) {
  if (atomicAdd(&g_chk_count, 1ull) == 0ull) {
    g_chk_first[0] = kind;
    g_chk_first[1] = task;
    g_chk_first[2] = index;
    g_chk_first[3] = detail;
  }
}
#endif

constexpr int kWarps = 8;          // warps per CTA
// target elements per row-mode unit: small enough that a copy of a few MB spreads over every
// resident warp and each warp's chain of dependent load batches stays short
constexpr int kRowElems = 256;
constexpr int kGatherUnit = 256;   // destination positions per gather unit
constexpr int kT = 32;             // transpose tile edge

enum CopyMode { kModeRow = 0, kModeTile = 1, kModeGather = 2 };

// Per-task launch data: mode, axis roles, tiling, gather order and division constants
// (q = (umulhi(n,m)+n) >> s equals n / ext for every n < 2^31).
struct TaskAux {
  int32_t mode, a, b, rows_per_unit;
  int64_t outer;  // row mode: rows; tile mode: tiles
  int32_t order[kMaxTaskDims];  // gather mode: axes by ascending destination stride
  uint32_t mag[kMaxTaskDims];
  uint32_t shf[kMaxTaskDims];
};

struct WarpView {
  int task, nd, mode, a, b, rpu;
  int64_t outer, soff, doff, first;
  int64_t ext[kMaxTaskDims], sstr[kMaxTaskDims], dstr[kMaxTaskDims];
  uint32_t mag[kMaxTaskDims], shf[kMaxTaskDims];
  int32_t order[kMaxTaskDims];
#ifdef MPSG_DEVICE_CHECKS
  int64_t slo, shi, dlo, dhi;  // address spans of the task
#endif
};

typedef double TileBuf[kT][kT + 1];

#ifdef MPSG_DEVICE_CHECKS
// Offsets of position q over every axis except skip0 / skip1, by plain division, compared with
// the kernel's magic-number decode; records a mismatch and returns false.
__device__ bool chk_decode(const WarpView& v, int skip0, int skip1, int64_t q, int64_t so,
                           int64_t dof) {
  int ax[kMaxTaskDims];
  int nax = 0;
  for (int i = 0; i < v.nd; ++i)
    if (i != skip0 && i != skip1) ax[nax++] = i;
  int64_t rs = v.soff, rd = v.doff;
  ref_decode(v.ext, v.sstr, v.dstr, ax, nax, q, rs, rd);
  if (rs == so && rd == dof) return true;
  chk_fail(kChkDecode, v.task, q, rs != so ? so - rs : dof - rd);
  return false;
}

__device__ __forceinline__ bool chk_addr(const WarpView& v, int64_t s, int64_t d) {
  if (s >= v.slo && s <= v.shi && d >= v.dlo && d <= v.dhi) return true;
  chk_fail(kChkSpan, v.task, s, d);
  return false;
}
#endif

// Dynamic shared memory: kWarps task views, then (only for plans with tile-mode tasks) kWarps
// transpose tiles; plans without tiles launch with the views alone. 64 registers per thread
// keep 4 CTAs (32 warps) resident per SM.
__global__ void __launch_bounds__(32 * kWarps, 4) copy_tasks_kernel(
    const CopyTask* __restrict__ tasks, const int64_t* __restrict__ prefix,
    const TaskAux* __restrict__ aux, int ntasks, int64_t nunits, const double* __restrict__ src,
    double* __restrict__ dst) {
  extern __shared__ __align__(16) unsigned char copy_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpView& v = reinterpret_cast<WarpView*>(copy_smem)[warp];
  TileBuf& tile = reinterpret_cast<TileBuf*>(copy_smem + sizeof(WarpView) * kWarps)[warp];
  if (lane == 0) v.task = -1;
  __syncwarp();
  const int64_t stride = (int64_t)gridDim.x * kWarps;
  for (int64_t u = (int64_t)blockIdx.x * kWarps + warp; u < nunits; u += stride) {
    int lo = 0, hi = ntasks - 1;  // largest k with prefix[k] <= u (same answer in every lane)
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(prefix + mid) <= u) lo = mid;
      else hi = mid - 1;
    }
#ifdef MPSG_DEVICE_CHECKS
    if (lo < 0 || lo >= ntasks || __ldg(prefix + lo) > u || __ldg(prefix + lo + 1) <= u) {
      if (lane == 0) chk_fail(kChkTask, lo, u, 0);
      continue;
    }
#endif
    if (lo != v.task) {
      __syncwarp();
      const CopyTask& T = tasks[lo];
      const TaskAux& X = aux[lo];
      const int nd = T.nd;
      if (lane < nd) {
        v.ext[lane] = T.ext[lane];
        v.sstr[lane] = T.sstr[lane];
        v.dstr[lane] = T.dstr[lane];
        v.mag[lane] = X.mag[lane];
        v.shf[lane] = X.shf[lane];
        v.order[lane] = X.order[lane];
      }
      if (lane == 0) {
        v.nd = nd;
        v.mode = X.mode;
        v.a = X.a;
        v.b = X.b;
        v.rpu = X.rows_per_unit;
        v.outer = X.outer;
        v.soff = T.soff;
        v.doff = T.doff;
        v.first = prefix[lo];
        v.task = lo;
#ifdef MPSG_DEVICE_CHECKS
        task_span(T.ext, T.sstr, nd, T.soff, v.slo, v.shi);
        task_span(T.ext, T.dstr, nd, T.doff, v.dlo, v.dhi);
#endif
      }
      __syncwarp();
    }
    const int64_t lu = u - v.first;
    const int nd = v.nd;
    if (v.mode == kModeRow) {
      const int a = v.a;
      const int64_t ea = v.ext[a];
      // rpu > 0: rows_per_unit whole rows; rpu < 0: each row is cut into -rpu chunks
      int64_t r0, r1, c0 = 0, c1 = ea;
      if (v.rpu > 0) {
        r0 = lu * v.rpu;
        r1 = min(r0 + v.rpu, v.outer);
      } else {
        r0 = lu / (-v.rpu);
        r1 = r0 + 1;
        c0 = (lu - r0 * (-v.rpu)) * kRowElems;
        c1 = min(c0 + kRowElems, ea);
      }
      for (int64_t row = r0; row < r1; ++row) {
        uint32_t q = (uint32_t)row;
        int64_t so = v.soff, dof = v.doff;
        for (int i = 0; i < nd; ++i) {
          if (i == a) continue;
          const uint32_t qi = fdiv(q, v.mag[i], v.shf[i]);
          const int64_t ii = (int64_t)(q - qi * (uint32_t)v.ext[i]);
          q = qi;
          so += ii * v.sstr[i];
          dof += ii * v.dstr[i];
        }
#ifdef MPSG_DEVICE_CHECKS
        if (row >= v.outer || c0 < 0 || c1 > ea || !chk_decode(v, a, -1, row, so, dof)) {
          if (lane == 0 && (row >= v.outer || c0 < 0 || c1 > ea)) chk_fail(kChkSpan, v.task, row, c1);
          continue;
        }
#endif
        // four loads in flight per lane before the stores
        for (int64_t ia = c0 + lane; ia < c1; ia += 128) {
          double x[4];
          bool ok[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            ok[k] = ia + 32 * k < c1;
#ifdef MPSG_DEVICE_CHECKS
            if (ok[k]) ok[k] = chk_addr(v, so + ia + 32 * k, dof + ia + 32 * k);
#endif
          }
#pragma unroll
          for (int k = 0; k < 4; ++k)
            if (ok[k]) x[k] = __ldg(src + so + ia + 32 * k);
#pragma unroll
          for (int k = 0; k < 4; ++k)
            if (ok[k]) dst[dof + ia + 32 * k] = x[k];
        }
      }
    } else if (v.mode == kModeTile) {
      const int a = v.a, b = v.b;
      const int64_t ea = v.ext[a], eb = v.ext[b];
      const int64_t ta = (ea + kT - 1) / kT, tb = (eb + kT - 1) / kT;
      int64_t q = lu;
      const int64_t ia = q % ta;
      q /= ta;
      const int64_t ib = q % tb;
      q /= tb;
      int64_t so = v.soff, dof = v.doff;
      uint32_t q32 = (uint32_t)q;
      for (int i = 0; i < nd; ++i) {
        if (i == a || i == b) continue;
        const uint32_t qi = fdiv(q32, v.mag[i], v.shf[i]);
        const int64_t ii = (int64_t)(q32 - qi * (uint32_t)v.ext[i]);
        q32 = qi;
        so += ii * v.sstr[i];
        dof += ii * v.dstr[i];
      }
#ifdef MPSG_DEVICE_CHECKS
      if (!chk_decode(v, a, b, q, so, dof)) continue;  // uniform over the warp
#endif
      const int64_t a0 = ia * kT, b0 = ib * kT;
      const int64_t sa = v.sstr[a], db = v.dstr[b];
#pragma unroll 8
      for (int r = 0; r < kT; ++r) {  // rows along a, lanes along b (source-contiguous)
        bool ok = a0 + r < ea && b0 + lane < eb;
#ifdef MPSG_DEVICE_CHECKS
        if (ok) ok = chk_addr(v, so + (a0 + r) * sa + b0 + lane, dof);
#endif
        if (ok) tile[r][lane] = __ldg(src + so + (a0 + r) * sa + b0 + lane);
      }
      __syncwarp();
#pragma unroll 8
      for (int c = 0; c < kT; ++c) {  // columns along b, lanes along a (destination-contiguous)
        bool ok = a0 + lane < ea && b0 + c < eb;
#ifdef MPSG_DEVICE_CHECKS
        if (ok) ok = chk_addr(v, so, dof + a0 + lane + (b0 + c) * db);
#endif
        if (ok) dst[dof + a0 + lane + (b0 + c) * db] = tile[lane][c];
      }
      __syncwarp();
    } else {
      // decode all of this lane's positions first, then issue every load, then every store
      constexpr int kPer = kGatherUnit / 32;
      const int64_t n = v.outer;
      const int64_t p0 = lu * kGatherUnit;
      int64_t so[kPer], dof[kPer];
#pragma unroll
      for (int k = 0; k < kPer; ++k) {
        const int64_t p = p0 + k * 32 + lane;
        uint32_t q = (uint32_t)(p < n ? p : 0);
        so[k] = v.soff;
        dof[k] = p < n ? v.doff : -1;
        for (int j = 0; j < nd; ++j) {
          const int i = v.order[j];
          const uint32_t qi = fdiv(q, v.mag[i], v.shf[i]);
          const int64_t ii = (int64_t)(q - qi * (uint32_t)v.ext[i]);
          q = qi;
          so[k] += ii * v.sstr[i];
          if (dof[k] >= 0) dof[k] += ii * v.dstr[i];
        }
#ifdef MPSG_DEVICE_CHECKS
        if (dof[k] >= 0) {
          int64_t rs = v.soff, rd = v.doff;
          ref_decode(v.ext, v.sstr, v.dstr, v.order, nd, p, rs, rd);
          if (rs != so[k] || rd != dof[k]) {
            chk_fail(kChkDecode, v.task, p, rs != so[k] ? so[k] - rs : dof[k] - rd);
            dof[k] = -1;
          } else if (!chk_addr(v, so[k], dof[k])) {
            dof[k] = -1;
          }
        }
#endif
      }
      double x[kPer];
#pragma unroll
      for (int k = 0; k < kPer; ++k)
        if (dof[k] >= 0) x[k] = __ldg(src + so[k]);
#pragma unroll
      for (int k = 0; k < kPer; ++k)
        if (dof[k] >= 0) dst[dof[k]] = x[k];
    }
  }
}

constexpr size_t kViewSmem = sizeof(WarpView) * kWarps;
constexpr size_t kTileSmem = kViewSmem + sizeof(TileBuf) * kWarps;

// ---- TMA-staged rows --------------------------------------------------------------------------
constexpr int kBulkWarps = 8;
constexpr int kBulkStages = 3;
constexpr int kSlotBytes = kBulkMaxRow * 8;  // a row's aligned interior is at most its bytes
constexpr size_t kBulkSmem = (size_t)kBulkWarps * kBulkStages * kSlotBytes +
                             sizeof(uint64_t) * kBulkWarps * kBulkStages;
constexpr long long kBulkWaitCycles = 4000000000LL;  // about 2 s at the maximum SM clock
enum BulkError { kBulkErrWait = 1, kBulkErrDrain = 2 };

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ bool bulk_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for a slot's phase; false after about 2 s.
__device__ __forceinline__ bool bulk_wait(uint64_t* bar, uint32_t parity) {
  if (bulk_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (!bulk_try_wait(bar, parity))
    if (clock64() - t0 > kBulkWaitCycles) return false;
  return true;
}

// Byte span [i0, i1) of row r's 16-byte-aligned interior in the source.
__device__ __forceinline__ void row_span(const double* src, const BulkRow& r, uint64_t& a0,
                                         uint64_t& i0, uint64_t& i1) {
  a0 = (uint64_t)(uintptr_t)(src + r.soff);
  row_interior(a0, r.len, i0, i1);
}

// Lane 0: stage row u's interior into `slot`, completion counted on `bar` (a strided row or an
// empty interior just arrives, so the phase still completes).
__device__ __forceinline__ void bulk_issue(const BulkRow* rows, int64_t u, const double* src,
                                           unsigned char* slot, uint64_t* bar) {
  const BulkRow r = rows[u];
  uint64_t a0, i0, i1;
  row_span(src, r, a0, i0, i1);
  const uint32_t bytes = r.sstr == 1 ? (uint32_t)(i1 - i0) : 0u;
  if (bytes == 0) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
    return;
  }
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(slot)),
      "l"(i0), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Persistent grid; warp w of the grid moves rows w, w + W, w + 2W, ... (W = warps in the grid),
// kBulkStages rows in flight. A wait that expires records kBulkErrWait in *err, and the warp
// stops after draining the copies it has in flight (bounded as well; kBulkErrDrain if that
// expires too).
__global__ void __launch_bounds__(32 * kBulkWarps, 2) copy_rows_bulk_kernel(
    const BulkRow* __restrict__ rows, int64_t nrows, const double* __restrict__ src,
    double* __restrict__ dst, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char bulk_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* slots = bulk_smem + (size_t)warp * kBulkStages * kSlotBytes;
  uint64_t* bars = reinterpret_cast<uint64_t*>(bulk_smem + (size_t)kBulkWarps * kBulkStages *
                                                               kSlotBytes) +
                   warp * kBulkStages;
  const int64_t W = (int64_t)gridDim.x * kBulkWarps;
  const int64_t first = (int64_t)blockIdx.x * kBulkWarps + warp;
  const int64_t mine = first < nrows ? (nrows - 1 - first) / W + 1 : 0;
  if (mine == 0) return;
  if (lane == 0) {
    for (int s = 0; s < kBulkStages; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[s])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    for (int64_t j = 0; j < mine && j < kBulkStages; ++j)
      bulk_issue(rows, first + j * W, src, slots + j * kSlotBytes, &bars[j]);
  }
  __syncwarp();
  for (int64_t j = 0; j < mine; ++j) {
    const int s = (int)(j % kBulkStages);
    const uint32_t parity = (uint32_t)((j / kBulkStages) & 1);
    const bool ok = bulk_wait(&bars[s], parity);
    if (!__all_sync(0xffffffffu, ok)) {
      // give up: wait (bounded) for every copy this warp still has in flight, this row's
      // included, before the block's shared memory goes away
      if (lane == 0) {
        atomicCAS(err, 0, kBulkErrWait);
        for (int64_t k = j; k < mine && k < j + kBulkStages; ++k)
          if (!bulk_wait(&bars[k % kBulkStages], (uint32_t)((k / kBulkStages) & 1))) {
            atomicCAS(err, kBulkErrWait, kBulkErrDrain);
            break;
          }
      }
      __syncwarp();
      return;
    }
    const BulkRow r = rows[first + j * W];
    uint64_t a0, i0, i1;
    row_span(src, r, a0, i0, i1);
    const double* slot = reinterpret_cast<const double*>(slots + s * kSlotBytes);
    const double* gsrc = src + r.soff;
    double* gdst = dst + r.doff;
    if (r.sstr == 1 && r.dstr == 1) {
#pragma unroll 4
      for (int i = lane; i < r.len; i += 32) {
        const uint64_t g = a0 + 8 * (uint64_t)i;
        gdst[i] = (g >= i0 && g < i1) ? slot[(g - i0) >> 3] : __ldg(gsrc + i);
      }
    } else if (r.sstr == 1) {
      for (int i = lane; i < r.len; i += 32) {
        const uint64_t g = a0 + 8 * (uint64_t)i;
        gdst[(int64_t)i * r.dstr] = (g >= i0 && g < i1) ? slot[(g - i0) >> 3] : __ldg(gsrc + i);
      }
    } else {  // a strided source row: plain loads
      for (int i = lane; i < r.len; i += 32)
        gdst[(int64_t)i * r.dstr] = __ldg(gsrc + (int64_t)i * r.sstr);
    }
    __syncwarp();  // every lane has read the slot before it is refilled
    if (lane == 0 && j + kBulkStages < mine) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      bulk_issue(rows, first + (j + kBulkStages) * W, src, slots + s * kSlotBytes, &bars[s]);
    }
  }
}

}  // namespace

size_t copy_aux_bytes() { return sizeof(TaskAux); }

void read_device_checks(Context* ctx, bool reset, int64_t* count, int64_t* first) {
#ifdef MPSG_DEVICE_CHECKS
  MPSG_CUDA(cudaSetDevice(ctx->device));
  MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
  unsigned long long n = 0;
  long long f[4] = {0, 0, 0, 0};
  MPSG_CUDA(cudaMemcpyFromSymbol(&n, g_chk_count, sizeof(n)));
  MPSG_CUDA(cudaMemcpyFromSymbol(f, g_chk_first, sizeof(f)));
  if (count) *count = (int64_t)n;
  if (first)
    for (int i = 0; i < 4; ++i) first[i] = f[i];
  if (reset) {
    const unsigned long long z = 0;
    const long long zf[4] = {0, 0, 0, 0};
    MPSG_CUDA(cudaMemcpyToSymbol(g_chk_count, &z, sizeof(z)));
    MPSG_CUDA(cudaMemcpyToSymbol(g_chk_first, zf, sizeof(zf)));
  }
#else
  (void)ctx;
  (void)reset;
  (void)count;
  (void)first;
  throw Error(kErrUnsupported, "library built without device checks (MPSG_DEVICE_CHECKS)");
#endif
}

void DevCopyPlan::upload(const std::vector<CopyTask>& tasks, bool identity_, cudaStream_t st) {
  release();
  stream = st;
  std::vector<CopyTask> rest;
  std::vector<int64_t> prefix;
  std::vector<unsigned char> aux;
  std::vector<BulkRow> rows;
  build_host(tasks, identity_, rest, prefix, aux, rows);
  // stream-ordered: no device-wide synchronisation, so contexts on one GPU do not serialise on
  // plan uploads (pageable sources are staged before the calls return)
  if (ntasks > 0) {
    MPSG_CUDA(cudaMallocAsync((void**)&d_tasks, sizeof(CopyTask) * ntasks, st));
    MPSG_CUDA(cudaMallocAsync((void**)&d_prefix, sizeof(int64_t) * (ntasks + 1), st));
    MPSG_CUDA(cudaMallocAsync(&d_aux, aux.size(), st));
    MPSG_CUDA(cudaMemcpyAsync(d_tasks, rest.data(), sizeof(CopyTask) * ntasks,
                              cudaMemcpyHostToDevice, st));
    MPSG_CUDA(cudaMemcpyAsync(d_prefix, prefix.data(), sizeof(int64_t) * (ntasks + 1),
                              cudaMemcpyHostToDevice, st));
    MPSG_CUDA(cudaMemcpyAsync(d_aux, aux.data(), aux.size(), cudaMemcpyHostToDevice, st));
  }
  if (nrows > 0) {
    MPSG_CUDA(cudaMallocAsync((void**)&d_rows, sizeof(BulkRow) * nrows, st));
    MPSG_CUDA(cudaMemcpyAsync(d_rows, rows.data(), sizeof(BulkRow) * nrows,
                              cudaMemcpyHostToDevice, st));
  }
}

void DevCopyPlan::build_host(const std::vector<CopyTask>& tasks, bool identity_,
                             std::vector<CopyTask>& rest, std::vector<int64_t>& prefix,
                             std::vector<unsigned char>& aux_bytes, std::vector<BulkRow>& rows) {
  identity = identity_;
  has_tile = false;
  rest.clear();
  rows.clear();
  aux_bytes.clear();
  prefix.assign(1, 0);
  elems = 0;
  // axis roles per task: a = destination's fastest axis, b = source's fastest axis
  const size_t nt = tasks.size();
  std::vector<int> ta(nt), tb(nt);
  int64_t bulk_elems = 0, other_rows = 0, bulk_rows = 0;
  for (size_t k = 0; k < nt; ++k) {
    const CopyTask& T = tasks[k];
    int a = 0, b = 0;
    for (int i = 1; i < T.nd; ++i) {
      if (T.dstr[i] < T.dstr[a]) a = i;
      if (T.sstr[i] < T.sstr[b]) b = i;
    }
    ta[k] = a;
    tb[k] = b;
    const int64_t n = T.numel();
    if (n >= ((int64_t)1 << 31)) throw Error(kErrUnsupported, "copy task above 2^31 elements");
    elems += n;
    if (n == 0) continue;
    const int64_t ea = T.nd > 0 ? T.ext[a] : 1;
    const int64_t nrow = (n / ea) * ((ea + kBulkMaxRow - 1) / kBulkMaxRow);
    if (T.nd > 0 && a == b && T.dstr[a] == 1 && T.sstr[a] == 1 && ea >= kBulkMinRow) {
      bulk_elems += n;
      bulk_rows += nrow;
    } else {
      other_rows += nrow;
    }
  }
  // the row table when nearly everything is long unit-stride rows and the other tasks add few
  // rows (each row costs one table entry and one pass of a warp)
  bool strides_fit = true;
  for (size_t k = 0; k < nt && strides_fit; ++k)
    if (tasks[k].nd > 0 && (std::abs(tasks[k].sstr[ta[k]]) >= ((int64_t)1 << 31) ||
                            std::abs(tasks[k].dstr[ta[k]]) >= ((int64_t)1 << 31)))
      strides_fit = false;
  const bool use_rows = !identity && strides_fit && bulk_elems > 0 &&
                        20 * (elems - bulk_elems) <= elems &&
                        other_rows <= std::max<int64_t>(4096, bulk_rows / 4);
  if (use_rows) {
    for (size_t k = 0; k < nt; ++k) {
      const CopyTask& T = tasks[k];
      if (T.numel() == 0) continue;
      if (T.nd == 0) {
        rows.push_back(BulkRow{T.soff, T.doff, 1, 1, 1, 0});
        continue;
      }
      append_bulk_rows(T.nd, T.ext, T.sstr, T.dstr, T.soff, T.doff, ta[k], kBulkMaxRow, rows);
    }
  } else {
    std::vector<TaskAux> aux;
    for (size_t k = 0; k < nt; ++k) {
      const CopyTask& T = tasks[k];
      const int64_t n = T.numel();
      if (n == 0) continue;
      const int a = ta[k], b = tb[k];
      const bool unit_a = T.nd > 0 && T.dstr[a] == 1, unit_b = T.nd > 0 && T.sstr[b] == 1;
      TaskAux X;
      std::memset(&X, 0, sizeof(X));
      for (int i = 0; i < T.nd; ++i) magic_u31((uint32_t)T.ext[i], X.mag[i], X.shf[i]);
      int64_t units;
      if (a == b && unit_a && unit_b && T.ext[a] >= 32) {
        X.mode = kModeRow;
        X.outer = n / T.ext[a];
        if (T.ext[a] > kRowElems) {  // long rows: several warps share a row
          const int64_t cpr = (T.ext[a] + kRowElems - 1) / kRowElems;
          X.rows_per_unit = -(int32_t)cpr;
          units = X.outer * cpr;
        } else {
          X.rows_per_unit =
              (int)std::max<int64_t>(1, std::min<int64_t>(X.outer, kRowElems / T.ext[a]));
          units = (X.outer + X.rows_per_unit - 1) / X.rows_per_unit;
        }
      } else if (a != b && unit_a && unit_b && T.ext[a] >= 16 && T.ext[b] >= 16) {
        X.mode = kModeTile;
        has_tile = true;
        const int64_t rest_ = n / (T.ext[a] * T.ext[b]);
        X.outer = ((T.ext[a] + kT - 1) / kT) * ((T.ext[b] + kT - 1) / kT) * rest_;
        units = X.outer;
      } else {
        X.mode = kModeGather;
        X.outer = n;
        for (int i = 0; i < T.nd; ++i) X.order[i] = i;
        std::stable_sort(X.order, X.order + T.nd,
                         [&](int x, int y) { return T.dstr[x] < T.dstr[y]; });
        units = (n + kGatherUnit - 1) / kGatherUnit;
      }
      X.a = a;
      X.b = b;
      rest.push_back(T);
      aux.push_back(X);
      prefix.push_back(prefix.back() + units);
    }
    aux_bytes.resize(sizeof(TaskAux) * aux.size());
    if (!aux.empty()) std::memcpy(aux_bytes.data(), aux.data(), aux_bytes.size());
  }
  ntasks = (int)rest.size();
  ntiles = prefix.back();
  nrows = (int64_t)rows.size();
}

void DevCopyPlan::release() {
  if (d_tasks) cudaFreeAsync(d_tasks, stream);
  if (d_prefix) cudaFreeAsync(d_prefix, stream);
  if (d_aux) cudaFreeAsync(d_aux, stream);
  if (d_rows) cudaFreeAsync(d_rows, stream);
  d_tasks = nullptr;
  d_prefix = nullptr;
  d_aux = nullptr;
  d_rows = nullptr;
  ntasks = 0;
  ntiles = 0;
  nrows = 0;
}

void launch_copy(Context* ctx, const DevCopyPlan& p, const double* src, double* dst) {
  if (p.elems == 0) return;
  if (p.identity) {
    if (src != dst)
      MPSG_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * p.elems, cudaMemcpyDeviceToDevice,
                                ctx->stream));
    return;
  }
  if (p.nrows > 0) {
    static std::once_flag bulk_set[kMaxDevices];
    set_smem_limit_once(ctx, bulk_set, copy_rows_bulk_kernel, (int)kBulkSmem);
    const int64_t ctas = (p.nrows + kBulkWarps - 1) / kBulkWarps;
    const int64_t grid = std::min<int64_t>(ctas, (int64_t)ctx->num_sms * 2);
    KernelTimer timer(ctx, kKindCopy);
    copy_rows_bulk_kernel<<<(unsigned)grid, 32 * kBulkWarps, kBulkSmem, ctx->stream>>>(
        p.d_rows, p.nrows, src, dst, ctx->d_copy_err);
    MPSG_CUDA(cudaGetLastError());
    ctx->kernel_launches++;
  }
  if (p.ntiles > 0) {
    static std::once_flag smem_set[kMaxDevices];  // the attribute is per device
    set_smem_limit_once(ctx, smem_set, copy_tasks_kernel, (int)kTileSmem);
    const size_t smem = p.has_tile ? kTileSmem : kViewSmem;
    const int64_t ctas = (p.ntiles + kWarps - 1) / kWarps;
    const int64_t grid = std::min<int64_t>(ctas, (int64_t)ctx->num_sms * (p.has_tile ? 3 : 8));
    KernelTimer timer(ctx, kKindCopy);
    copy_tasks_kernel<<<(unsigned)grid, 32 * kWarps, smem, ctx->stream>>>(
        p.d_tasks, p.d_prefix, (const TaskAux*)p.d_aux, p.ntasks, p.ntiles, src, dst);
    MPSG_CUDA(cudaGetLastError());
    ctx->kernel_launches++;
  }
  if (ctx->debug_sync && p.nrows > 0) {
    const int e = read_copy_error(ctx);
    if (e)
      throw Error(kErrCuda, "block copy: a bounded wait expired (code " + std::to_string(e) + ")");
  }
}

int read_copy_error(Context* ctx) {
  int e = 0;
  MPSG_CUDA(cudaMemcpyAsync(&e, ctx->d_copy_err, sizeof(int), cudaMemcpyDeviceToHost,
                            ctx->stream));
  MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (e) MPSG_CUDA(cudaMemsetAsync(ctx->d_copy_err, 0, sizeof(int), ctx->stream));
  return e;
}

}  // namespace mpsg
