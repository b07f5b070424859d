// Block-permute engine: executes a list of strided N-d copy tasks (permutelegs, fuselegs,
// splitleg, SymMatrix fusion and the split+permute of contraction outputs are all such lists).
//
// Two tile shapes, chosen per task on the host:
//   * rows : source and destination share their unit-stride axis a (or one side has none);
//            the task is walked as rows along axis a: each warp decodes a row's multi-index once
//            (magic-number division, no per-element div/mod) and its lanes stream the row, so
//            reads and writes are coalesced along a;
//   * tile : the unit-stride axes differ (a transpose); a 32x32 tile is staged in shared
//            memory so that reads are coalesced along the source axis and writes along the
//            destination axis.
// The kernel is persistent: a grid sized to the SM count walks a global tile index and finds its
// task by binary search in the per-task tile prefix sums.
#include <cstring>

#include "runtime.hpp"

namespace mpsg {

namespace {

constexpr int kRowTile = 2048;  // target elements per row-mode tile
constexpr int kT = 32;

// Per-task launch data: axis roles, tiling and division constants (q = (umulhi(n,m)+n) >> s
// equals n / ext for every n < 2^31).
struct TaskAux {
  int32_t mode, a, b, rows_per_tile;
  int64_t outer;                  // rows (row mode)
  uint32_t mag[kMaxTaskDims];
  uint32_t shf[kMaxTaskDims];
};

struct TaskView {
  int nd, a, b, mode, rpt;
  int64_t outer;
  int64_t ext[kMaxTaskDims], sstr[kMaxTaskDims], dstr[kMaxTaskDims];
  uint32_t mag[kMaxTaskDims], shf[kMaxTaskDims];
  int64_t soff, doff, first_tile;
};

__device__ __forceinline__ uint32_t fdiv(uint32_t n, uint32_t m, uint32_t s) {
  return (__umulhi(n, m) + n) >> s;
}

__global__ void __launch_bounds__(256) copy_tasks_kernel(
    const CopyTask* __restrict__ tasks, const int64_t* __restrict__ prefix,
    const TaskAux* __restrict__ aux, int ntasks, int64_t ntiles, const double* __restrict__ src,
    double* __restrict__ dst) {
  __shared__ double tile[kT][kT + 1];
  __shared__ TaskView tv;
  __shared__ int cur_task;
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const int warp = tid >> 5, lane = tid & 31;
  if (tid == 0) cur_task = -1;
  __syncthreads();
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    if (tid == 0) {
      int lo = 0, hi = ntasks - 1;  // largest k with prefix[k] <= t
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= t) lo = mid;
        else hi = mid - 1;
      }
      if (lo != cur_task) {
        const CopyTask& T = tasks[lo];
        const TaskAux& X = aux[lo];
        tv.nd = T.nd;
        for (int i = 0; i < T.nd; ++i) {
          tv.ext[i] = T.ext[i];
          tv.sstr[i] = T.sstr[i];
          tv.dstr[i] = T.dstr[i];
          tv.mag[i] = X.mag[i];
          tv.shf[i] = X.shf[i];
        }
        tv.soff = T.soff;
        tv.doff = T.doff;
        tv.mode = X.mode;
        tv.a = X.a;
        tv.b = X.b;
        tv.rpt = X.rows_per_tile;
        tv.outer = X.outer;
        tv.first_tile = prefix[lo];
        cur_task = lo;
      }
    }
    __syncthreads();
    const int64_t lt = t - tv.first_tile;
    const int nd = tv.nd;
    if (tv.mode == 0) {
      // row walk along axis a
      const int a = tv.a;
      const int64_t ea = tv.ext[a];
      const int64_t sa = tv.sstr[a], da = tv.dstr[a];
      const int64_t r0 = lt * tv.rpt;
      const int64_t r1 = min(r0 + tv.rpt, tv.outer);
      for (int64_t row = r0 + warp; row < r1; row += 8) {
        uint32_t q = (uint32_t)row;
        int64_t so = tv.soff, dof = tv.doff;
        for (int i = 0; i < nd; ++i) {
          if (i == a) continue;
          const uint32_t qi = fdiv(q, tv.mag[i], tv.shf[i]);
          const int64_t ii = (int64_t)(q - qi * (uint32_t)tv.ext[i]);
          q = qi;
          so += ii * tv.sstr[i];
          dof += ii * tv.dstr[i];
        }
        for (int64_t ia = lane; ia < ea; ia += 32) dst[dof + ia * da] = __ldg(src + so + ia * sa);
      }
    } else {
      const int a = tv.a, b = tv.b;
      const int64_t ea = tv.ext[a], eb = tv.ext[b];
      const int64_t ta = (ea + kT - 1) / kT, tb = (eb + kT - 1) / kT;
      int64_t q = lt;
      const int64_t ia = q % ta;
      q /= ta;
      const int64_t ib = q % tb;
      q /= tb;
      int64_t so = tv.soff, dof = tv.doff;
      uint32_t q32 = (uint32_t)q;
      for (int i = 0; i < nd; ++i) {
        if (i == a || i == b) continue;
        const uint32_t qi = fdiv(q32, tv.mag[i], tv.shf[i]);
        const int64_t ii = (int64_t)(q32 - qi * (uint32_t)tv.ext[i]);
        q32 = qi;
        so += ii * tv.sstr[i];
        dof += ii * tv.dstr[i];
      }
      const int64_t a0 = ia * kT, b0 = ib * kT;
      const int tx = threadIdx.x, ty = threadIdx.y;
      for (int j = ty; j < kT; j += 8) {
        if (a0 + j < ea && b0 + tx < eb)
          tile[j][tx] = __ldg(src + so + (a0 + j) * tv.sstr[a] + (b0 + tx) * tv.sstr[b]);
      }
      __syncthreads();
      for (int j = ty; j < kT; j += 8) {
        if (a0 + tx < ea && b0 + j < eb)
          dst[dof + (a0 + tx) * tv.dstr[a] + (b0 + j) * tv.dstr[b]] = tile[tx][j];
      }
    }
    __syncthreads();
  }
}

void magic_u31(uint32_t d, uint32_t& m, uint32_t& s) {
  uint32_t l = 0;
  while (((uint64_t)1 << l) < d) ++l;
  m = (uint32_t)((((uint64_t)1 << 32) * (((uint64_t)1 << l) - d)) / d + 1);
  s = l;
}

}  // namespace

size_t copy_aux_bytes() { return sizeof(TaskAux); }

void DevCopyPlan::upload(const std::vector<CopyTask>& tasks, bool identity_) {
  release();
  std::vector<int64_t> prefix;
  std::vector<unsigned char> aux;
  build_host(tasks, identity_, prefix, aux);
  if (ntasks == 0) return;
  MPSG_CUDA(cudaMalloc(&d_tasks, sizeof(CopyTask) * ntasks));
  MPSG_CUDA(cudaMalloc(&d_prefix, sizeof(int64_t) * (ntasks + 1)));
  MPSG_CUDA(cudaMalloc(&d_aux, aux.size()));
  MPSG_CUDA(cudaMemcpy(d_tasks, tasks.data(), sizeof(CopyTask) * ntasks, cudaMemcpyHostToDevice));
  MPSG_CUDA(cudaMemcpy(d_prefix, prefix.data(), sizeof(int64_t) * (ntasks + 1),
                       cudaMemcpyHostToDevice));
  MPSG_CUDA(cudaMemcpy(d_aux, aux.data(), aux.size(), cudaMemcpyHostToDevice));
}

void DevCopyPlan::build_host(const std::vector<CopyTask>& tasks, bool identity_,
                             std::vector<int64_t>& prefix, std::vector<unsigned char>& aux_bytes) {
  identity = identity_;
  ntasks = (int)tasks.size();
  prefix.assign(ntasks + 1, 0);
  std::vector<TaskAux> aux(ntasks);
  elems = 0;
  for (int k = 0; k < ntasks; ++k) {
    const CopyTask& T = tasks[k];
    int a = 0, b = 0;
    for (int i = 1; i < T.nd; ++i) {
      if (T.dstr[i] < T.dstr[a]) a = i;
      if (T.sstr[i] < T.sstr[b]) b = i;
    }
    const int64_t n = T.numel();
    if (n >= ((int64_t)1 << 31)) throw Error(kErrUnsupported, "copy task above 2^31 elements");
    elems += n;
    TaskAux& X = aux[k];
    for (int i = 0; i < T.nd; ++i) magic_u31((uint32_t)T.ext[i], X.mag[i], X.shf[i]);
    int64_t tiles;
    if (a == b || T.nd == 1 || T.sstr[b] != 1 || T.dstr[a] != 1) {
      X.mode = 0;
      X.outer = n / T.ext[a];
      X.rows_per_tile = (int)std::max<int64_t>(1, std::min<int64_t>(X.outer, kRowTile / T.ext[a]));
      tiles = (X.outer + X.rows_per_tile - 1) / X.rows_per_tile;
    } else {
      X.mode = 1;
      X.outer = 0;
      X.rows_per_tile = 0;
      int64_t rest = n / (T.ext[a] * T.ext[b]);
      tiles = ((T.ext[a] + kT - 1) / kT) * ((T.ext[b] + kT - 1) / kT) * rest;
    }
    X.a = a;
    X.b = b;
    prefix[k + 1] = prefix[k] + tiles;
  }
  ntiles = prefix[ntasks];
  aux_bytes.resize(sizeof(TaskAux) * ntasks);
  if (ntasks) std::memcpy(aux_bytes.data(), aux.data(), aux_bytes.size());
}

void DevCopyPlan::release() {
  if (d_tasks) cudaFree(d_tasks);
  if (d_prefix) cudaFree(d_prefix);
  if (d_aux) cudaFree(d_aux);
  d_tasks = nullptr;
  d_prefix = nullptr;
  d_aux = nullptr;
  ntasks = 0;
  ntiles = 0;
}

void launch_copy(Context* ctx, const DevCopyPlan& p, const double* src, double* dst) {
  if (p.ntiles == 0) return;
  if (p.identity) {
    if (src != dst)
      MPSG_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * p.elems, cudaMemcpyDeviceToDevice,
                                ctx->stream));
    return;
  }
  int64_t grid = std::min<int64_t>(p.ntiles, (int64_t)ctx->num_sms * 8);
  KernelTimer timer(ctx, kKindCopy);
  copy_tasks_kernel<<<(unsigned)grid, dim3(32, 8), 0, ctx->stream>>>(
      p.d_tasks, p.d_prefix, (const TaskAux*)p.d_aux, p.ntasks, p.ntiles, src, dst);
  MPSG_CUDA(cudaGetLastError());
  ctx->kernel_launches++;
}

}  // namespace mpsg
