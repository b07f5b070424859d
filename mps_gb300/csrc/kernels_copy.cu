// Block-permute engine: executes a list of strided N-d copy tasks (permutelegs, fuselegs,
// splitleg, SymMatrix fusion and the split+permute of contraction outputs are all such lists).
//
// Two tile shapes, chosen per task on the host:
//   * flat  : source and destination share their unit-stride axis (or one side has none);
//             the task is walked in destination order, 2048 elements per tile, so writes and
//             reads are both coalesced along that axis;
//   * tile  : the unit-stride axes differ (a transpose); a 32x32 tile is staged in shared
//             memory so that reads are coalesced along the source axis and writes along the
//             destination axis.
// The kernel is persistent: a grid sized to the SM count walks a global tile index and finds its
// task by binary search in the per-task tile prefix sums.
#include "runtime.hpp"

namespace mpsg {

namespace {

constexpr int kFlatTile = 2048;
constexpr int kT = 32;

struct TaskView {
  int nd;
  int a, b, mode;
  int64_t ext[kMaxTaskDims], sstr[kMaxTaskDims], dstr[kMaxTaskDims];
  int64_t soff, doff, first_tile;
};

__global__ void __launch_bounds__(256) copy_tasks_kernel(
    const CopyTask* __restrict__ tasks, const int64_t* __restrict__ prefix,
    const int32_t* __restrict__ modes, int ntasks, int64_t ntiles,
    const double* __restrict__ src, double* __restrict__ dst) {
  __shared__ double tile[kT][kT + 1];
  __shared__ TaskView tv;
  __shared__ int cur_task;
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
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
        tv.nd = T.nd;
        for (int i = 0; i < T.nd; ++i) {
          tv.ext[i] = T.ext[i];
          tv.sstr[i] = T.sstr[i];
          tv.dstr[i] = T.dstr[i];
        }
        tv.soff = T.soff;
        tv.doff = T.doff;
        int32_t m = modes[lo];
        tv.mode = m & 0xff;
        tv.a = (m >> 8) & 0xff;
        tv.b = (m >> 16) & 0xff;
        tv.first_tile = prefix[lo];
        cur_task = lo;
      }
    }
    __syncthreads();
    const int64_t lt = t - tv.first_tile;
    const int nd = tv.nd;
    if (tv.mode == 0) {
      // flat walk, axis a innermost
      const int a = tv.a;
      int64_t total = 1;
      for (int i = 0; i < nd; ++i) total *= tv.ext[i];
      const int64_t base = lt * kFlatTile;
      for (int e = tid; e < kFlatTile; e += 256) {
        int64_t f = base + e;
        if (f >= total) break;
        int64_t q = f / tv.ext[a];
        int64_t ia = f - q * tv.ext[a];
        int64_t so = tv.soff + ia * tv.sstr[a], dof = tv.doff + ia * tv.dstr[a];
        for (int i = 0; i < nd; ++i) {
          if (i == a) continue;
          int64_t qi = q / tv.ext[i];
          int64_t ii = q - qi * tv.ext[i];
          q = qi;
          so += ii * tv.sstr[i];
          dof += ii * tv.dstr[i];
        }
        dst[dof] = __ldg(src + so);
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
      for (int i = 0; i < nd; ++i) {
        if (i == a || i == b) continue;
        int64_t qi = q / tv.ext[i];
        int64_t ii = q - qi * tv.ext[i];
        q = qi;
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

}  // namespace

void DevCopyPlan::upload(const std::vector<CopyTask>& tasks, bool identity_) {
  release();
  identity = identity_;
  ntasks = (int)tasks.size();
  std::vector<int64_t> prefix(ntasks + 1, 0);
  std::vector<int32_t> modes(ntasks, 0);
  elems = 0;
  for (int k = 0; k < ntasks; ++k) {
    const CopyTask& T = tasks[k];
    int a = 0, b = 0;
    for (int i = 1; i < T.nd; ++i) {
      if (T.dstr[i] < T.dstr[a]) a = i;
      if (T.sstr[i] < T.sstr[b]) b = i;
    }
    int64_t n = T.numel();
    elems += n;
    int64_t tiles;
    int mode;
    if (a == b || T.nd == 1 || T.sstr[b] != 1 || T.dstr[a] != 1) {
      mode = 0;
      tiles = (n + kFlatTile - 1) / kFlatTile;
    } else {
      mode = 1;
      int64_t rest = n / (T.ext[a] * T.ext[b]);
      tiles = ((T.ext[a] + kT - 1) / kT) * ((T.ext[b] + kT - 1) / kT) * rest;
    }
    modes[k] = mode | (a << 8) | (b << 16);
    prefix[k + 1] = prefix[k] + tiles;
  }
  ntiles = prefix[ntasks];
  if (ntasks == 0) return;
  MPSG_CUDA(cudaMalloc(&d_tasks, sizeof(CopyTask) * ntasks));
  MPSG_CUDA(cudaMalloc(&d_prefix, sizeof(int64_t) * (ntasks + 1)));
  MPSG_CUDA(cudaMalloc(&d_mode, sizeof(int32_t) * ntasks));
  MPSG_CUDA(cudaMemcpy(d_tasks, tasks.data(), sizeof(CopyTask) * ntasks, cudaMemcpyHostToDevice));
  MPSG_CUDA(cudaMemcpy(d_prefix, prefix.data(), sizeof(int64_t) * (ntasks + 1),
                       cudaMemcpyHostToDevice));
  MPSG_CUDA(cudaMemcpy(d_mode, modes.data(), sizeof(int32_t) * ntasks, cudaMemcpyHostToDevice));
}

void DevCopyPlan::release() {
  if (d_tasks) cudaFree(d_tasks);
  if (d_prefix) cudaFree(d_prefix);
  if (d_mode) cudaFree(d_mode);
  d_tasks = nullptr;
  d_prefix = nullptr;
  d_mode = nullptr;
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
      p.d_tasks, p.d_prefix, p.d_mode, p.ntasks, p.ntiles, src, dst);
  MPSG_CUDA(cudaGetLastError());
  ctx->kernel_launches++;
}

}  // namespace mpsg
