// Device runtime: context (device, stream, plan cache), device tensors and the launchers of the
// CUDA kernels.  Everything here is called from the C ABI in capi.cu.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <atomic>
#include <list>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "copy_decode.hpp"
#include "planner.hpp"

namespace mpsg {

#define MPSG_CUDA(call)                                                                     \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      throw ::mpsg::Error(::mpsg::kErrCuda, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

struct Context;
struct HeffPlans;
namespace split {
struct SplitPlan;
}

// Stream-ordered device allocation.  Every buffer co-owns its context, so the context (stream,
// caches) outlives the last tensor whatever order a caller releases handles in.
struct Buffer {
  std::shared_ptr<Context> owner;
  double* ptr = nullptr;
  int64_t n = 0;
  ~Buffer();
};
std::shared_ptr<Buffer> alloc_buffer(Context* ctx, int64_t n);

struct DeviceTensor {
  Context* ctx = nullptr;
  TensorMeta meta;
  std::shared_ptr<Buffer> buf;  // shared by views (dual) of the same data
  bool diag = false;            // singular values stored as dense diagonal blocks
  double* data() const { return buf ? buf->ptr : nullptr; }
};

// Copy-task list on the device, in one of two forms. When nearly all elements sit in tasks
// whose source and destination share a unit-stride axis of at least kBulkMinRow elements, every
// task becomes rows of a table moved by the TMA-staged row kernel (the few other tasks as
// strided rows along their destination's fastest axis). Otherwise every task keeps its unit
// prefix sums and launch data for the warp-unit kernel.
constexpr int kBulkMinRow = 32;    // shortest unit-stride row that counts as bulk (elements)
constexpr int kBulkMaxRow = 512;   // longest row unit of the row kernel (elements)
struct DevCopyPlan {
  int ntasks = 0;                // tasks of the warp-unit kernel
  int64_t ntiles = 0;            // ... and their units
  int64_t nrows = 0;             // rows of the TMA-staged kernel
  int64_t elems = 0;
  bool identity = false;
  bool has_tile = false;         // some task is a transpose staged through shared memory
  CopyTask* d_tasks = nullptr;
  int64_t* d_prefix = nullptr;   // ntasks+1 tile prefix
  void* d_aux = nullptr;         // per task: tile shape, axis roles, division constants
  BulkRow* d_rows = nullptr;     // nrows rows of the TMA-staged path
  cudaStream_t stream = nullptr;  // tables are allocated and freed in this stream's order
  void upload(const std::vector<CopyTask>& tasks, bool identity_, cudaStream_t st);
  // Host half of upload: either the row table (`rows`, `rest` empty) or the warp-unit tasks
  // (`rest` with their unit prefix sums and launch data); sets every field except the device
  // pointers (used by callers that place the tables in memory they own).
  void build_host(const std::vector<CopyTask>& tasks, bool identity_, std::vector<CopyTask>& rest,
                  std::vector<int64_t>& prefix, std::vector<unsigned char>& aux_bytes,
                  std::vector<BulkRow>& rows);
  void release();
};
size_t copy_aux_bytes();  // bytes of launch data per copy task
// Device-checked build only (MPSG_DEVICE_CHECKS): violations recorded by the copy kernel since
// the last reset, and the first one (kind, task, index, detail); kErrUnsupported otherwise.
void read_device_checks(Context* ctx, bool reset, int64_t* count, int64_t* first);

// FP64 GEMM tasks split by shape: tiled (64 x 64 tiles), thin-N (one thread per output row) and
// thin-M (one thread per output column), each with its work-unit prefix sums.
enum GemmPart { kTiled = 0, kRows = 1, kCols = 2 };
struct GemmTables {
  std::vector<GemmTask> part[3];
  std::vector<int64_t> prefix[3];
};

struct DevGemmPlan {
  int n = 0;          // tiled tasks
  int64_t ntiles = 0;
  double flops = 0;
  GemmTask* d_tasks = nullptr;   // = d_part[kTiled]
  int64_t* d_prefix = nullptr;   // = d_part_prefix[kTiled]
  int count[3] = {0, 0, 0};      // tasks per part
  int64_t units[3] = {0, 0, 0};  // work units per part (tiles, rows, columns)
  GemmTask* d_part[3] = {nullptr, nullptr, nullptr};
  int64_t* d_part_prefix[3] = {nullptr, nullptr, nullptr};
  std::vector<GemmTask> host;
  std::shared_ptr<split::SplitPlan> splitp[8];  // split-precision plans by slice count
  cudaStream_t stream = nullptr;  // tables are allocated and freed in this stream's order
  size_t device_bytes() const;    // packed-slice scratch of the split plans (the bulk)
  void upload(const std::vector<GemmTask>& g, double flops_, cudaStream_t st);
  // Host half of upload: every field except the device pointers, plus the per-part tables.
  void build_host(const std::vector<GemmTask>& g, double flops_, GemmTables& t);
  void release();
};

struct DevContract {
  std::shared_ptr<ContractPlan> host;
  DevCopyPlan fa, fb, split;
  DevGemmPlan mm;
  size_t device_bytes() const { return mm.device_bytes(); }
  ~DevContract();
};

// Live contexts of the process: the plan-cache budgets below are shares of a per-process total,
// so many concurrent contexts (independent chains) together stay within the device memory.
extern std::atomic<int> g_live_contexts;
inline size_t cache_share(size_t total) {
  const int n = g_live_contexts.load();
  return total / (size_t)(n > 1 ? n : 1);
}

// Plans by structure key, least recently used first, trimmed to a device-byte budget (split
// plans carry packed operand scratch as large as their operands, and a sweep meets a new
// structure at every bond). Entries are shared: evicting one that a caller still holds only
// drops the cache's reference.
template <class T>
struct PlanCache {
  size_t total_budget = size_t(16) << 30;  // per process, shared by the live contexts
  std::list<std::string> order;
  std::unordered_map<std::string, std::pair<std::shared_ptr<T>, std::list<std::string>::iterator>>
      map;
  std::shared_ptr<T> get(const std::string& k) {
    auto it = map.find(k);
    if (it == map.end()) return nullptr;
    order.splice(order.end(), order, it->second.second);
    return it->second.first;
  }
  void put(const std::string& k, std::shared_ptr<T> v) {
    order.push_back(k);
    map[k] = {std::move(v), std::prev(order.end())};
    trim();
  }
  // evict least recently used entries (never the most recent one) while over budget
  void trim() {
    size_t total = 0;
    for (const auto& e : map) total += e.second.first->device_bytes();
    const size_t budget = cache_share(total_budget);
    while (total > budget && order.size() > 1) {
      auto it = map.find(order.front());
      total -= it->second.first->device_bytes();
      map.erase(it);
      order.pop_front();
    }
  }
  void clear() {
    map.clear();
    order.clear();
  }
};

struct DevReleg {
  RelegPlan host;
  DevCopyPlan cp;
  ~DevReleg();
};

struct Context : std::enable_shared_from_this<Context> {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  double* d_partials = nullptr;   // reduction partials (one per CTA of a reduction launch)
  int* d_copy_err = nullptr;      // set by the TMA-staged copy kernel when a bounded wait expires
  // small pinned host scratch: [0, 64) scalar results, [64, 64 + 3 * 128) the batched Lanczos
  static constexpr int kPinnedDoubles = 64 + 3 * 128;
  double* h_pinned = nullptr;
  PlanCache<DevContract> contract_cache;
  std::unordered_map<std::string, std::shared_ptr<DevReleg>> releg_cache;
  PlanCache<DevGemmPlan> matmul_cache;
  // idle prepared-H_eff plans by structure + precision, least recently returned first
  std::unordered_map<std::string, std::shared_ptr<HeffPlans>> heff_cache;
  std::vector<std::string> heff_lru;
  size_t heff_bytes = 0;
  cudaStream_t copy_stream = nullptr;   // host<->device transfers overlapped with compute
  cudaEvent_t copy_ev[4] = {};          // ... and the events that order them
  bool counted = false;           // included in g_live_contexts
  int64_t kernel_launches = 0;    // launches of this library's kernels
  bool debug_sync = false;        // MPSG_DEBUG_SYNC=1: synchronise and check after tensor-core GEMMs
  double gemm_flops = 0;          // algorithmic flops issued through block GEMMs
  // split-GEMM tuner (batch.cu): when on, a new shape class of problem lists is timed over the
  // kernel's N tiles and tile orders and the fastest (N tile, order) kept by class
  bool autotune = false;
  std::unordered_map<std::string, std::array<int, 3>> tune_cache;  // (N tile, order, split-K)
  int64_t tune_runs = 0, tune_hits = 0;
  int forced_bn = -1, forced_order = -1, forced_splitk = 0;  // mpsg_ctx_set_split_tuning
  void* solver = nullptr;         // cusolverDnHandle_t, created on first SVD
  void (*solver_destroy)(void*) = nullptr;
  // optional per-kernel-class event timing (see mpsg_ctx_set_timing)
  static constexpr int kKinds = 6;
  bool timing = false;
  struct TimedLaunch {
    cudaEvent_t a, b;
    double flops;
  };
  std::vector<TimedLaunch> events[kKinds];
  std::vector<cudaEvent_t> event_pool;
  double timed_ms[kKinds] = {0, 0, 0, 0, 0, 0};
  int64_t timed_launches[kKinds] = {0, 0, 0, 0, 0, 0};
  double timed_flops[kKinds] = {0, 0, 0, 0, 0, 0};
  ~Context();
};

enum KernelKind {
  kKindCopy = 0,
  kKindGemmF64 = 1,
  kKindGemmSplit = 2,
  kKindPack = 3,       // split operand packing: exponent pass
  kKindVec = 4,
  kKindPackSlices = 5  // split operand packing: slice pass
};

// RAII bracket of one launch with events when timing is enabled.
struct KernelTimer {
  Context* ctx;
  int kind;
  double flops;
  cudaEvent_t a = nullptr, b = nullptr;
  KernelTimer(Context* c, int k, double f = 0.0);
  ~KernelTimer();
};
void collect_kernel_times(Context* ctx);

// Raises a kernel's dynamic shared-memory limit on the context's device.  A function attribute
// belongs to one device's context, so it is set once per device: ``flags`` is the caller's
// per-kernel array of once-flags, indexed by device ordinal.  Thread-safe; a failed attempt
// throws and is retried on the next launch.
constexpr int kMaxDevices = 64;
template <class Kernel>
void set_smem_limit_once(Context* ctx, std::once_flag (&flags)[kMaxDevices], Kernel kernel,
                         int bytes) {
  if (ctx->device < 0 || ctx->device >= kMaxDevices)
    throw Error(kErrArgument, "device ordinal out of range");
  std::call_once(flags[ctx->device], [&] {
    int cur = -1;
    MPSG_CUDA(cudaGetDevice(&cur));
    if (cur != ctx->device) MPSG_CUDA(cudaSetDevice(ctx->device));
    const cudaError_t e =
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (cur != ctx->device) cudaSetDevice(cur);
    if (e != cudaSuccess)
      throw Error(kErrCuda, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
  });
}

// ---- kernel launchers (kernels_*.cu) ----
void launch_copy(Context* ctx, const DevCopyPlan& p, const double* src, double* dst);
// Error code of the TMA-staged copy kernel since the last call (0 = none), then cleared;
// synchronises the context's stream.
int read_copy_error(Context* ctx);
void launch_gemm_f64(Context* ctx, const DevGemmPlan& p, const double* A, const double* B,
                     double* C);
void launch_fill(Context* ctx, double* x, int64_t n, double v);
void launch_axpby(Context* ctx, int64_t n, double a, const double* x, double b, double* y);
void launch_scale(Context* ctx, int64_t n, double a, const double* x, double* y);
// sum_i x_i*y_i into *out (device), deterministic two-pass reduction
void launch_dot(Context* ctx, int64_t n, const double* x, const double* y, double* d_out);
// Many dot products in one pair of launches; writes the host array out and synchronises.
struct VecPair {
  const double* x;
  const double* y;
  int64_t n;
};
void dots_host(Context* ctx, const std::vector<VecPair>& pairs, double* out);
// y = sum_i c[i] xs[i] (elementwise, n elements; y may alias an operand)
void launch_lincomb(Context* ctx, int64_t n, const std::vector<const double*>& xs,
                    const std::vector<double>& c, double* y);
// The same two operations with every table in device memory and no host synchronisation:
// d_out[i] = dot(pairs[i]) (d_part holds np * dots_grid(ctx, nmax) partial sums, nmax = the
// longest pair), and y = sum_i d_c[i] d_xs[i] over m operands.
int dots_grid(Context* ctx, int64_t nmax);
void launch_dots_device(Context* ctx, const VecPair* d_pairs, int np, int64_t nmax,
                        double* d_part, double* d_out);
void launch_lincomb_device(Context* ctx, int64_t n, int m, const double* const* d_xs,
                           const double* d_c, double* y);

}  // namespace mpsg
