// contract() without any device allocation: mpsg_contract_noalloc.
//
// Some callers cannot let the library allocate device memory during a call: a host application
// that hands the GPU's memory to its own pool allocator up front (a Julia or C++ code that
// already manages a fixed arena), or one that must keep allocation out of a latency-critical
// loop. mpsg_contract computes the same FP64 contraction but allocates its fused operands, the
// GEMM output and its cached task tables with cudaMallocAsync/cudaMalloc. This variant instead
// takes the output tensor from the caller and keeps every temporary in one fixed device array
// of kScratchBytes (64 MiB), declared below at file scope. That array exists on every GPU that
// loads the library and stays there until the process exits.
//
// Set-up: the first call on a device looks up the array's address with cudaGetSymbolAddress
// (with that device current) and remembers it; later calls on that device reuse it. Make that
// first call before any stream capture begins.
//
// Sharing: all calls on a device use the same array and leave their contents in it. Two calls
// whose kernels overlap on the GPU (different streams without ordering, or different contexts
// on one device) race on it; calls issued on one context's stream are ordered and safe. Nothing
// here accumulates into scratch: the task tables are written by a host-to-device copy and the
// fused operands and the GEMM output are fully rewritten by the copy and GEMM kernels of each
// call, so no part of the array needs clearing between calls.
//
// Cost: every call plans the contraction on the host, rebuilds its task tables and waits for the
// context's stream before it returns (the tables are staged from host memory owned by the call).
// mpsg_contract caches both and returns without waiting, so in a loop this variant pays the
// host planning and one stream synchronisation per call.
#include <cstring>
#include <mutex>

#include "capi_internal.hpp"

namespace {

constexpr size_t kScratchBytes = size_t(64) << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_mu;
unsigned char* g_base[kMaxDevices] = {nullptr};

// Address of g_scratch on `device`, looked up once per device with that device current.
unsigned char* scratch_base(int device) {
  if (device < 0 || device >= kMaxDevices)
    throw mpsg::Error(mpsg::kErrArgument, "device ordinal out of range for the scratch table");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_base[device]) {
    int prev = -1;
    MPSG_CUDA(cudaGetDevice(&prev));
    if (prev != device) MPSG_CUDA(cudaSetDevice(device));
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (prev != device) cudaSetDevice(prev);
    if (e != cudaSuccess)
      throw mpsg::Error(mpsg::kErrCuda,
                        std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_base[device] = (unsigned char*)p;
  }
  return g_base[device];
}

size_t align256(size_t n) { return (n + 255) & ~size_t(255); }

// Places the tables of one copy plan (warp-unit tasks, their prefix sums and launch data, and
// the rows of the TMA-staged path) in the staging image at `cur` and points the plan there.
void stage_copy(mpsg::DevCopyPlan& p, const std::vector<mpsg::CopyTask>& tasks, bool identity,
                std::vector<unsigned char>& img, size_t& cur, unsigned char* dev) {
  std::vector<mpsg::CopyTask> rest;
  std::vector<int64_t> prefix;
  std::vector<unsigned char> aux;
  std::vector<mpsg::BulkRow> rows;
  p.build_host(tasks, identity, rest, prefix, aux, rows);
  if (p.identity) return;
  const size_t bt = sizeof(mpsg::CopyTask) * rest.size();
  const size_t bp = sizeof(int64_t) * prefix.size();
  const size_t br = sizeof(mpsg::BulkRow) * rows.size();
  const size_t o1 = cur, o2 = align256(o1 + bt), o3 = align256(o2 + bp),
               o4 = align256(o3 + aux.size());
  cur = align256(o4 + br);
  if (cur > kScratchBytes) return;  // reported by the caller's size check
  img.resize(cur);
  if (bt) std::memcpy(img.data() + o1, rest.data(), bt);
  std::memcpy(img.data() + o2, prefix.data(), bp);
  if (!aux.empty()) std::memcpy(img.data() + o3, aux.data(), aux.size());
  if (br) std::memcpy(img.data() + o4, rows.data(), br);
  p.d_tasks = (mpsg::CopyTask*)(dev + o1);
  p.d_prefix = (int64_t*)(dev + o2);
  p.d_aux = dev + o3;
  p.d_rows = (mpsg::BulkRow*)(dev + o4);
}

bool same_structure(const mpsg::TensorMeta& x, const mpsg::TensorMeta& y) {
  if (x.charge != y.charge || x.space.size() != y.space.size()) return false;
  for (size_t i = 0; i < x.space.size(); ++i)
    if (!(x.space[i] == y.space[i])) return false;
  return true;
}

}  // namespace

extern "C" int mpsg_contract_noalloc(mpsg_ctx* ctx, const mpsg_tensor* a, const int32_t* idxa,
                                     const mpsg_tensor* b, const int32_t* idxb,
                                     mpsg_tensor* out) {
  using namespace mpsg;
  return mpsg_capi::guarded([&] {
    mpsg_capi::need(ctx, "ctx");
    mpsg_capi::need(a, "a");
    mpsg_capi::need(b, "b");
    mpsg_capi::need(idxa, "idxa");
    mpsg_capi::need(idxb, "idxb");
    mpsg_capi::need(out, "out");
    Context* c = &ctx->c;
    // a tensor of another context may live on another device: its pointer would be written
    // by this device's kernels
    if (a->t.ctx != c || b->t.ctx != c || out->t.ctx != c)
      throw Error(kErrArgument, "mpsg_contract_noalloc: a, b and out must belong to ctx");
    unsigned char* dev = scratch_base(c->device);
    auto plan = plan_contract(a->t.meta, mpsg_capi::ivec(idxa, a->t.meta.N()), b->t.meta,
                              mpsg_capi::ivec(idxb, b->t.meta.N()));
    if (plan->scalar)
      throw Error(kErrUnsupported,
                  "mpsg_contract_noalloc: every leg is contracted (scalar result); use "
                  "mpsg_contract");
    if (out->t.diag || !same_structure(out->t.meta, plan->split.out))
      throw Error(kErrSpaceMismatch,
                  "mpsg_contract_noalloc: out does not have the charge and spaces of the result");
    double* dout = out->t.data();
    if (plan->split.out.total > 0 && (!dout || dout == a->t.data() || dout == b->t.data()))
      throw Error(kErrArgument, "mpsg_contract_noalloc: out must own storage distinct from a, b");

    // task tables first, then the fused operands and the GEMM output, each 256-byte aligned
    std::vector<unsigned char> img;
    size_t cur = 0;
    DevCopyPlan fa, fb, split;
    DevGemmPlan mm;
    stage_copy(fa, plan->fa.tasks, plan->fa.identity, img, cur, dev);
    stage_copy(fb, plan->fb.tasks, plan->fb.identity, img, cur, dev);
    stage_copy(split, plan->split.tasks, plan->split.identity, img, cur, dev);
    GemmTables gt;
    mm.build_host(plan->mm.gemms, plan->mm.flops, gt);
    for (int q = 0; q < 3; ++q) {  // tiled, thin-N and thin-M task tables
      if (mm.count[q] == 0) continue;
      const size_t bt = sizeof(GemmTask) * mm.count[q], bp = sizeof(int64_t) * gt.prefix[q].size();
      const size_t o1 = cur, o2 = align256(o1 + bt);
      cur = align256(o2 + bp);
      if (cur > kScratchBytes) continue;  // reported by the size check below
      img.resize(cur);
      std::memcpy(img.data() + o1, gt.part[q].data(), bt);
      std::memcpy(img.data() + o2, gt.prefix[q].data(), bp);
      mm.d_part[q] = (GemmTask*)(dev + o1);
      mm.d_part_prefix[q] = (int64_t*)(dev + o2);
    }
    mm.d_tasks = mm.d_part[kTiled];
    mm.d_prefix = mm.d_part_prefix[kTiled];
    const size_t tables = cur;
    auto take = [&](int64_t doubles) {
      const size_t o = cur;
      cur = align256(cur + sizeof(double) * (size_t)doubles);
      return (double*)(dev + o);
    };
    const double* pa = a->t.data();
    const double* pb = b->t.data();
    double* fused_a = plan->fa.identity ? nullptr : take(plan->fa.out.total);
    double* fused_b = plan->fb.identity ? nullptr : take(plan->fb.out.total);
    double* cmat = plan->split.identity ? dout : take(plan->mm.out.total);
    if (cur > kScratchBytes)
      throw Error(kErrUnsupported,
                  "mpsg_contract_noalloc: this contraction needs " + std::to_string(cur) +
                      " bytes of scratch, more than the fixed " + std::to_string(kScratchBytes) +
                      " bytes (64 MiB); use mpsg_contract for it");

    if (tables > 0)
      MPSG_CUDA(cudaMemcpyAsync(dev, img.data(), tables, cudaMemcpyHostToDevice, c->stream));
    if (fused_a) {
      launch_copy(c, fa, pa, fused_a);
      pa = fused_a;
    }
    if (fused_b) {
      launch_copy(c, fb, pb, fused_b);
      pb = fused_b;
    }
    launch_gemm_f64(c, mm, pa, pb, cmat);
    if (!plan->split.identity) launch_copy(c, split, cmat, dout);
    // the staging image is host memory owned by this frame: wait until the copy has read it
    MPSG_CUDA(cudaStreamSynchronize(c->stream));
  });
}
