// Many prepared two-site H_eff applied as one (independent DMRG chains on one GPU), the
// lock-step Lanczos over them, and the split-GEMM tuner.  The reference runs one chain per
// process (src/dmrg.jl:58-179, KrylovKit eigsolve at dmrg.jl:77-82); the batched form has no
// counterpart there.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <tuple>

#include "batch.hpp"
#include "small_eigh.cuh"

namespace mpsg {

// ------------------------------------------------------------------------------------------
// tuner
// ------------------------------------------------------------------------------------------
namespace {

int log2_ceil(int64_t x) {
  int b = 0;
  while (b < 62 && (int64_t(1) << b) < x) ++b;
  return b;
}

// Extents of the FP64 operands a task list reads and writes (column-major windows).
void operand_extents(const std::vector<GemmTask>& g, int64_t& na, int64_t& nb, int64_t& nc) {
  na = nb = nc = 1;
  for (const GemmTask& t : g) {
    if (t.M > 0 && t.K > 0) na = std::max(na, t.offA + t.lda * (t.K - 1) + t.M);
    if (t.K > 0 && t.N > 0) nb = std::max(nb, t.offB + t.ldb * (t.N - 1) + t.K);
    if (t.M > 0 && t.N > 0) nc = std::max(nc, t.offC + t.ldc * (t.N - 1) + t.M);
  }
}

}  // namespace

std::string tune_shape_class(const std::vector<GemmTask>& g, int S) {
  // what the configuration choice depends on: the slice count, how many waves of 128 x 128
  // output tiles the problems give a GB300 (factor-2 buckets) and how long their K loops are
  // (tile-weighted mean K, factor-2 buckets)
  double tiles = 0, ktiles = 0;
  for (const GemmTask& t : g) {
    if (t.M <= 0 || t.N <= 0) continue;
    const double nt = (double)((t.M + 127) / 128) * (double)((t.N + 127) / 128);
    tiles += nt;
    ktiles += nt * (double)t.K;
  }
  const int waves = log2_ceil((int64_t)(1 + 4.0 * tiles / 152.0));
  const int kb = log2_ceil((int64_t)(1 + (tiles > 0 ? ktiles / tiles : 0.0)));
  return "S" + std::to_string(S) + "|w" + std::to_string(waves) + "|k" + std::to_string(kb);
}

split::Tuning tune_split(Context* ctx, const std::vector<GemmTask>& g, int S) {
  std::vector<split::Tuning> cands;
  std::vector<int> bns = {split::exact_bn(S)};
  if (split::exact_bn(S) != 64) bns.push_back(64);
  for (int bn : bns)
    for (int order : {split::kOrderK, split::kOrderProblem})
      for (int sk : {0, 1}) cands.push_back({bn, order, sk});
  int64_t na, nb, nc;
  operand_extents(g, na, nb, nc);
  // operand values do not change the kernels' work: ones
  auto A = alloc_buffer(ctx, na), B = alloc_buffer(ctx, nb), C = alloc_buffer(ctx, nc);
  launch_fill(ctx, A->ptr, na, 1.0);
  launch_fill(ctx, B->ptr, nb, 1.0);
  cudaEvent_t e0, e1;
  MPSG_CUDA(cudaEventCreate(&e0));
  MPSG_CUDA(cudaEventCreate(&e1));
  split::Tuning best;
  float best_ms = 1e30f;
  try {
    for (const split::Tuning& t : cands) {
      split::SplitPlan sp;
      sp.build(ctx, g, S, t);
      // the fast kernel has one tile shape and no split-K: only the order is a choice; a
      // split-K candidate that splits nothing is the candidate without it
      if (sp.fast && (t.bn != bns[0] || t.splitk)) continue;
      if (t.splitk && sp.nsplit == 0) continue;
      split::launch_split_gemm(ctx, sp, A->ptr, B->ptr, C->ptr, split::kAll);  // warm-up
      constexpr int kReps = 2;
      MPSG_CUDA(cudaEventRecord(e0, ctx->stream));
      for (int r = 0; r < kReps; ++r)
        split::launch_split_gemm(ctx, sp, nullptr, nullptr, C->ptr, split::kRunGemm);
      MPSG_CUDA(cudaEventRecord(e1, ctx->stream));
      MPSG_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      MPSG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best_ms) {
        best_ms = ms;
        best = t;
      }
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->tune_runs++;
  return best;
}

split::Tuning choose_tuning(Context* ctx, const std::vector<GemmTask>& g, int S) {
  if (ctx->forced_bn >= 0) {  // a configuration fixed by the caller
    split::Tuning t;
    t.bn = (ctx->forced_bn == 64 || ctx->forced_bn == split::exact_bn(S)) ? ctx->forced_bn : 0;
    t.order = ctx->forced_order;
    t.splitk = ctx->forced_splitk;
    return t;
  }
  if (!ctx->autotune || g.empty()) return split::Tuning();
  const std::string key = tune_shape_class(g, S);
  auto it = ctx->tune_cache.find(key);
  if (it != ctx->tune_cache.end()) {
    ctx->tune_hits++;
    split::Tuning t;
    t.bn = it->second[0];
    t.order = it->second[1];
    t.splitk = it->second[2];
    return t;
  }
  const split::Tuning t = tune_split(ctx, g, S);
  ctx->tune_cache[key] = {t.bn, t.order, t.splitk};
  return t;
}

// ------------------------------------------------------------------------------------------
// batched operator
// ------------------------------------------------------------------------------------------
namespace {

int64_t align32(int64_t x) { return (x + 31) & ~int64_t(31); }

CopyTask contiguous_task(int64_t n, int64_t soff, int64_t doff) {
  CopyTask t;
  t.nd = 1;
  t.ext[0] = n;
  t.sstr[0] = 1;
  t.dstr[0] = 1;
  t.soff = soff;
  t.doff = doff;
  return t;
}

void append_shifted(std::vector<CopyTask>& out, const std::vector<CopyTask>& in, int64_t ds,
                    int64_t dd) {
  for (CopyTask t : in) {
    t.soff += ds;
    t.doff += dd;
    out.push_back(t);
  }
}

void append_shifted(std::vector<GemmTask>& out, const std::vector<GemmTask>& in, int64_t da,
                    int64_t db, int64_t dc) {
  for (GemmTask t : in) {
    t.offA += da;
    t.offB += db;
    t.offC += dc;
    out.push_back(t);
  }
}

}  // namespace

namespace {

// What the batch needs of one chain: its structure-only plans (host task lists) and how its
// FP64 fused constant operands get into the batch's buffers.
struct ChainPart {
  TensorMeta vmeta;
  std::shared_ptr<HeffPlans> plans;
  double ref_flops = 0;
  const double* A1 = nullptr;  // fused constant operands prepared elsewhere (copied in), or
  const double* B2 = nullptr;  // null: folded straight into the batch's buffers by `fold`
};

std::unique_ptr<HeffBatch> build_batch(
    Context* ctx, std::unique_ptr<HeffBatch> B, const std::vector<ChainPart>& ch, int precision,
    const std::function<void(int, double*, double*)>& fold) {
  const int n = (int)ch.size();
  B->ctx = ctx;
  B->S = precision;
  B->n = n;
  for (const ChainPart& c : ch) {
    B->vmeta.push_back(c.vmeta);
    B->ref_flops += c.ref_flops;
  }
  // segments: chain i's data in every shared buffer, 32-element aligned
  std::vector<int64_t> oA1(n), oB1(n), oC1(n), oA2(n), oB2(n), oC2(n);
  int64_t nA1 = 0, nB1 = 0, nC1 = 0, nA2 = 0, nB2 = 0, nC2 = 0;
  B->voff.resize(n);
  for (int i = 0; i < n; ++i) {
    const ContractPlan& h1 = *ch[i].plans->c1->host;
    const ContractPlan& h2 = *ch[i].plans->c2->host;
    B->voff[i] = B->vtot;
    B->vtot += align32(ch[i].vmeta.total);
    oA1[i] = nA1, nA1 += align32(h1.fa.out.total);
    oB1[i] = nB1, nB1 += align32(h1.fb.out.total);
    oC1[i] = nC1, nC1 += align32(h1.mm.out.total);
    oA2[i] = nA2, nA2 += align32(h2.fa.out.total);
    oB2[i] = nB2, nB2 += align32(h2.fb.out.total);
    oC2[i] = nC2, nC2 += align32(h2.mm.out.total);
  }
  B->vin = alloc_buffer(ctx, std::max<int64_t>(B->vtot, 1));
  B->vout = alloc_buffer(ctx, std::max<int64_t>(B->vtot, 1));
  MPSG_CUDA(cudaMemsetAsync(B->vin->ptr, 0, sizeof(double) * std::max<int64_t>(B->vtot, 1),
                            ctx->stream));
  B->B1 = alloc_buffer(ctx, std::max<int64_t>(nB1, 1));
  B->C1 = alloc_buffer(ctx, std::max<int64_t>(nC1, 1));
  B->A2 = alloc_buffer(ctx, std::max<int64_t>(nA2, 1));
  B->C2 = alloc_buffer(ctx, std::max<int64_t>(nC2, 1));
  auto A1 = alloc_buffer(ctx, std::max<int64_t>(nA1, 1));
  auto B2 = alloc_buffer(ctx, std::max<int64_t>(nB2, 1));
  // every chain's constant operands into the shared buffers
  for (int i = 0; i < n; ++i) {
    const ContractPlan& h1 = *ch[i].plans->c1->host;
    const ContractPlan& h2 = *ch[i].plans->c2->host;
    if (ch[i].A1) {
      MPSG_CUDA(cudaMemcpyAsync(A1->ptr + oA1[i], ch[i].A1, sizeof(double) * h1.fa.out.total,
                                cudaMemcpyDeviceToDevice, ctx->stream));
      MPSG_CUDA(cudaMemcpyAsync(B2->ptr + oB2[i], ch[i].B2, sizeof(double) * h2.fb.out.total,
                                cudaMemcpyDeviceToDevice, ctx->stream));
    } else {
      fold(i, A1->ptr + oA1[i], B2->ptr + oB2[i]);
    }
  }
  // one problem list per GEMM over all chains
  std::vector<GemmTask> g1, g2;
  for (int i = 0; i < n; ++i) {
    append_shifted(g1, ch[i].plans->c1->mm.host, oA1[i], oB1[i], oC1[i]);
    append_shifted(g2, ch[i].plans->c2->mm.host, oA2[i], oB2[i], oC2[i]);
  }
  const char* at = std::getenv("MPSG_AUTOTUNE");
  const bool was = ctx->autotune;
  ctx->autotune = !(at && at[0] == '0');
  try {
    B->t1 = choose_tuning(ctx, g1, precision);
    B->t2 = choose_tuning(ctx, g2, precision);
  } catch (...) {
    ctx->autotune = was;
    throw;
  }
  ctx->autotune = was;
  B->g1.build(ctx, g1, precision, B->t1);
  B->g2.build(ctx, g2, precision, B->t2);
  split::launch_split_gemm(ctx, B->g1, A1->ptr, nullptr, nullptr, split::kPackA);
  split::launch_split_gemm(ctx, B->g2, nullptr, B2->ptr, nullptr, split::kPackB);
  A1.reset();  // the packed slices are all the GEMMs read (frees ordered after the packing)
  B2.reset();
  // one copy list per copy stage over all chains
  std::vector<CopyTask> tin, tx2a, tout;
  for (int i = 0; i < n; ++i) {
    const HeffPlans& P = *ch[i].plans;
    const ContractPlan& h1 = *P.c1->host;
    const ContractPlan& h2 = *P.c2->host;
    if (h1.fb.identity)
      tin.push_back(contiguous_task(ch[i].vmeta.total, B->voff[i], oB1[i]));
    else
      append_shifted(tin, h1.fb.tasks, B->voff[i], oB1[i]);
    append_shifted(tx2a, P.x2a_host, oC1[i], oA2[i]);
    if (h2.split.identity)
      tout.push_back(contiguous_task(ch[i].vmeta.total, oC2[i], B->voff[i]));
    else
      append_shifted(tout, h2.split.tasks, oC2[i], B->voff[i]);
  }
  if (ctx->debug_sync) {  // host self-check of the concatenated lists
    validate_copy_tasks(tin, B->vtot, nB1);
    validate_copy_tasks(tx2a, nC1, nA2);
    validate_copy_tasks(tout, nC2, B->vtot);
    validate_gemms(g1, nA1, nB1, nC1);
    validate_gemms(g2, nA2, nB2, nC2);
  }
  B->cin.upload(tin, false, ctx->stream);
  B->cx2a.upload(tx2a, false, ctx->stream);
  B->cout.upload(tout, false, ctx->stream);
  return B;
}

}  // namespace

std::unique_ptr<HeffBatch> heff_batch_create(Context* ctx, const std::vector<TensorMeta>& vmeta,
                                             const std::vector<const DeviceTensor*>& envL,
                                             const std::vector<const DeviceTensor*>& envR,
                                             const std::vector<const DeviceTensor*>& W1,
                                             const std::vector<const DeviceTensor*>& W2,
                                             int precision, bool use_graph) {
  const int n = (int)vmeta.size();
  if (n < 1) throw Error(kErrArgument, "a batch needs at least one operator");
  if (envL.size() != (size_t)n || envR.size() != (size_t)n || W1.size() != (size_t)n ||
      W2.size() != (size_t)n)
    throw Error(kErrArgument, "batch: operand lists of different lengths");
  if (precision < 2 || precision > split::kMaxSlices)
    throw Error(kErrUnsupported, "a batch runs the split-precision path: precision 2..7");
  auto B = std::make_unique<HeffBatch>();
  B->use_graph = use_graph;
  std::vector<HeffParts> parts;
  std::vector<ChainPart> ch(n);
  parts.reserve(n);
  for (int i = 0; i < n; ++i) {
    for (const DeviceTensor* t : {envL[i], envR[i], W1[i], W2[i]})
      if (!t || !t->ctx || t->ctx->device != ctx->device)
        throw Error(kErrArgument, "batch: operand missing or on another device");
    parts.push_back(heff_parts(ctx, vmeta[i], *envL[i], *envR[i], *W1[i], *W2[i], precision));
    B->keys.push_back(parts.back().key);
    B->plans.push_back(parts.back().plans);  // handed back to this context's cache at the end
    ch[i].vmeta = vmeta[i];
    ch[i].plans = parts.back().plans;
    ch[i].ref_flops = applymps2site_flops(ctx, vmeta[i], envL[i]->meta, envR[i]->meta,
                                          W1[i]->meta, W2[i]->meta);
  }
  return build_batch(ctx, std::move(B), ch, precision, [&](int i, double* a1, double* b2) {
    heff_fold(ctx, parts[i], *envL[i], *envR[i], *W1[i], *W2[i], a1, b2);
  });
}

std::unique_ptr<HeffBatch> heff_batch_from_ops(Context* ctx,
                                               const std::vector<const HeffOp*>& ops,
                                               bool use_graph) {
  const int n = (int)ops.size();
  if (n < 1) throw Error(kErrArgument, "a batch needs at least one operator");
  std::vector<ChainPart> ch(n);
  int S = 0;
  for (int i = 0; i < n; ++i) {
    const HeffOp* op = ops[i];
    if (!op || !op->batch_only || !op->plans || !op->fusedA1 || !op->fusedB2)
      throw Error(kErrArgument, "batch: operator not prepared for a batch");
    if (op->ctx->device != ctx->device) throw Error(kErrArgument, "batch: operator on another device");
    if (i == 0) S = op->precision;
    if (op->precision != S) throw Error(kErrArgument, "batch: operators of different precision");
    ch[i].vmeta = op->vmeta;
    ch[i].plans = op->plans;  // read here only: the operator's context keeps its plans
    ch[i].ref_flops = op->ref_flops;
    ch[i].A1 = op->fusedA1->ptr;
    ch[i].B2 = op->fusedB2->ptr;
  }
  auto B = std::make_unique<HeffBatch>();
  B->use_graph = use_graph;
  return build_batch(ctx, std::move(B), ch, S, nullptr);
}

void HeffBatch::run_launches() {
  launch_copy(ctx, cin, vin->ptr, B1->ptr);
  split::launch_split_gemm(ctx, g1, nullptr, B1->ptr, C1->ptr, split::kPackB | split::kRunGemm);
  launch_copy(ctx, cx2a, C1->ptr, A2->ptr);
  split::launch_split_gemm(ctx, g2, A2->ptr, nullptr, C2->ptr, split::kPackA | split::kRunGemm);
  launch_copy(ctx, cout, C2->ptr, vout->ptr);
}

void HeffBatch::apply() {
  // the first application runs eagerly (it also sets the kernels' shared-memory limits); the
  // second is captured into a graph that every later application replays
  if (!use_graph || ctx->debug_sync || ctx->timing || applies == 0) {
    run_launches();
    ++applies;
    return;
  }
  if (!exec) {
    const int64_t k0 = ctx->kernel_launches;
    const double f0 = ctx->gemm_flops;
    MPSG_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    try {
      run_launches();
    } catch (...) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(ctx->stream, &g);
      if (g) cudaGraphDestroy(g);
      ctx->kernel_launches = k0;
      ctx->gemm_flops = f0;
      throw;
    }
    MPSG_CUDA(cudaStreamEndCapture(ctx->stream, &graph));
    graph_kernels = ctx->kernel_launches - k0;
    ctx->kernel_launches = k0;
    ctx->gemm_flops = f0;
    MPSG_CUDA(cudaGraphInstantiate(&exec, graph, 0));
  }
  MPSG_CUDA(cudaGraphLaunch(exec, ctx->stream));
  ctx->kernel_launches += graph_kernels;
  ctx->gemm_flops += g1.flops + g2.flops;
  ++applies;
}

HeffBatch::~HeffBatch() {
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  cin.release();
  cx2a.release();
  cout.release();
  for (int i = 0; i < (int)plans.size(); ++i) heff_plans_return(ctx, keys[i], plans[i]);
}

// ------------------------------------------------------------------------------------------
// lock-step Lanczos
// ------------------------------------------------------------------------------------------
namespace {

constexpr int kMaxChains = 128;
constexpr int kMaxKd = 32;
constexpr int kBT = 256;  // threads of the per-chain vector kernels

struct ChainGeom {
  int64_t off, n;
};

enum : int {
  kFOrth = 1,     // reorthogonalise w against V_0 .. V_{K-1}
  kFNorm = 2,     // norm of w
  kFEig = 4,      // eigen-decomposition of the K x K projected matrix
  kFFinish = 8,   // x = sum_j U(j, 0) V_j
  kFRestart = 16, // V_i <- sum_j U(j, i) V_j (i < keep), projected matrix restarted
  kFNewVec = 32,  // V_K = w / beta (and the application input)
  kFSetBeta = 64, // ... with H(K, K-1) = H(K-1, K) = beta
  kFNormX = 128   // norm of x
};

// Per-step arguments, passed by value (no host-to-device copy between host decisions).
struct StepArgs {
  double beta[kMaxChains];
  int32_t K[kMaxChains];
  int32_t flags[kMaxChains];
  int32_t keep[kMaxChains];
};

__device__ __forceinline__ double block_sum_b(double v, double* red) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  return s;  // valid in thread 0
}

// partial dots <V_j, w>, j < K, over this block's part of chain c's segment
__global__ void __launch_bounds__(kBT) bl_orth_partial(const double* __restrict__ V, int64_t vtot,
                                                      const double* __restrict__ w,
                                                      const ChainGeom* __restrict__ geo,
                                                      StepArgs st, double* __restrict__ part) {
  const int c = blockIdx.y;
  if (!(st.flags[c] & kFOrth)) return;
  const int K = st.K[c];
  const int64_t off = geo[c].off, n = geo[c].n;
  double acc[kMaxKd];
#pragma unroll
  for (int j = 0; j < kMaxKd; ++j) acc[j] = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kBT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kBT) {
    const double wi = w[off + i];
#pragma unroll
    for (int j = 0; j < kMaxKd; ++j)
      if (j < K) acc[j] = fma(V[(int64_t)j * vtot + off + i], wi, acc[j]);
  }
  __shared__ double red[kBT / 32][kMaxKd];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < kMaxKd; ++j) {
    if (j < K) {
      double s = acc[j];
      for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) red[warp][j] = s;
    }
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double s = 0.0;
    for (int wp = 0; wp < kBT / 32; ++wp) s += red[wp][threadIdx.x];
    part[((int64_t)c * kMaxKd + threadIdx.x) * gridDim.x + blockIdx.x] = s;
  }
}

// dots (fixed summation order), the update coefficients, and H(K-1, K-1) += dots[K-1]
__global__ void bl_orth_finish(const double* __restrict__ part, int G, StepArgs st,
                               double* __restrict__ coef, double* __restrict__ H, int ld) {
  const int c = blockIdx.x;
  if (!(st.flags[c] & kFOrth)) return;
  const int K = st.K[c], j = threadIdx.x;
  if (j < K) {
    double s = 0.0;
    for (int b = 0; b < G; ++b) s += part[((int64_t)c * kMaxKd + j) * G + b];
    coef[c * kMaxKd + j] = -s;
    if (j == K - 1) H[(int64_t)c * ld * ld + (K - 1) + (int64_t)ld * (K - 1)] += s;
  }
}

// w <- w - sum_j dots_j V_j
__global__ void __launch_bounds__(kBT) bl_orth_update(const double* __restrict__ V, int64_t vtot,
                                                     double* __restrict__ w,
                                                     const ChainGeom* __restrict__ geo,
                                                     StepArgs st, const double* __restrict__ coef) {
  const int c = blockIdx.y;
  if (!(st.flags[c] & kFOrth)) return;
  const int K = st.K[c];
  const int64_t off = geo[c].off, n = geo[c].n;
  __shared__ double cf[kMaxKd];
  if (threadIdx.x < K) cf[threadIdx.x] = coef[c * kMaxKd + threadIdx.x];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * kBT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kBT) {
    double y = w[off + i];
#pragma unroll
    for (int j = 0; j < kMaxKd; ++j)
      if (j < K) y = fma(cf[j], V[(int64_t)j * vtot + off + i], y);
    w[off + i] = y;
  }
}

// partial sums of squares of x over chains with `flag`
__global__ void __launch_bounds__(kBT) bl_norm_partial(const double* __restrict__ x,
                                                      const ChainGeom* __restrict__ geo,
                                                      StepArgs st, int flag,
                                                      double* __restrict__ part) {
  const int c = blockIdx.y;
  if (!(st.flags[c] & flag)) return;
  const int64_t off = geo[c].off, n = geo[c].n;
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kBT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kBT)
    acc = fma(x[off + i], x[off + i], acc);
  __shared__ double red[kBT / 32];
  const double s = block_sum_b(acc, red);
  if (threadIdx.x == 0) part[(int64_t)c * gridDim.x + blockIdx.x] = s;
}

__global__ void bl_norm_finish(const double* __restrict__ part, int G, int nch, StepArgs st,
                               int flag, double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nch || !(st.flags[c] & flag)) return;
  double s = 0.0;
  for (int b = 0; b < G; ++b) s += part[(int64_t)c * G + b];
  out[c] = sqrt(s);
}

// eigen-decomposition of chain c's K x K projected matrix; (D[0], U(K-1, 0)) to eigout
__global__ void bl_eig(const double* __restrict__ H, int ld, StepArgs st, double* __restrict__ D,
                       double* __restrict__ U, double* __restrict__ eigout) {
  const int c = blockIdx.x;
  if (!(st.flags[c] & kFEig)) return;
  const int K = st.K[c];
  double* Dc = D + (int64_t)c * kMaxKd;
  double* Uc = U + (int64_t)c * kMaxKd * kMaxKd;
  warp_eigh(H + (int64_t)c * ld * ld, ld, K, Dc, Uc);
  __syncwarp();
  if (threadIdx.x == 0) {
    eigout[2 * c] = Dc[0];
    eigout[2 * c + 1] = Uc[K - 1];
  }
}

// finish: X = sum_j U(j, 0) V_j; restart: V_q <- sum_j U(j, q) V_j for q < keep (in place:
// every element reads all K old values before writing)
__global__ void __launch_bounds__(kBT) bl_combine(double* __restrict__ V, int64_t vtot,
                                                 const ChainGeom* __restrict__ geo, StepArgs st,
                                                 const double* __restrict__ U,
                                                 double* __restrict__ X) {
  const int c = blockIdx.y;
  const int fl = st.flags[c];
  if (!(fl & (kFFinish | kFRestart))) return;
  const int K = st.K[c], keep = (fl & kFFinish) ? 1 : st.keep[c];
  const int64_t off = geo[c].off, n = geo[c].n;
  __shared__ double u[kMaxKd * kMaxKd];
  for (int e = threadIdx.x; e < K * K; e += kBT) u[e] = U[(int64_t)c * kMaxKd * kMaxKd + e];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * kBT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kBT) {
    double v[kMaxKd];
#pragma unroll
    for (int j = 0; j < kMaxKd; ++j)
      if (j < K) v[j] = V[(int64_t)j * vtot + off + i];
    for (int q = 0; q < keep; ++q) {
      double s = 0.0;
#pragma unroll
      for (int j = 0; j < kMaxKd; ++j)
        if (j < K) s = fma(u[j + K * q], v[j], s);
      if (fl & kFFinish)
        X[off + i] = s;
      else
        V[(int64_t)q * vtot + off + i] = s;
    }
  }
}

// restart of the projected matrix: H <- 0, H(i, i) = D(i), H(keep, i) = H(i, keep) =
// beta U(K-1, i) for i < keep
__global__ void bl_restart_h(double* __restrict__ H, int ld, StepArgs st,
                             const double* __restrict__ D, const double* __restrict__ U) {
  const int c = blockIdx.x;
  if (!(st.flags[c] & kFRestart)) return;
  double* Hc = H + (int64_t)c * ld * ld;
  const int K = st.K[c], keep = st.keep[c];
  for (int e = threadIdx.x; e < ld * ld; e += blockDim.x) Hc[e] = 0.0;
  __syncthreads();
  const int i = threadIdx.x;
  if (i < keep) {
    Hc[i + (int64_t)ld * i] = D[(int64_t)c * kMaxKd + i];
    const double b = st.beta[c] * U[(int64_t)c * kMaxKd * kMaxKd + (K - 1) + (int64_t)K * i];
    Hc[keep + (int64_t)ld * i] = b;
    Hc[i + (int64_t)ld * keep] = b;
  }
}

// V_K = w / beta, also into the application input; H(K, K-1) = H(K-1, K) = beta when asked
// (w may be V_0 itself: each element is read before it is written by the same thread)
__global__ void __launch_bounds__(kBT) bl_newvec(const double* w, double* V, int64_t vtot,
                                                double* __restrict__ vin,
                                                const ChainGeom* __restrict__ geo, StepArgs st,
                                                double* __restrict__ H, int ld) {
  const int c = blockIdx.y;
  const int fl = st.flags[c];
  if (!(fl & kFNewVec)) return;
  const int K = st.K[c];
  const double a = 1.0 / st.beta[c];
  const int64_t off = geo[c].off, n = geo[c].n;
  for (int64_t i = (int64_t)blockIdx.x * kBT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kBT) {
    const double y = a * w[off + i];
    V[(int64_t)K * vtot + off + i] = y;
    vin[off + i] = y;
  }
  if ((fl & kFSetBeta) && blockIdx.x == 0 && threadIdx.x == 0) {
    double* Hc = H + (int64_t)c * ld * ld;
    Hc[K + (int64_t)ld * (K - 1)] = st.beta[c];
    Hc[(K - 1) + (int64_t)ld * K] = st.beta[c];
  }
}

__global__ void __launch_bounds__(kBT) bl_scale_by_inverse(double* __restrict__ x,
                                                          const ChainGeom* __restrict__ geo,
                                                          StepArgs st, int flag,
                                                          const double* __restrict__ nrm) {
  const int c = blockIdx.y;
  if (!(st.flags[c] & flag)) return;
  const double a = 1.0 / nrm[c];
  const int64_t off = geo[c].off, n = geo[c].n;
  for (int64_t i = (int64_t)blockIdx.x * kBT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kBT)
    x[off + i] = a * x[off + i];
}

}  // namespace

std::vector<EigResult> eigsolve_heff2_batch(HeffBatch& B, const std::vector<const DeviceTensor*>& x0,
                                            int krylovdim, int maxiter, double tol) {
  Context* ctx = B.ctx;
  const int nch = B.n;
  if (krylovdim < 2) throw Error(kErrArgument, "krylovdim must be at least 2");
  if (krylovdim > kMaxKd) throw Error(kErrArgument, "krylovdim must be at most 32");
  if (maxiter < 1) throw Error(kErrArgument, "maxiter must be at least 1");
  if (nch > kMaxChains)
    throw Error(kErrUnsupported, "a batched eigensolve takes at most 128 chains");
  if ((int)x0.size() != nch) throw Error(kErrArgument, "batch: one start vector per chain");
  for (int c = 0; c < nch; ++c) {
    if (!x0[c] || !x0[c]->ctx || x0[c]->ctx->device != ctx->device)
      throw Error(kErrArgument, "batch: start vector missing or on another device");
    if (!same_meta(x0[c]->meta, B.vmeta[c]))
      throw Error(kErrSpaceMismatch, "batch: start vector of another structure");
  }
  const int kd = krylovdim, ld = kd + 1;
  const cudaStream_t st = ctx->stream;
  int64_t nmax = 1;
  std::vector<ChainGeom> geo(nch);
  for (int c = 0; c < nch; ++c) {
    geo[c] = ChainGeom{B.voff[c], B.vmeta[c].total};
    nmax = std::max(nmax, geo[c].n);
  }
  const int G =
      (int)std::min<int64_t>(32, std::max<int64_t>(1, (nmax + kBT * 16 - 1) / (kBT * 16)));
  const int64_t vtot = B.vtot;
  // device storage: Krylov basis (kd + 1 vectors), result vectors, projected matrices, tables
  auto Vb = alloc_buffer(ctx, (int64_t)(kd + 1) * vtot);
  auto Xb = alloc_buffer(ctx, vtot);
  const int64_t nH = (int64_t)nch * ld * ld, nD = (int64_t)nch * kMaxKd,
                nU = (int64_t)nch * kMaxKd * kMaxKd, nC = (int64_t)nch * kMaxKd,
                nP = (int64_t)nch * kMaxKd * G, nE = 2 * (int64_t)nch, nN = nch;
  auto Wb = alloc_buffer(ctx, nH + nD + nU + nC + nP + nE + 2 * nN);
  double* H = Wb->ptr;
  double* D = H + nH;
  double* U = D + nD;
  double* coef = U + nU;
  double* part = coef + nC;
  double* eigout = part + nP;
  double* nrm = eigout + nE;
  double* nrmx = nrm + nN;
  MPSG_CUDA(cudaMemsetAsync(H, 0, sizeof(double) * nH, st));
  ChainGeom* d_geo = nullptr;
  MPSG_CUDA(cudaMallocAsync((void**)&d_geo, sizeof(ChainGeom) * nch, st));
  MPSG_CUDA(cudaMemcpyAsync(d_geo, geo.data(), sizeof(ChainGeom) * nch, cudaMemcpyHostToDevice, st));
  double* h_out = ctx->h_pinned + 64;  // pinned: norms and eigen outputs read by the host
  static_assert(Context::kPinnedDoubles >= 64 + 3 * kMaxChains, "pinned scratch too small");
  struct Guard {
    ChainGeom* g;
    cudaStream_t s;
    ~Guard() {
      if (g) cudaFreeAsync(g, s);
    }
  } guard{d_geo, st};
  double* V = Vb->ptr;
  double* w = B.vout->ptr;
  const dim3 vgrid((unsigned)G, (unsigned)nch);
  auto launched = [&](int k) {
    MPSG_CUDA(cudaGetLastError());
    ctx->kernel_launches += k;
  };
  // norms of x over the chains flagged `flag` into out (device) and h_out[0..nch) (host)
  auto norms = [&](const StepArgs& a, const double* x, int flag, double* out) {
    bl_norm_partial<<<vgrid, kBT, 0, st>>>(x, d_geo, a, flag, part);
    bl_norm_finish<<<(nch + 127) / 128, 128, 0, st>>>(part, G, nch, a, flag, out);
    launched(2);
    MPSG_CUDA(cudaMemcpyAsync(h_out, out, sizeof(double) * nch, cudaMemcpyDeviceToHost, st));
    MPSG_CUDA(cudaStreamSynchronize(st));
  };
  auto orthogonalize = [&](const StepArgs& a) {
    for (int pass = 0; pass < 2; ++pass) {
      bl_orth_partial<<<vgrid, kBT, 0, st>>>(V, vtot, w, d_geo, a, part);
      bl_orth_finish<<<nch, kMaxKd, 0, st>>>(part, G, a, coef, H, ld);
      bl_orth_update<<<vgrid, kBT, 0, st>>>(V, vtot, w, d_geo, a, coef);
      launched(3);
    }
  };

  // per-chain host state, the same recurrence as eigsolve_heff2
  std::vector<int> K(nch, 0), numops(nch, 0), numiter(nch, 1);
  std::vector<char> arrow(nch, 0), active(nch, 1);
  std::vector<double> beta(nch, 0.0);
  std::vector<EigResult> R(nch);
  StepArgs a;
  std::memset(&a, 0, sizeof(a));

  // start: V_0 = x0 / |x0|
  for (int c = 0; c < nch; ++c)
    MPSG_CUDA(cudaMemcpyAsync(V + geo[c].off, x0[c]->data(), sizeof(double) * geo[c].n,
                              cudaMemcpyDeviceToDevice, st));
  for (int c = 0; c < nch; ++c) a.flags[c] = kFNormX;
  norms(a, V, kFNormX, nrm);
  for (int c = 0; c < nch; ++c) {
    beta[c] = h_out[c];
    if (!(beta[c] > 0)) throw Error(kErrArgument, "eigsolve: zero start vector");
    a.flags[c] = kFNewVec;
    a.K[c] = 0;
    a.beta[c] = beta[c];
  }
  bl_newvec<<<vgrid, kBT, 0, st>>>(V, V, vtot, B.vin->ptr, d_geo, a, H, ld);
  launched(1);
  B.apply();
  for (int c = 0; c < nch; ++c) {
    K[c] = 1;
    numops[c] = 1;
    a.flags[c] = kFOrth | kFNorm;
    a.K[c] = 1;
  }
  orthogonalize(a);
  norms(a, w, kFNorm, nrm);
  for (int c = 0; c < nch; ++c) beta[c] = h_out[c];

  for (;;) {
    // 1. chains whose basis is full (or exhausted) solve their projected problem
    std::vector<int> eig;
    for (int c = 0; c < nch; ++c)
      if (active[c] && (K[c] == kd || beta[c] <= tol)) eig.push_back(c);
    std::memset(a.flags, 0, sizeof(a.flags));
    if (!eig.empty()) {
      for (int c : eig) {
        a.flags[c] = kFEig;
        a.K[c] = K[c];
      }
      bl_eig<<<nch, 32, 0, st>>>(H, ld, a, D, U, eigout);
      launched(1);
      MPSG_CUDA(cudaMemcpyAsync(h_out + nch, eigout, sizeof(double) * 2 * nch,
                                cudaMemcpyDeviceToHost, st));
      MPSG_CUDA(cudaStreamSynchronize(st));
      std::memset(a.flags, 0, sizeof(a.flags));
      bool any_finish = false, any_restart = false;
      for (int c : eig) {
        const double lam = h_out[nch + 2 * c], ulast = h_out[nch + 2 * c + 1];
        const double normres = std::fabs(beta[c] * ulast);
        const bool converged = normres <= tol;
        a.K[c] = K[c];
        a.beta[c] = beta[c];
        if (converged || beta[c] <= tol || numiter[c] >= maxiter) {
          a.flags[c] = kFFinish | kFNormX;
          R[c].value = lam;
          R[c].normres = normres;
          R[c].numiter = numiter[c];
          R[c].numops = numops[c];
          R[c].converged = converged;
          active[c] = 0;
          any_finish = true;
        } else {
          const int keep = std::max(1, (3 * kd + 2 * (converged ? 1 : 0)) / 5);
          a.flags[c] = kFRestart;
          a.keep[c] = keep;
          ++numiter[c];
          arrow[c] = 1;
          K[c] = keep;
          any_restart = true;
        }
      }
      bl_combine<<<vgrid, kBT, 0, st>>>(V, vtot, d_geo, a, U, Xb->ptr);
      launched(1);
      if (any_restart) {
        bl_restart_h<<<nch, 64, 0, st>>>(H, ld, a, D, U);
        launched(1);
      }
      if (any_finish) {
        bl_norm_partial<<<vgrid, kBT, 0, st>>>(Xb->ptr, d_geo, a, kFNormX, part);
        bl_norm_finish<<<(nch + 127) / 128, 128, 0, st>>>(part, G, nch, a, kFNormX, nrmx);
        bl_scale_by_inverse<<<vgrid, kBT, 0, st>>>(Xb->ptr, d_geo, a, kFNormX, nrmx);
        launched(3);
      }
    }
    // 2. every chain still running takes its next Krylov vector and one application
    bool any = false;
    std::memset(a.flags, 0, sizeof(a.flags));
    for (int c = 0; c < nch; ++c) {
      if (!active[c]) continue;
      any = true;
      a.flags[c] = kFNewVec | (arrow[c] ? 0 : kFSetBeta);
      a.K[c] = K[c];
      a.beta[c] = beta[c];
      arrow[c] = 0;
    }
    if (!any) break;
    bl_newvec<<<vgrid, kBT, 0, st>>>(w, V, vtot, B.vin->ptr, d_geo, a, H, ld);
    launched(1);
    B.apply();
    std::memset(a.flags, 0, sizeof(a.flags));
    for (int c = 0; c < nch; ++c) {
      if (!active[c]) continue;
      ++K[c];
      ++numops[c];
      a.flags[c] = kFOrth | kFNorm;
      a.K[c] = K[c];
    }
    orthogonalize(a);
    norms(a, w, kFNorm, nrm);
    for (int c = 0; c < nch; ++c)
      if (active[c]) beta[c] = h_out[c];
  }
  for (int c = 0; c < nch; ++c) {
    R[c].vec = new_tensor(ctx, B.vmeta[c], false);
    MPSG_CUDA(cudaMemcpyAsync(R[c].vec.data(), Xb->ptr + geo[c].off, sizeof(double) * geo[c].n,
                              cudaMemcpyDeviceToDevice, st));
  }
  return R;
}

}  // namespace mpsg
