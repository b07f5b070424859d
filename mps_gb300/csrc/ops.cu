// Tensor-level operations: plan lookup (cached per structure), scratch management and the
// launch sequences of each SymTensors operation.
#include <algorithm>
#include <sstream>

#include "ops.hpp"
#include "split.hpp"

namespace mpsg {

// ------------------------------------------------------------------------------------------
// context and buffers
// ------------------------------------------------------------------------------------------
Buffer::~Buffer() {
  if (ptr) cudaFreeAsync(ptr, owner->stream);
}

std::shared_ptr<Buffer> alloc_buffer(Context* ctx, int64_t n) {
  auto b = std::make_shared<Buffer>();
  b->owner = ctx->shared_from_this();
  b->n = n;
  if (n > 0) MPSG_CUDA(cudaMallocAsync((void**)&b->ptr, sizeof(double) * n, ctx->stream));
  return b;
}

std::atomic<int> g_live_contexts{0};

void context_init(Context* ctx, int device) {
  ctx->device = device;
  ++g_live_contexts;
  ctx->counted = true;
  MPSG_CUDA(cudaSetDevice(device));
  MPSG_CUDA(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
  MPSG_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  cudaMemPool_t pool;
  MPSG_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
  uint64_t thr = UINT64_MAX;  // keep freed blocks cached in the pool
  MPSG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
  MPSG_CUDA(cudaMalloc(&ctx->d_partials, sizeof(double) * (ctx->num_sms * 4 + 64)));
  MPSG_CUDA(cudaMalloc(&ctx->d_copy_err, sizeof(int)));
  MPSG_CUDA(cudaMemset(ctx->d_copy_err, 0, sizeof(int)));
  MPSG_CUDA(cudaMallocHost(&ctx->h_pinned, sizeof(double) * Context::kPinnedDoubles));
  const char* dbg = std::getenv("MPSG_DEBUG_SYNC");
  ctx->debug_sync = dbg && dbg[0] == '1';
}

static cudaEvent_t take_event(Context* ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  MPSG_CUDA(cudaEventCreate(&e));
  return e;
}

KernelTimer::KernelTimer(Context* c, int k, double f) : ctx(c), kind(k), flops(f) {
  if (!ctx->timing) return;
  a = take_event(ctx);
  b = take_event(ctx);
  MPSG_CUDA(cudaEventRecord(a, ctx->stream));
}

KernelTimer::~KernelTimer() {
  if (!a) return;
  cudaEventRecord(b, ctx->stream);
  ctx->events[kind].push_back({a, b, flops});
}

void collect_kernel_times(Context* ctx) {
  MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int k = 0; k < Context::kKinds; ++k) {
    for (auto& ev : ctx->events[k]) {
      float ms = 0.f;
      MPSG_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
      ctx->timed_ms[k] += ms;
      ctx->timed_launches[k] += 1;
      ctx->timed_flops[k] += ev.flops;
      ctx->event_pool.push_back(ev.a);
      ctx->event_pool.push_back(ev.b);
    }
    ctx->events[k].clear();
  }
}

Context::~Context() {
  if (counted) --g_live_contexts;
  heff_cache.clear();
  heff_lru.clear();
  contract_cache.clear();
  releg_cache.clear();
  matmul_cache.clear();
  if (stream) cudaStreamSynchronize(stream);
  for (auto& v : events)
    for (auto& ev : v) {
      cudaEventDestroy(ev.a);
      cudaEventDestroy(ev.b);
    }
  for (auto e : event_pool) cudaEventDestroy(e);
  if (copy_stream) cudaStreamSynchronize(copy_stream);
  for (auto e : copy_ev)
    if (e) cudaEventDestroy(e);
  if (copy_stream) cudaStreamDestroy(copy_stream);
  if (solver && solver_destroy) solver_destroy(solver);
  if (d_partials) cudaFree(d_partials);
  if (d_copy_err) cudaFree(d_copy_err);
  if (h_pinned) cudaFreeHost(h_pinned);
  if (stream) cudaStreamDestroy(stream);
}

DevContract::~DevContract() {
  fa.release();
  fb.release();
  split.release();
  mm.release();
}

DevReleg::~DevReleg() { cp.release(); }

// ------------------------------------------------------------------------------------------
// tensors
// ------------------------------------------------------------------------------------------
DeviceTensor new_tensor(Context* ctx, const TensorMeta& meta, bool zero) {
  DeviceTensor t;
  t.ctx = ctx;
  t.meta = meta;
  t.buf = alloc_buffer(ctx, meta.total);
  if (zero && meta.total)
    MPSG_CUDA(cudaMemsetAsync(t.buf->ptr, 0, sizeof(double) * meta.total, ctx->stream));
  return t;
}

DeviceTensor copy_tensor(Context* ctx, const DeviceTensor& a) {
  DeviceTensor t = new_tensor(ctx, a.meta, false);
  t.diag = a.diag;
  if (a.meta.total)
    MPSG_CUDA(cudaMemcpyAsync(t.data(), a.data(), sizeof(double) * a.meta.total,
                              cudaMemcpyDeviceToDevice, ctx->stream));
  return t;
}

DeviceTensor dual_view(const DeviceTensor& a) {
  DeviceTensor t = a;
  t.meta.charge = -a.meta.charge;
  for (auto& V : t.meta.space) V.dual = !V.dual;
  return t;
}

void require_similar(const DeviceTensor& a, const DeviceTensor& b, const char* msg) {
  if (!same_meta(a.meta, b.meta)) throw Error(kErrSpaceMismatch, msg);
}

// ------------------------------------------------------------------------------------------
// releg
// ------------------------------------------------------------------------------------------
static std::string vkey(const std::vector<int>& v) {
  std::ostringstream os;
  for (int x : v) os << x << ',';
  return os.str();
}

static std::string spaces_key(const std::vector<Space>& sp) {
  TensorMeta m;
  m.space = sp;
  return meta_key(m);
}

template <class Build>
static std::shared_ptr<DevReleg> releg_plan(Context* ctx, const std::string& key, Build&& build) {
  auto it = ctx->releg_cache.find(key);
  if (it != ctx->releg_cache.end()) return it->second;
  auto p = std::make_shared<DevReleg>();
  p->host = build();
  p->cp.upload(p->host.tasks, p->host.identity, ctx->stream);
  ctx->releg_cache[key] = p;
  return p;
}

static DeviceTensor run_releg(Context* ctx, const DevReleg& p, const DeviceTensor& a) {
  DeviceTensor t;
  t.ctx = ctx;
  t.meta = p.host.out;
  if (p.host.identity) {
    t.buf = a.buf;  // same bytes: share the buffer
    return t;
  }
  t.buf = alloc_buffer(ctx, t.meta.total);
  launch_copy(ctx, p.cp, a.data(), t.data());
  return t;
}

DeviceTensor permutelegs(Context* ctx, const DeviceTensor& a, const std::vector<int>& perm1) {
  auto p = releg_plan(ctx, "P|" + meta_key(a.meta) + vkey(perm1),
                      [&] { return plan_permutelegs(a.meta, perm1); });
  DeviceTensor t = run_releg(ctx, *p, a);
  t.diag = a.diag;
  return t;
}

DeviceTensor fuselegs(Context* ctx, const DeviceTensor& a, int l1, int n, bool dual) {
  auto p = releg_plan(ctx, "F|" + meta_key(a.meta) + vkey({l1, n, (int)dual}),
                      [&] { return plan_fuselegs(a.meta, l1, n, dual); });
  return run_releg(ctx, *p, a);
}

DeviceTensor splitleg(Context* ctx, const DeviceTensor& a, int l1, const std::vector<Space>& sp) {
  auto p = releg_plan(ctx, "S|" + meta_key(a.meta) + vkey({l1}) + spaces_key(sp),
                      [&] { return plan_splitleg(a.meta, l1, sp); });
  return run_releg(ctx, *p, a);
}

DeviceTensor symmatrix(Context* ctx, const DeviceTensor& a, const std::vector<int>& rows,
                       const std::vector<int>& cols) {
  auto p = releg_plan(ctx, "M|" + meta_key(a.meta) + vkey(rows) + "/" + vkey(cols), [&] {
    FusePlan f = plan_symmatrix(a.meta, rows, cols);
    RelegPlan r;
    r.out = f.out;
    r.tasks = f.tasks;
    r.identity = f.identity;
    return r;
  });
  return run_releg(ctx, *p, a);
}

// ------------------------------------------------------------------------------------------
// block GEMM dispatch
// ------------------------------------------------------------------------------------------
static void run_gemm(Context* ctx, DevGemmPlan& g, const double* A, const double* B,
                     double* C, int precision) {
  if (precision == 0) {
    launch_gemm_f64(ctx, g, A, B, C);
    return;
  }
  if (precision < 2 || precision > split::kMaxSlices)
    throw Error(kErrUnsupported, "precision must be 0 (FP64) or 2..7 bf16 slices");
  auto& sp = g.splitp[precision];
  if (!sp) {
    sp = std::make_shared<split::SplitPlan>();
    sp->build(ctx, g.host, precision, choose_tuning(ctx, g.host, precision));
    // the new scratch counts against the plan caches' budgets (the caller holds `g`)
    ctx->contract_cache.trim();
    ctx->matmul_cache.trim();
  }
  split::launch_split_gemm(ctx, *sp, A, B, C);
}

DeviceTensor matmul(Context* ctx, const DeviceTensor& a, const DeviceTensor& b, int precision) {
  std::string key = "G|" + meta_key(a.meta) + "*" + meta_key(b.meta);
  std::shared_ptr<DevGemmPlan> g;
  std::shared_ptr<TensorMeta> outmeta;
  g = ctx->matmul_cache.get(key);
  if (!g) {
    MatmulPlan mp = plan_matmul(a.meta, b.meta);
    g = std::make_shared<DevGemmPlan>();
    g->upload(mp.gemms, mp.flops, ctx->stream);
    ctx->matmul_cache.put(key, g);
  }
  DeviceTensor t;
  t.ctx = ctx;
  t.meta = TensorMeta::build(a.meta.charge + b.meta.charge, {a.meta.space[0], b.meta.space[1]});
  t.buf = alloc_buffer(ctx, t.meta.total);
  run_gemm(ctx, *g, a.data(), b.data(), t.data(), precision);
  return t;
}

// ------------------------------------------------------------------------------------------
// contract
// ------------------------------------------------------------------------------------------
std::shared_ptr<DevContract> get_contract_plan(Context* ctx, const TensorMeta& A,
                                               const std::vector<int>& idxA,
                                               const TensorMeta& B,
                                               const std::vector<int>& idxB) {
  std::string key = "C|" + meta_key(A) + vkey(idxA) + "|" + meta_key(B) + vkey(idxB);
  if (auto hit = ctx->contract_cache.get(key)) return hit;
  auto p = std::make_shared<DevContract>();
  p->host = plan_contract(A, idxA, B, idxB);
  if (!p->host->scalar) {
    p->fa.upload(p->host->fa.tasks, p->host->fa.identity, ctx->stream);
    p->fb.upload(p->host->fb.tasks, p->host->fb.identity, ctx->stream);
    p->mm.upload(p->host->mm.gemms, p->host->mm.flops, ctx->stream);
    p->split.upload(p->host->split.tasks, p->host->split.identity, ctx->stream);
  }
  ctx->contract_cache.put(key, p);
  return p;
}

std::shared_ptr<Buffer> contract_gemm(Context* ctx, DevContract& p, const DeviceTensor& a,
                                      const DeviceTensor& b, int precision) {
  std::shared_ptr<Buffer> fa, fb;
  const double* pa = a.data();
  const double* pb = b.data();
  if (!p.fa.identity) {
    fa = alloc_buffer(ctx, p.host->fa.out.total);
    launch_copy(ctx, p.fa, a.data(), fa->ptr);
    pa = fa->ptr;
  }
  if (!p.fb.identity) {
    fb = alloc_buffer(ctx, p.host->fb.out.total);
    launch_copy(ctx, p.fb, b.data(), fb->ptr);
    pb = fb->ptr;
  }
  auto fc = alloc_buffer(ctx, p.host->mm.out.total);
  run_gemm(ctx, p.mm, pa, pb, fc->ptr, precision);
  return fc;
}

DeviceTensor contract(Context* ctx, const DeviceTensor& a, const std::vector<int>& idxA,
                      const DeviceTensor& b, const std::vector<int>& idxB, int precision,
                      double* scalar) {
  auto p = get_contract_plan(ctx, a.meta, idxA, b.meta, idxB);
  if (p->host->scalar) {
    // SymVector(A) .* SymVector(B) summed (contract.jl:24-28, 226-232)
    std::vector<int> ra, ca, tf, rb, cb, tfb;
    contract_index_perm(idxA, ra, ca, tf);
    contract_index_perm(idxB, rb, cb, tfb);
    DeviceTensor va = fuselegs(ctx, permutelegs(ctx, a, ca), 1, a.meta.N(), false);
    DeviceTensor vb = fuselegs(ctx, permutelegs(ctx, b, cb), 1, b.meta.N(), true);
    double s = 0.0;
    if (va.meta.nblocks() && vb.meta.nblocks()) {
      long ib = vb.meta.find(va.meta.sec.labels(0));
      if (ib < 0) throw Error(kErrSpaceMismatch, "KeyError in SymVector product");
      int64_t n = va.meta.sec.numel(0);
      launch_dot(ctx, n, va.data() + va.meta.off[0], vb.data() + vb.meta.off[ib],
                 ctx->d_partials + ctx->num_sms * 4);
      MPSG_CUDA(cudaMemcpyAsync(ctx->h_pinned, ctx->d_partials + ctx->num_sms * 4,
                                sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
      MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
      s = ctx->h_pinned[0];
    }
    if (scalar) *scalar = s;
    return DeviceTensor();
  }
  std::shared_ptr<Buffer> fc = contract_gemm(ctx, *p, a, b, precision);
  DeviceTensor t;
  t.ctx = ctx;
  t.meta = p->host->split.out;
  if (p->split.identity) {
    t.buf = fc;
  } else {
    t.buf = alloc_buffer(ctx, t.meta.total);
    launch_copy(ctx, p->split, fc->ptr, t.data());
  }
  return t;
}

// ------------------------------------------------------------------------------------------
// effective Hamiltonian and environments (apply.jl:17-25, 49-58, 93-105)
// ------------------------------------------------------------------------------------------
static const std::vector<int> kH1A = {-1, 2, 1}, kH1B = {-1, 3, 4, 5};
static const std::vector<int> kH2A = {1, -1, -2, 4, 5}, kH2B = {-1, 2, 3, -2};
static const std::vector<int> kH3A = {1, 2, -1, -2, 5}, kH3B = {-1, 3, 4, -2};
static const std::vector<int> kH4A = {1, 2, 3, -1, -2}, kH4B = {-2, -1, 4};

DeviceTensor applymps2site(Context* ctx, const DeviceTensor& v, const DeviceTensor& envL,
                           const DeviceTensor& envR, const DeviceTensor& W1,
                           const DeviceTensor& W2, int precision) {
  if (precision != 0) {  // tensor-core path: prepared (W-folded) operator, built per call here
    auto op = heff_create(ctx, v.meta, envL, envR, W1, W2, precision);
    return heff_apply(*op, v);
  }
  DeviceTensor t1 = contract(ctx, envL, kH1A, v, kH1B, precision, nullptr);
  DeviceTensor t2 = contract(ctx, t1, kH2A, W1, kH2B, precision, nullptr);
  t1 = DeviceTensor();
  DeviceTensor t3 = contract(ctx, t2, kH3A, W2, kH3B, precision, nullptr);
  t2 = DeviceTensor();
  return contract(ctx, t3, kH4A, envR, kH4B, precision, nullptr);
}

void ensure_copy_stream(Context* ctx) {
  if (ctx->copy_stream) return;
  MPSG_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
  for (auto& e : ctx->copy_ev) MPSG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
}

AsyncCopy::~AsyncCopy() {
  if (done) {
    cudaEventSynchronize(done);
    cudaEventDestroy(done);
  }
}

std::unique_ptr<AsyncCopy> copy_async(Context* ctx, const DeviceTensor& t, double* host,
                                      bool to_host) {
  ensure_copy_stream(ctx);
  auto c = std::make_unique<AsyncCopy>();
  c->owner = ctx->shared_from_this();
  c->buf = t.buf;
  MPSG_CUDA(cudaEventCreateWithFlags(&c->done, cudaEventDisableTiming));
  // after the kernels that wrote t (download), or t's allocation and every queued reader of its
  // old contents (upload)
  MPSG_CUDA(cudaEventRecord(ctx->copy_ev[3], ctx->stream));
  MPSG_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->copy_ev[3], 0));
  const size_t bytes = sizeof(double) * (size_t)t.meta.total;
  if (bytes) {
    if (to_host)
      MPSG_CUDA(cudaMemcpyAsync(host, t.data(), bytes, cudaMemcpyDeviceToHost, ctx->copy_stream));
    else
      MPSG_CUDA(cudaMemcpyAsync(t.data(), host, bytes, cudaMemcpyHostToDevice, ctx->copy_stream));
  }
  MPSG_CUDA(cudaEventRecord(c->done, ctx->copy_stream));
  return c;
}

DeviceTensor applymps2site_host(Context* ctx, const DeviceTensor& v, const DeviceTensor& envL,
                                const DeviceTensor& envR, const DeviceTensor& W1,
                                const DeviceTensor& W2, const double* const host_in[5],
                                int precision, double* host_out) {
  ensure_copy_stream(ctx);
  cudaStream_t cs = ctx->copy_stream;
  // the uploads overwrite the inputs: after everything already queued on the context stream
  MPSG_CUDA(cudaEventRecord(ctx->copy_ev[3], ctx->stream));
  MPSG_CUDA(cudaStreamWaitEvent(cs, ctx->copy_ev[3], 0));
  const DeviceTensor* dst[5] = {&W1, &envL, &W2, &envR, &v};
  const int src_of[5] = {3, 1, 4, 2, 0};  // host_in order: v, envL, envR, W1, W2
  for (int i = 0; i < 5; ++i) {
    const DeviceTensor& t = *dst[i];
    if (t.meta.total)
      MPSG_CUDA(cudaMemcpyAsync(t.data(), host_in[src_of[i]], sizeof(double) * t.meta.total,
                                cudaMemcpyHostToDevice, cs));
    if (i == 1) MPSG_CUDA(cudaEventRecord(ctx->copy_ev[0], cs));  // W1, envL: left fold
    if (i == 3) MPSG_CUDA(cudaEventRecord(ctx->copy_ev[1], cs));  // W2, envR: right fold
  }
  MPSG_CUDA(cudaEventRecord(ctx->copy_ev[2], cs));  // v
  DeviceTensor out;
  if (precision != 0) {
    auto op = heff_create(ctx, v.meta, envL, envR, W1, W2, precision, ctx->copy_ev[0],
                          ctx->copy_ev[1]);
    MPSG_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->copy_ev[2], 0));
    out = heff_apply(*op, v);
  } else {
    MPSG_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->copy_ev[2], 0));
    out = applymps2site(ctx, v, envL, envR, W1, W2, 0);
  }
  if (out.meta.total)
    MPSG_CUDA(cudaMemcpyAsync(host_out, out.data(), sizeof(double) * out.meta.total,
                              cudaMemcpyDeviceToHost, ctx->stream));
  MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
  return out;
}

double applymps2site_flops(Context* ctx, const TensorMeta& v, const TensorMeta& envL,
                           const TensorMeta& envR, const TensorMeta& W1, const TensorMeta& W2) {
  auto p1 = get_contract_plan(ctx, envL, kH1A, v, kH1B);
  auto p2 = get_contract_plan(ctx, p1->host->split.out, kH2A, W1, kH2B);
  auto p3 = get_contract_plan(ctx, p2->host->split.out, kH3A, W2, kH3B);
  auto p4 = get_contract_plan(ctx, p3->host->split.out, kH4A, envR, kH4B);
  return p1->host->flops + p2->host->flops + p3->host->flops + p4->host->flops;
}

DeviceTensor mpsupdateleft(Context* ctx, const DeviceTensor& env, const DeviceTensor& A,
                           const DeviceTensor& W, int precision) {
  DeviceTensor t = contract(ctx, env, {-1, 3, 4}, A, {-1, 2, 1}, precision, nullptr);
  t = contract(ctx, t, {1, -1, -2, 4}, W, {-2, 2, 3, -1}, precision, nullptr);
  return contract(ctx, t, {1, -1, 2, -2}, dual_view(A), {-2, -1, 3}, precision, nullptr);
}

DeviceTensor mpsupdateright(Context* ctx, const DeviceTensor& env, const DeviceTensor& A,
                            const DeviceTensor& W, int precision) {
  DeviceTensor t = contract(ctx, env, {-1, 3, 4}, A, {1, 2, -1}, precision, nullptr);
  t = contract(ctx, t, {1, -1, -2, 4}, W, {3, 2, -2, -1}, precision, nullptr);
  return contract(ctx, t, {1, -1, 2, -2}, dual_view(A), {3, -1, -2}, precision, nullptr);
}

// ------------------------------------------------------------------------------------------
// prepared effective Hamiltonian
// ------------------------------------------------------------------------------------------
static std::shared_ptr<DevContract> private_contract_plan(Context* ctx, const TensorMeta& A,
                                                          const std::vector<int>& idxA,
                                                          const TensorMeta& B,
                                                          const std::vector<int>& idxB) {
  auto p = std::make_shared<DevContract>();
  p->host = plan_contract(A, idxA, B, idxB);
  if (p->host->scalar) throw Error(kErrArgument, "unexpected full contraction");
  p->fa.upload(p->host->fa.tasks, p->host->fa.identity, ctx->stream);
  p->fb.upload(p->host->fb.tasks, p->host->fb.identity, ctx->stream);
  p->mm.upload(p->host->mm.gemms, p->host->mm.flops, ctx->stream);
  p->split.upload(p->host->split.tasks, p->host->split.identity, ctx->stream);
  return p;
}

static const std::vector<int> kLW_A = {1, -1, 3}, kLW_B = {-1, 5, 4, 2};
static const std::vector<int> kRW_A = {2, 4, -1, 3}, kRW_B = {1, -1, 5};
static const std::vector<int> kX_A = {-1, -2, 1, 3, 2}, kX_B = {-1, -2, 4, 5};
static const std::vector<int> kO_A = {1, 2, -1, -2, -3}, kO_B = {-3, -1, -2, 3, 4};

FoldedHeffPlans plan_heff_folded(const TensorMeta& v, const TensorMeta& envL,
                                 const TensorMeta& envR, const TensorMeta& W1,
                                 const TensorMeta& W2) {
  FoldedHeffPlans F;
  F.lw = plan_contract(envL, kLW_A, W1, kLW_B);
  F.rw = plan_contract(W2, kRW_A, envR, kRW_B);
  F.c1 = plan_contract(F.lw->split.out, kX_A, v, kX_B);
  F.c2 = plan_contract(F.c1->split.out, kO_A, F.rw->split.out, kO_B);
  std::vector<BlockMap> src_of_x, dst_of_x;
  const ContractPlan& c1 = *F.c1;
  const ContractPlan& c2 = *F.c2;
  plan_split_permute_rec(c1.mm.out, c1.rlegs, c1.clegs, c1.perm, &src_of_x);
  plan_symmatrix_rec(c1.split.out, c2.rowsA, c2.colsA, &dst_of_x);
  F.x2a = compose_through(c1.split.out, src_of_x, dst_of_x);
  for (int side = 0; side < 2; ++side) {  // fold output -> fused GEMM operand
    const ContractPlan& f = side ? *F.rw : *F.lw;
    std::vector<BlockMap> src, dst;
    plan_split_permute_rec(f.mm.out, f.rlegs, f.clegs, f.perm, &src);
    if (side)
      plan_symmatrix_rec(f.split.out, c2.rowsB, c2.colsB, &dst);
    else
      plan_symmatrix_rec(f.split.out, c1.rowsA, c1.colsA, &dst);
    (side ? F.rw2b : F.lw2a) = compose_through(f.split.out, src, dst);
  }
  return F;
}

void check_heff_folded(const TensorMeta& v, const TensorMeta& envL, const TensorMeta& envR,
                       const TensorMeta& W1, const TensorMeta& W2) {
  FoldedHeffPlans F = plan_heff_folded(v, envL, envR, W1, W2);
  for (auto* c : {F.lw.get(), F.rw.get(), F.c1.get(), F.c2.get()}) {
    const TensorMeta* A = c == F.lw.get() ? &envL : c == F.rw.get() ? &W2
                          : c == F.c1.get() ? &F.lw->split.out : &F.c1->split.out;
    const TensorMeta* B = c == F.lw.get() ? &W1 : c == F.rw.get() ? &envR
                          : c == F.c1.get() ? &v : &F.rw->split.out;
    validate_contract(*c, *A, *B);
  }
  check_composition(F.c1->split.tasks, F.c1->mm.out.total, F.c1->split.out.total,
                    F.c2->fa.tasks, F.c2->fa.out.total, F.x2a);
  check_composition(F.lw->split.tasks, F.lw->mm.out.total, F.lw->split.out.total,
                    F.c1->fa.tasks, F.c1->fa.out.total, F.lw2a);
  check_composition(F.rw->split.tasks, F.rw->mm.out.total, F.rw->split.out.total,
                    F.c2->fb.tasks, F.c2->fb.out.total, F.rw2b);
  if (!same_meta(F.c2->split.out, v)) throw Error(kErrSpaceMismatch, "folded H_eff changes v's structure");
}

HeffParts heff_parts(Context* ctx, const TensorMeta& vmeta, const DeviceTensor& envL,
                     const DeviceTensor& envR, const DeviceTensor& W1, const DeviceTensor& W2,
                     int precision) {
  if (precision < 2 || precision > split::kMaxSlices)
    throw Error(kErrUnsupported, "precision must be 0 (FP64) or 2..7 bf16 slices");
  HeffParts H;
  H.plw = get_contract_plan(ctx, envL.meta, kLW_A, W1.meta, kLW_B);
  H.prw = get_contract_plan(ctx, W2.meta, kRW_A, envR.meta, kRW_B);
  const TensorMeta& lwmeta = H.plw->host->split.out;
  const TensorMeta& rwmeta = H.prw->host->split.out;
  H.key = "H" + std::to_string(precision) + "|" + meta_key(vmeta) + "|" + meta_key(envL.meta) +
          "|" + meta_key(envR.meta) + "|" + meta_key(W1.meta) + "|" + meta_key(W2.meta);
  auto hit = ctx->heff_cache.find(H.key);
  if (hit != ctx->heff_cache.end()) {  // take the idle plans of this structure
    H.plans = hit->second;
    ctx->heff_cache.erase(hit);
    auto& lru = ctx->heff_lru;
    lru.erase(std::find(lru.begin(), lru.end(), H.key));
    ctx->heff_bytes -= H.plans->bytes;
    return H;
  }
  auto P = std::make_shared<HeffPlans>();
  P->c1 = private_contract_plan(ctx, lwmeta, kX_A, vmeta, kX_B);
  P->c2 = private_contract_plan(ctx, P->c1->host->split.out, kO_A, rwmeta, kO_B);
  const ContractPlan& h1 = *P->c1->host;
  const ContractPlan& h2 = *P->c2->host;
  std::vector<BlockMap> src_of_x, dst_of_x;
  plan_split_permute_rec(h1.mm.out, h1.rlegs, h1.clegs, h1.perm, &src_of_x);
  plan_symmatrix_rec(h1.split.out, h2.rowsA, h2.colsA, &dst_of_x);
  P->x2a_host = compose_through(h1.split.out, src_of_x, dst_of_x);
  P->x2a.upload(P->x2a_host, false, ctx->stream);
  for (int side = 0; side < 2; ++side) {
    const ContractPlan& f = side ? *H.prw->host : *H.plw->host;
    std::vector<BlockMap> src, dst;
    plan_split_permute_rec(f.mm.out, f.rlegs, f.clegs, f.perm, &src);
    if (side)
      plan_symmatrix_rec(f.split.out, h2.rowsB, h2.colsB, &dst);
    else
      plan_symmatrix_rec(f.split.out, h1.rowsA, h1.colsA, &dst);
    (side ? P->rw2b : P->lw2a).upload(compose_through(f.split.out, src, dst), false, ctx->stream);
  }
  H.plans = P;
  return H;
}

void heff_fold(Context* ctx, HeffParts& H, const DeviceTensor& envL, const DeviceTensor& envR,
               const DeviceTensor& W1, const DeviceTensor& W2, double* dstA1, double* dstB2,
               cudaEvent_t wait_left, cudaEvent_t wait_right) {
  // the W folds (FP64): their fused GEMM outputs go straight into GEMM 1's A and GEMM 2's B
  // operands through composed copies, so envLW and envRW are never materialised
  if (wait_left) MPSG_CUDA(cudaStreamWaitEvent(ctx->stream, wait_left, 0));
  {
    auto clw = contract_gemm(ctx, *H.plw, envL, W1, 0);
    launch_copy(ctx, H.plans->lw2a, clw->ptr, dstA1);
  }
  if (wait_right) MPSG_CUDA(cudaStreamWaitEvent(ctx->stream, wait_right, 0));
  {
    auto crw = contract_gemm(ctx, *H.prw, W2, envR, 0);
    launch_copy(ctx, H.plans->rw2b, crw->ptr, dstB2);
  }
}

void heff_plans_return(Context* ctx, const std::string& key, std::shared_ptr<HeffPlans> plans) {
  if (!plans || key.empty() || !ctx) return;
  // idle plans kept (device bytes): a share of 8 GiB per process
  const size_t kBudget = cache_share(size_t(8) << 30);
  if (ctx->heff_cache.count(key)) return;  // an idle copy exists already: drop this one
  ctx->heff_cache[key] = plans;
  ctx->heff_lru.push_back(key);
  ctx->heff_bytes += plans->bytes;
  while (ctx->heff_bytes > kBudget && !ctx->heff_lru.empty()) {
    const std::string k = ctx->heff_lru.front();
    ctx->heff_lru.erase(ctx->heff_lru.begin());
    auto it = ctx->heff_cache.find(k);
    if (it != ctx->heff_cache.end()) {
      ctx->heff_bytes -= it->second->bytes;
      ctx->heff_cache.erase(it);
    }
  }
}

std::shared_ptr<HeffOp> heff_create(Context* ctx, const TensorMeta& vmeta, const DeviceTensor& envL,
                                    const DeviceTensor& envR, const DeviceTensor& W1,
                                    const DeviceTensor& W2, int precision, cudaEvent_t wait_left,
                                    cudaEvent_t wait_right) {
  auto op = std::make_shared<HeffOp>();
  op->ctx = ctx;
  op->precision = precision;
  op->vmeta = vmeta;
  op->ref_flops = applymps2site_flops(ctx, vmeta, envL.meta, envR.meta, W1.meta, W2.meta);
  if (precision == 0) {
    op->envL = envL;
    op->envR = envR;
    op->W1 = W1;
    op->W2 = W2;
    return op;
  }
  HeffParts H = heff_parts(ctx, vmeta, envL, envR, W1, W2, precision);
  op->plans = H.plans;
  op->plan_key = H.key;
  DevContract& c1 = *op->plans->c1;
  DevContract& c2 = *op->plans->c2;
  for (auto* c : {&c1, &c2}) {  // the split plans of this operator's own GEMMs (once per plans)
    auto& sp = c->mm.splitp[precision];
    if (sp) continue;
    sp = std::make_shared<split::SplitPlan>();
    sp->build(ctx, c->mm.host, precision, choose_tuning(ctx, c->mm.host, precision));
    op->plans->bytes += (size_t)sp->S * (size_t)(sp->rowsA + sp->rowsB) * 128;
  }
  // constant operands: fuse once, slice once
  op->copy_bytes = 16.0 * (double)(c1.fb.elems + op->plans->x2a.elems + c2.split.elems);
  op->pack_bytes = (16.0 + 2.0 * precision) *
                   (double)(c1.host->fb.out.total + c2.host->fa.out.total);
  op->fusedA1 = alloc_buffer(ctx, c1.host->fa.out.total);
  op->fusedB2 = alloc_buffer(ctx, c2.host->fb.out.total);
  heff_fold(ctx, H, envL, envR, W1, W2, op->fusedA1->ptr, op->fusedB2->ptr, wait_left,
            wait_right);
  split::launch_split_gemm(ctx, *c1.mm.splitp[precision], op->fusedA1->ptr, nullptr, nullptr,
                           split::kPackA);
  split::launch_split_gemm(ctx, *c2.mm.splitp[precision], nullptr, op->fusedB2->ptr, nullptr,
                           split::kPackB);
  // the packed slices are all the GEMMs read: the FP64 operands go back to the pool (the frees
  // are ordered after the packing on the stream)
  op->fusedA1.reset();
  op->fusedB2.reset();
  return op;
}

std::shared_ptr<HeffOp> heff_prepare(Context* ctx, const TensorMeta& vmeta,
                                     const DeviceTensor& envL, const DeviceTensor& envR,
                                     const DeviceTensor& W1, const DeviceTensor& W2, int precision) {
  if (precision < 2) throw Error(kErrUnsupported, "a batch runs the split-precision path: precision 2..7");
  auto op = std::make_shared<HeffOp>();
  op->ctx = ctx;
  op->precision = precision;
  op->vmeta = vmeta;
  op->batch_only = true;
  op->ref_flops = applymps2site_flops(ctx, vmeta, envL.meta, envR.meta, W1.meta, W2.meta);
  HeffParts H = heff_parts(ctx, vmeta, envL, envR, W1, W2, precision);
  op->plans = H.plans;
  op->plan_key = H.key;
  op->fusedA1 = alloc_buffer(ctx, op->plans->c1->host->fa.out.total);
  op->fusedB2 = alloc_buffer(ctx, op->plans->c2->host->fb.out.total);
  heff_fold(ctx, H, envL, envR, W1, W2, op->fusedA1->ptr, op->fusedB2->ptr);
  return op;
}

HeffOp::~HeffOp() { heff_plans_return(ctx, plan_key, plans); }

DeviceTensor heff_apply(HeffOp& op, const DeviceTensor& v) {
  Context* ctx = op.ctx;
  if (!same_meta(v.meta, op.vmeta))
    throw Error(kErrSpaceMismatch, "H_eff applied to a tensor of another structure");
  if (op.precision == 0) return applymps2site(ctx, v, op.envL, op.envR, op.W1, op.W2, 0);
  if (op.batch_only) throw Error(kErrUnsupported, "operator prepared for a batch only");
  const int S = op.precision;
  // X = envLW . v
  DevContract& c1 = *op.plans->c1;
  auto fb = alloc_buffer(ctx, c1.host->fb.out.total);
  launch_copy(ctx, c1.fb, v.data(), fb->ptr);
  auto fc1 = alloc_buffer(ctx, c1.host->mm.out.total);
  split::launch_split_gemm(ctx, *c1.mm.splitp[S], nullptr, fb->ptr, fc1->ptr,
                           split::kPackB | split::kRunGemm);
  fb.reset();
  // v' = X . envRW, with GEMM 1's fused output moved straight into GEMM 2's fused A operand
  DevContract& c2 = *op.plans->c2;
  auto fa = alloc_buffer(ctx, c2.host->fa.out.total);
  launch_copy(ctx, op.plans->x2a, fc1->ptr, fa->ptr);
  fc1.reset();
  auto fc2 = alloc_buffer(ctx, c2.host->mm.out.total);
  split::launch_split_gemm(ctx, *c2.mm.splitp[S], fa->ptr, nullptr, fc2->ptr,
                           split::kPackA | split::kRunGemm);
  DeviceTensor out;
  out.ctx = ctx;
  out.meta = c2.host->split.out;
  if (c2.split.identity) {
    out.buf = fc2;
  } else {
    out.buf = alloc_buffer(ctx, out.meta.total);
    launch_copy(ctx, c2.split, fc2->ptr, out.data());
  }
  return out;
}

// ------------------------------------------------------------------------------------------
// reductions
// ------------------------------------------------------------------------------------------
double dot(Context* ctx, const DeviceTensor& a, const DeviceTensor& b) {
  double* d_out = ctx->d_partials + ctx->num_sms * 4;
  launch_dot(ctx, a.meta.total, a.data(), b.data(), d_out);
  MPSG_CUDA(cudaMemcpyAsync(ctx->h_pinned, d_out, sizeof(double), cudaMemcpyDeviceToHost,
                            ctx->stream));
  MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
  return ctx->h_pinned[0];
}

}  // namespace mpsg
