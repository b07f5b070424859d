// C ABI (include/mpsgb300.h): contexts, device tensors, releg, contraction, the effective
// Hamiltonian / environment updates and the Krylov vector operations.
#include <cstring>
#include <sstream>

#include "capi_internal.hpp"
#include "batch.hpp"
#include "linalg.hpp"

namespace {
thread_local std::string g_last_error;
}  // namespace

void mpsg_capi::set_last_error(const std::string& msg) { g_last_error = msg; }

namespace {

using mpsg_capi::guarded;
using mpsg_capi::ivec;
using mpsg_capi::need;

std::vector<mpsg::Space> parse_spaces(int32_t nlegs, const int32_t* nsect, const int32_t* charges,
                                      const int64_t* dims, const int32_t* isdual) {
  if (nlegs < 1 || nlegs > mpsg::kMaxLegs)
    throw mpsg::Error(mpsg::kErrArgument, "number of legs out of range");
  need(nsect, "nsect");
  need(isdual, "isdual");
  std::vector<mpsg::Space> sp;
  int64_t p = 0;
  for (int l = 0; l < nlegs; ++l) {
    if (nsect[l] < 1) throw mpsg::Error(mpsg::kErrArgument, "a leg needs at least one charge");
    need(charges, "charges");
    need(dims, "dims");
    std::vector<std::pair<int, int64_t>> pairs;
    for (int k = 0; k < nsect[l]; ++k, ++p) pairs.push_back({charges[p], dims[p]});
    sp.push_back(mpsg::Space::make(pairs, isdual[l] != 0));
  }
  return sp;
}

mpsg_tensor* wrap(mpsg::DeviceTensor&& t) {
  auto* h = new mpsg_tensor;
  h->t = std::move(t);
  return h;
}

}  // namespace

extern "C" {

int mpsg_version(void) { return 1; }

const char* mpsg_last_error(void) { return g_last_error.c_str(); }

int mpsg_ctx_create(int device, mpsg_ctx** out) {
  return guarded([&] {
    need(out, "out");
    auto c = std::make_shared<mpsg::Context>();
    mpsg::context_init(c.get(), device);
    *out = new mpsg_ctx(c);
  });
}

int mpsg_ctx_destroy(mpsg_ctx* ctx) {
  return guarded([&] {
    if (!ctx) return;
    cudaStreamSynchronize(ctx->c.stream);
    delete ctx;
  });
}

int mpsg_ctx_synchronize(mpsg_ctx* ctx) {
  return guarded([&] {
    need(ctx, "ctx");
    MPSG_CUDA(cudaStreamSynchronize(ctx->c.stream));
  });
}

int mpsg_ctx_counters(mpsg_ctx* ctx, int64_t* launches, double* flops) {
  return guarded([&] {
    need(ctx, "ctx");
    if (launches) *launches = ctx->c.kernel_launches;
    if (flops) *flops = ctx->c.gemm_flops;
  });
}

int mpsg_ctx_clear_caches(mpsg_ctx* ctx) {
  return guarded([&] {
    need(ctx, "ctx");
    MPSG_CUDA(cudaStreamSynchronize(ctx->c.stream));
    ctx->c.contract_cache.clear();
    ctx->c.releg_cache.clear();
    ctx->c.matmul_cache.clear();
    ctx->c.heff_cache.clear();
    ctx->c.heff_lru.clear();
    ctx->c.heff_bytes = 0;
  });
}

int mpsg_ctx_stream(mpsg_ctx* ctx, void** stream) {
  return guarded([&] {
    need(ctx, "ctx");
    need(stream, "stream");
    *stream = (void*)ctx->c.stream;
  });
}

int mpsg_ctx_set_timing(mpsg_ctx* ctx, int32_t enable) {
  return guarded([&] {
    need(ctx, "ctx");
    mpsg::collect_kernel_times(&ctx->c);
    ctx->c.timing = enable != 0;
    for (int k = 0; k < mpsg::Context::kKinds; ++k) {
      ctx->c.timed_ms[k] = 0;
      ctx->c.timed_launches[k] = 0;
      ctx->c.timed_flops[k] = 0;
    }
  });
}

int mpsg_ctx_kernel_time(mpsg_ctx* ctx, int32_t kind, double* total_ms, int64_t* launches,
                         double* flops) {
  return guarded([&] {
    need(ctx, "ctx");
    if (kind < 0 || kind >= mpsg::Context::kKinds)
      throw mpsg::Error(mpsg::kErrArgument, "kernel kind out of range");
    mpsg::collect_kernel_times(&ctx->c);
    if (total_ms) *total_ms = ctx->c.timed_ms[kind];
    if (launches) *launches = ctx->c.timed_launches[kind];
    if (flops) *flops = ctx->c.timed_flops[kind];
  });
}

int mpsg_tensor_create(mpsg_ctx* ctx, int32_t charge, int32_t nlegs, const int32_t* nsect,
                       const int32_t* charges, const int64_t* dims, const int32_t* isdual,
                       mpsg_tensor** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(out, "out");
    auto sp = parse_spaces(nlegs, nsect, charges, dims, isdual);
    auto meta = mpsg::TensorMeta::build(charge, sp);
    *out = wrap(mpsg::new_tensor(&ctx->c, meta, /*zero=*/true));
  });
}

int mpsg_tensor_free(mpsg_tensor* t) {
  return guarded([&] { delete t; });
}

int mpsg_tensor_rank(const mpsg_tensor* t, int32_t* n) {
  return guarded([&] {
    need(t, "t");
    need(n, "n");
    *n = t->t.meta.N();
  });
}

int mpsg_tensor_charge(const mpsg_tensor* t, int32_t* c) {
  return guarded([&] {
    need(t, "t");
    need(c, "c");
    *c = t->t.meta.charge;
  });
}

int mpsg_tensor_numel(const mpsg_tensor* t, int64_t* nb, int64_t* ne) {
  return guarded([&] {
    need(t, "t");
    if (nb) *nb = (int64_t)t->t.meta.nblocks();
    if (ne) *ne = t->t.meta.total;
  });
}

int mpsg_tensor_is_diagonal(const mpsg_tensor* t, int32_t* d) {
  return guarded([&] {
    need(t, "t");
    need(d, "d");
    *d = t->t.diag ? 1 : 0;
  });
}

int mpsg_tensor_space(const mpsg_tensor* t, int32_t leg, int32_t* nsect, int32_t* charges,
                      int64_t* dims, int32_t* isdual) {
  return guarded([&] {
    need(t, "t");
    if (leg < 1 || leg > t->t.meta.N()) throw mpsg::Error(mpsg::kErrArgument, "leg out of range");
    const mpsg::Space& V = t->t.meta.space[leg - 1];
    if (nsect) *nsect = V.size();
    if (isdual) *isdual = V.dual ? 1 : 0;
    for (int i = 0; i < V.size(); ++i) {
      if (charges) charges[i] = V.ch[i];
      if (dims) dims[i] = V.dm[i];
    }
  });
}

int mpsg_tensor_sectors(const mpsg_tensor* t, int32_t* labels, int64_t* sizes, int64_t* offsets) {
  return guarded([&] {
    need(t, "t");
    const auto& m = t->t.meta;
    if (labels)
      for (size_t i = 0; i < m.sec.lab.size(); ++i) labels[i] = m.sec.lab[i];
    if (sizes) std::memcpy(sizes, m.sec.sz.data(), sizeof(int64_t) * m.sec.sz.size());
    if (offsets) std::memcpy(offsets, m.off.data(), sizeof(int64_t) * m.off.size());
  });
}

int mpsg_tensor_upload(mpsg_tensor* t, const double* host, int64_t n) {
  return guarded([&] {
    need(t, "t");
    if (n != t->t.meta.total) throw mpsg::Error(mpsg::kErrArgument, "upload: size mismatch");
    if (n == 0) return;
    need(host, "host");
    MPSG_CUDA(cudaMemcpyAsync(t->t.data(), host, sizeof(double) * n, cudaMemcpyHostToDevice,
                              t->t.ctx->stream));
    MPSG_CUDA(cudaStreamSynchronize(t->t.ctx->stream));
  });
}

int mpsg_tensor_download(const mpsg_tensor* t, double* host, int64_t n) {
  return guarded([&] {
    need(t, "t");
    if (n != t->t.meta.total) throw mpsg::Error(mpsg::kErrArgument, "download: size mismatch");
    if (n == 0) return;
    need(host, "host");
    MPSG_CUDA(cudaMemcpyAsync(host, t->t.data(), sizeof(double) * n, cudaMemcpyDeviceToHost,
                              t->t.ctx->stream));
    MPSG_CUDA(cudaStreamSynchronize(t->t.ctx->stream));
  });
}

int mpsg_device_checks(mpsg_ctx* ctx, int32_t reset, int64_t* violations, int64_t* first) {
  return guarded([&] {
#ifdef MPSG_DEVICE_CHECKS
    need(ctx, "ctx");
#endif
    mpsg::read_device_checks(ctx ? &ctx->c : nullptr, reset != 0, violations, first);
  });
}

struct mpsg_copy {
  std::unique_ptr<mpsg::AsyncCopy> c;
};

int mpsg_host_alloc(int64_t n, double** host) {
  return guarded([&] {
    need(host, "host");
    if (n < 0) throw mpsg::Error(mpsg::kErrArgument, "host_alloc: negative size");
    *host = nullptr;
    MPSG_CUDA(cudaMallocHost((void**)host, sizeof(double) * (size_t)std::max<int64_t>(n, 1)));
  });
}

int mpsg_host_free(double* host) {
  return guarded([&] {
    if (host) MPSG_CUDA(cudaFreeHost(host));
  });
}

static void check_async_args(mpsg_ctx* ctx, const mpsg_tensor* t, const void* host, int64_t n,
                             mpsg_copy** copy) {
  need(ctx, "ctx");
  need(t, "t");
  need(copy, "copy");
  if (t->t.ctx != &ctx->c)
    throw mpsg::Error(mpsg::kErrArgument, "async copy: tensor belongs to another context");
  if (n != t->t.meta.total) throw mpsg::Error(mpsg::kErrArgument, "async copy: size mismatch");
  if (n) need(host, "host");
}

int mpsg_tensor_download_async(mpsg_ctx* ctx, const mpsg_tensor* t, double* host, int64_t n,
                               mpsg_copy** copy) {
  return guarded([&] {
    check_async_args(ctx, t, host, n, copy);
    auto c = mpsg::copy_async(&ctx->c, t->t, host, /*to_host=*/true);
    *copy = new mpsg_copy{std::move(c)};
  });
}

int mpsg_tensor_upload_async(mpsg_ctx* ctx, mpsg_tensor* t, const double* host, int64_t n,
                             mpsg_copy** copy) {
  return guarded([&] {
    check_async_args(ctx, t, host, n, copy);
    auto c = mpsg::copy_async(&ctx->c, t->t, const_cast<double*>(host), /*to_host=*/false);
    *copy = new mpsg_copy{std::move(c)};
  });
}

int mpsg_copy_wait(mpsg_ctx* ctx, mpsg_copy* copy) {
  return guarded([&] {
    need(ctx, "ctx");
    need(copy, "copy");
    MPSG_CUDA(cudaStreamWaitEvent(ctx->c.stream, copy->c->done, 0));
  });
}

int mpsg_copy_query(mpsg_copy* copy, int32_t* done) {
  return guarded([&] {
    need(copy, "copy");
    need(done, "done");
    cudaError_t e = cudaEventQuery(copy->c->done);
    if (e == cudaErrorNotReady) {
      (void)cudaGetLastError();  // not an error: the copy is still running
      *done = 0;
      return;
    }
    MPSG_CUDA(e);
    *done = 1;
  });
}

int mpsg_copy_synchronize(mpsg_copy* copy) {
  return guarded([&] {
    need(copy, "copy");
    MPSG_CUDA(cudaEventSynchronize(copy->c->done));
  });
}

int mpsg_copy_free(mpsg_copy* copy) {
  return guarded([&] { delete copy; });
}

int mpsg_tensor_device_ptr(const mpsg_tensor* t, double** p) {
  return guarded([&] {
    need(t, "t");
    need(p, "p");
    *p = t->t.data();
  });
}

int mpsg_tensor_copy(mpsg_ctx* ctx, const mpsg_tensor* t, mpsg_tensor** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(t, "t");
    need(out, "out");
    *out = wrap(mpsg::copy_tensor(&ctx->c, t->t));
  });
}

int mpsg_dual(mpsg_ctx* ctx, const mpsg_tensor* a, mpsg_tensor** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(out, "out");
    *out = wrap(mpsg::dual_view(a->t));
  });
}

int mpsg_permutelegs(mpsg_ctx* ctx, const mpsg_tensor* a, const int32_t* perm,
                     mpsg_tensor** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(perm, "perm");
    need(out, "out");
    *out = wrap(mpsg::permutelegs(&ctx->c, a->t, ivec(perm, a->t.meta.N())));
  });
}

int mpsg_fuselegs(mpsg_ctx* ctx, const mpsg_tensor* a, int32_t l, int32_t n, int32_t dual,
                  mpsg_tensor** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(out, "out");
    *out = wrap(mpsg::fuselegs(&ctx->c, a->t, l, n, dual != 0));
  });
}

int mpsg_splitleg(mpsg_ctx* ctx, const mpsg_tensor* a, int32_t l, int32_t nspaces,
                  const int32_t* nsect, const int32_t* charges, const int64_t* dims,
                  const int32_t* isdual, mpsg_tensor** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(out, "out");
    auto sp = parse_spaces(nspaces, nsect, charges, dims, isdual);
    *out = wrap(mpsg::splitleg(&ctx->c, a->t, l, sp));
  });
}

int mpsg_symmatrix(mpsg_ctx* ctx, const mpsg_tensor* a, int32_t nrows, const int32_t* rows,
                   int32_t ncols, const int32_t* cols, mpsg_tensor** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(out, "out");
    if (nrows < 0 || ncols < 0) throw mpsg::Error(mpsg::kErrArgument, "negative count");
    std::vector<int> r = nrows ? ivec(rows, nrows) : std::vector<int>();
    std::vector<int> c = ncols ? ivec(cols, ncols) : std::vector<int>();
    *out = wrap(mpsg::symmatrix(&ctx->c, a->t, r, c));
  });
}

int mpsg_matmul(mpsg_ctx* ctx, const mpsg_tensor* a, const mpsg_tensor* b, int32_t precision,
                mpsg_tensor** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(b, "b");
    need(out, "out");
    *out = wrap(mpsg::matmul(&ctx->c, a->t, b->t, precision));
  });
}

int mpsg_contract(mpsg_ctx* ctx, const mpsg_tensor* a, const int32_t* idxa, const mpsg_tensor* b,
                  const int32_t* idxb, int32_t precision, mpsg_tensor** out, double* scalar) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(b, "b");
    need(idxa, "idxa");
    need(idxb, "idxb");
    need(out, "out");
    double s = 0.0;
    mpsg::DeviceTensor r = mpsg::contract(&ctx->c, a->t, ivec(idxa, a->t.meta.N()), b->t,
                                          ivec(idxb, b->t.meta.N()), precision, &s);
    if (!r.buf && r.meta.space.empty()) {
      *out = nullptr;
      if (scalar) *scalar = s;
    } else {
      *out = wrap(std::move(r));
    }
  });
}

int mpsg_contract_complex(mpsg_ctx* ctx, const mpsg_tensor* ar, const mpsg_tensor* ai,
                          double sa, const int32_t* idxa, const mpsg_tensor* br,
                          const mpsg_tensor* bi, double sb, const int32_t* idxb,
                          int32_t precision, mpsg_tensor** cr, mpsg_tensor** ci,
                          double* scalar_re, double* scalar_im) {
  return guarded([&] {
    need(ctx, "ctx");
    need(ar, "ar");
    need(br, "br");
    need(idxa, "idxa");
    need(idxb, "idxb");
    need(cr, "cr");
    need(ci, "ci");
    if (ai) mpsg::require_similar(ar->t, ai->t, "real and imaginary parts differ in structure");
    if (bi) mpsg::require_similar(br->t, bi->t, "real and imaginary parts differ in structure");
    mpsg::Context* c = &ctx->c;
    const auto ia = ivec(idxa, ar->t.meta.N());
    const auto ib = ivec(idxb, br->t.meta.N());
    double srr = 0, sri = 0, sir = 0, sii = 0;
    mpsg::DeviceTensor rr = mpsg::contract(c, ar->t, ia, br->t, ib, precision, &srr);
    mpsg::DeviceTensor ri, ir, ii;
    if (bi) ri = mpsg::contract(c, ar->t, ia, bi->t, ib, precision, &sri);
    if (ai) ir = mpsg::contract(c, ai->t, ia, br->t, ib, precision, &sir);
    if (ai && bi) ii = mpsg::contract(c, ai->t, ia, bi->t, ib, precision, &sii);
    if (!rr.buf && rr.meta.space.empty()) {  // every leg contracted: a complex number
      *cr = nullptr;
      *ci = nullptr;
      if (scalar_re) *scalar_re = srr - sa * sb * sii;
      if (scalar_im) *scalar_im = sb * sri + sa * sir;
      return;
    }
    const int64_t n = rr.meta.total;
    // re = rr - sa sb ii, im = sb ri + sa ir, both formed in place in one launch each
    if (ai && bi) mpsg::launch_lincomb(c, n, {rr.data(), ii.data()}, {1.0, -sa * sb}, rr.data());
    *cr = wrap(std::move(rr));
    if (ri.buf && ir.buf) {
      mpsg::launch_lincomb(c, n, {ri.data(), ir.data()}, {sb, sa}, ri.data());
      *ci = wrap(std::move(ri));
    } else if (ri.buf) {
      if (sb != 1.0) mpsg::launch_lincomb(c, n, {ri.data()}, {sb}, ri.data());
      *ci = wrap(std::move(ri));
    } else if (ir.buf) {
      if (sa != 1.0) mpsg::launch_lincomb(c, n, {ir.data()}, {sa}, ir.data());
      *ci = wrap(std::move(ir));
    } else {
      *ci = nullptr;
    }
  });
}

int mpsg_contract_flops(mpsg_ctx* ctx, const mpsg_tensor* a, const int32_t* idxa,
                        const mpsg_tensor* b, const int32_t* idxb, double* flops) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(b, "b");
    need(flops, "flops");
    auto p = mpsg::get_contract_plan(&ctx->c, a->t.meta, ivec(idxa, a->t.meta.N()), b->t.meta,
                                     ivec(idxb, b->t.meta.N()));
    *flops = p->host->flops;
  });
}

int mpsg_applymps2site(mpsg_ctx* ctx, const mpsg_tensor* v, const mpsg_tensor* envl,
                       const mpsg_tensor* envr, const mpsg_tensor* w1, const mpsg_tensor* w2,
                       int32_t precision, mpsg_tensor** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(v, "v");
    need(envl, "envl");
    need(envr, "envr");
    need(w1, "w1");
    need(w2, "w2");
    need(out, "out");
    *out = wrap(mpsg::applymps2site(&ctx->c, v->t, envl->t, envr->t, w1->t, w2->t, precision));
  });
}

int mpsg_applymps2site_host(mpsg_ctx* ctx, mpsg_tensor* v, mpsg_tensor* envl, mpsg_tensor* envr,
                            mpsg_tensor* w1, mpsg_tensor* w2, const double* hv,
                            const double* henvl, const double* henvr, const double* hw1,
                            const double* hw2, int32_t precision, double* hout,
                            mpsg_tensor** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(v, "v");
    need(envl, "envl");
    need(envr, "envr");
    need(w1, "w1");
    need(w2, "w2");
    need(hout, "hout");
    const double* hin[5] = {hv, henvl, henvr, hw1, hw2};
    const mpsg_tensor* ts[5] = {v, envl, envr, w1, w2};
    for (int i = 0; i < 5; ++i)
      if (ts[i]->t.meta.total) need(hin[i], "host input");
    auto r = mpsg::applymps2site_host(&ctx->c, v->t, envl->t, envr->t, w1->t, w2->t, hin,
                                      precision, hout);
    if (out) *out = wrap(std::move(r));
  });
}

int mpsg_applymps2site_flops(mpsg_ctx* ctx, const mpsg_tensor* v, const mpsg_tensor* envl,
                             const mpsg_tensor* envr, const mpsg_tensor* w1,
                             const mpsg_tensor* w2, double* flops) {
  return guarded([&] {
    need(ctx, "ctx");
    need(v, "v");
    need(envl, "envl");
    need(envr, "envr");
    need(w1, "w1");
    need(w2, "w2");
    need(flops, "flops");
    *flops = mpsg::applymps2site_flops(&ctx->c, v->t.meta, envl->t.meta, envr->t.meta,
                                       w1->t.meta, w2->t.meta);
  });
}

int mpsg_mpsupdateleft(mpsg_ctx* ctx, const mpsg_tensor* env, const mpsg_tensor* a,
                       const mpsg_tensor* w, int32_t precision, mpsg_tensor** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(env, "env");
    need(a, "a");
    need(w, "w");
    need(out, "out");
    *out = wrap(mpsg::mpsupdateleft(&ctx->c, env->t, a->t, w->t, precision));
  });
}

int mpsg_mpsupdateright(mpsg_ctx* ctx, const mpsg_tensor* env, const mpsg_tensor* a,
                        const mpsg_tensor* w, int32_t precision, mpsg_tensor** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(env, "env");
    need(a, "a");
    need(w, "w");
    need(out, "out");
    *out = wrap(mpsg::mpsupdateright(&ctx->c, env->t, a->t, w->t, precision));
  });
}

int mpsg_svd(mpsg_ctx* ctx, const mpsg_tensor* a, mpsg_tensor** u, mpsg_tensor** s,
             mpsg_tensor** v) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(u, "u");
    need(s, "s");
    need(v, "v");
    auto R = mpsg::svd_blocks(&ctx->c, a->t, false, 0, 0.0, 0.0);
    *u = wrap(std::move(R.u));
    *s = wrap(std::move(R.s));
    *v = wrap(std::move(R.v));
  });
}

int mpsg_svdtrunc(mpsg_ctx* ctx, const mpsg_tensor* a, int64_t maxdim, double tol,
                  double tieband, mpsg_tensor** u, mpsg_tensor** s, mpsg_tensor** v) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(u, "u");
    need(s, "s");
    need(v, "v");
    auto R = mpsg::svd_blocks(&ctx->c, a->t, true, maxdim, tol, tieband);
    *u = wrap(std::move(R.u));
    *s = wrap(std::move(R.s));
    *v = wrap(std::move(R.v));
  });
}

int mpsg_svdtrunc_gram(mpsg_ctx* ctx, const mpsg_tensor* a, int64_t maxdim, double tol,
                       double tieband, int32_t side, mpsg_tensor** u, mpsg_tensor** s,
                       mpsg_tensor** v) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(u, "u");
    need(s, "s");
    need(v, "v");
    if (side != 0 && side != 1) throw mpsg::Error(mpsg::kErrArgument, "side must be 0 or 1");
    auto R = mpsg::svd_blocks(&ctx->c, a->t, true, maxdim, tol, tieband,
                              side == 0 ? mpsg::kSvdGramLeft : mpsg::kSvdGramRight);
    *u = wrap(std::move(R.u));
    *s = wrap(std::move(R.s));
    *v = wrap(std::move(R.v));
  });
}

int mpsg_svd_complex(mpsg_ctx* ctx, const mpsg_tensor* a_re, const mpsg_tensor* a_im,
                     int32_t truncate, int64_t maxdim, double tol, double tieband,
                     mpsg_tensor** u_re, mpsg_tensor** u_im, mpsg_tensor** s,
                     mpsg_tensor** v_re, mpsg_tensor** v_im) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a_re, "a_re");
    need(a_im, "a_im");
    need(u_re, "u_re");
    need(u_im, "u_im");
    need(s, "s");
    need(v_re, "v_re");
    need(v_im, "v_im");
    auto R = mpsg::svd_blocks_complex(&ctx->c, a_re->t, a_im->t, truncate != 0, maxdim, tol,
                                      tieband);
    *u_re = wrap(std::move(R.ure));
    *u_im = wrap(std::move(R.uim));
    *s = wrap(std::move(R.s));
    *v_re = wrap(std::move(R.vre));
    *v_im = wrap(std::move(R.vim));
  });
}

int mpsg_truncatedsizes(int32_t nsect, const int64_t* lens, const double* values, int64_t maxdim,
                        double tol, double tieband, int64_t* ns) {
  return guarded([&] {
    need(lens, "lens");
    need(values, "values");
    need(ns, "ns");
    if (nsect < 1) throw mpsg::Error(mpsg::kErrArgument, "no sectors");
    std::vector<std::vector<double>> S(nsect);
    int64_t p = 0;
    for (int i = 0; i < nsect; ++i) {
      if (lens[i] < 1) throw mpsg::Error(mpsg::kErrArgument, "empty sector");
      S[i].assign(values + p, values + p + lens[i]);
      p += lens[i];
    }
    auto r = mpsg::truncatedsizes(S, maxdim, tol, tieband);
    for (int i = 0; i < nsect; ++i) ns[i] = r[i];
  });
}

int mpsg_small_eigh(int32_t n, const double* a, double* evals, double* evecs) {
  return guarded([&] {
    need(a, "a");
    need(evals, "evals");
    need(evecs, "evecs");
    if (n < 1) throw mpsg::Error(mpsg::kErrArgument, "n < 1");
    mpsg::small_eigh(n, a, evals, evecs);
  });
}

int mpsg_eigsolve_heff2(mpsg_ctx* ctx, const mpsg_tensor* x0, const mpsg_tensor* envl,
                        const mpsg_tensor* envr, const mpsg_tensor* w1, const mpsg_tensor* w2,
                        int32_t krylovdim, int32_t maxiter, double tol, int32_t precision,
                        double* eigenvalue, mpsg_tensor** eigenvector, double* normres,
                        int32_t* numiter, int32_t* numops, int32_t* converged) {
  return guarded([&] {
    need(ctx, "ctx");
    need(x0, "x0");
    need(envl, "envl");
    need(envr, "envr");
    need(w1, "w1");
    need(w2, "w2");
    need(eigenvalue, "eigenvalue");
    need(eigenvector, "eigenvector");
    auto R = mpsg::eigsolve_heff2(&ctx->c, x0->t, envl->t, envr->t, w1->t, w2->t, krylovdim,
                                  maxiter, tol, precision);
    *eigenvalue = R.value;
    *eigenvector = wrap(std::move(R.vec));
    if (normres) *normres = R.normres;
    if (numiter) *numiter = R.numiter;
    if (numops) *numops = R.numops;
    if (converged) *converged = R.converged ? 1 : 0;
  });
}

struct mpsg_heff {
  std::shared_ptr<mpsg::HeffOp> op;
};

int mpsg_heff2_create(mpsg_ctx* ctx, const mpsg_tensor* v_like, const mpsg_tensor* envl,
                      const mpsg_tensor* envr, const mpsg_tensor* w1, const mpsg_tensor* w2,
                      int32_t precision, mpsg_heff** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(v_like, "v_like");
    need(envl, "envl");
    need(envr, "envr");
    need(w1, "w1");
    need(w2, "w2");
    need(out, "out");
    auto h = new mpsg_heff;
    try {
      h->op = mpsg::heff_create(&ctx->c, v_like->t.meta, envl->t, envr->t, w1->t, w2->t,
                                precision);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

int mpsg_heff2_apply(mpsg_ctx* ctx, mpsg_heff* op, const mpsg_tensor* v, mpsg_tensor** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(op, "op");
    need(v, "v");
    need(out, "out");
    *out = wrap(mpsg::heff_apply(*op->op, v->t));
  });
}

int mpsg_heff2_flops(const mpsg_heff* op, double* flops) {
  return guarded([&] {
    need(op, "op");
    need(flops, "flops");
    *flops = op->op->ref_flops;
  });
}

int mpsg_heff2_traffic(const mpsg_heff* op, double* copy_bytes, double* pack_bytes) {
  return guarded([&] {
    need(op, "op");
    if (copy_bytes) *copy_bytes = op->op->copy_bytes;
    if (pack_bytes) *pack_bytes = op->op->pack_bytes;
  });
}

int mpsg_heff2_free(mpsg_heff* op) {
  return guarded([&] { delete op; });
}

struct mpsg_heff_batch {
  std::shared_ptr<mpsg::Context> owner;  // the batch's buffers hold it too
  std::unique_ptr<mpsg::HeffBatch> b;
};

int mpsg_heff2_batch_create(mpsg_ctx* ctx, int32_t n, const mpsg_tensor* const* v_like,
                            const mpsg_tensor* const* envl, const mpsg_tensor* const* envr,
                            const mpsg_tensor* const* w1, const mpsg_tensor* const* w2,
                            int32_t precision, int32_t use_graph, mpsg_heff_batch** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(out, "out");
    if (n < 1) throw mpsg::Error(mpsg::kErrArgument, "a batch needs at least one operator");
    for (auto* p : {(const void*)v_like, (const void*)envl, (const void*)envr, (const void*)w1,
                    (const void*)w2})
      need(p, "operand list");
    std::vector<mpsg::TensorMeta> vm;
    std::vector<const mpsg::DeviceTensor*> L, R, A, B;
    for (int i = 0; i < n; ++i) {
      for (const mpsg_tensor* t : {v_like[i], envl[i], envr[i], w1[i], w2[i]}) need(t, "operand");
      vm.push_back(v_like[i]->t.meta);
      L.push_back(&envl[i]->t);
      R.push_back(&envr[i]->t);
      A.push_back(&w1[i]->t);
      B.push_back(&w2[i]->t);
    }
    auto h = std::make_unique<mpsg_heff_batch>();
    h->owner = ctx->owner;
    h->b = mpsg::heff_batch_create(&ctx->c, vm, L, R, A, B, precision, use_graph != 0);
    *out = h.release();
  });
}

int mpsg_heff2_prepare(mpsg_ctx* ctx, const mpsg_tensor* v_like, const mpsg_tensor* envl,
                       const mpsg_tensor* envr, const mpsg_tensor* w1, const mpsg_tensor* w2,
                       int32_t precision, mpsg_heff** out) {
  return guarded([&] {
    need(ctx, "ctx");
    for (const void* p : {(const void*)v_like, (const void*)envl, (const void*)envr,
                          (const void*)w1, (const void*)w2, (const void*)out})
      need(p, "argument");
    auto h = std::make_unique<mpsg_heff>();
    h->op = mpsg::heff_prepare(&ctx->c, v_like->t.meta, envl->t, envr->t, w1->t, w2->t,
                               precision);
    *out = h.release();
  });
}

int mpsg_heff2_batch_from(mpsg_ctx* ctx, int32_t n, const mpsg_heff* const* ops,
                          int32_t use_graph, mpsg_heff_batch** out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(ops, "ops");
    need(out, "out");
    if (n < 1) throw mpsg::Error(mpsg::kErrArgument, "a batch needs at least one operator");
    std::vector<const mpsg::HeffOp*> v;
    for (int i = 0; i < n; ++i) {
      need(ops[i], "ops[i]");
      v.push_back(ops[i]->op.get());
    }
    auto h = std::make_unique<mpsg_heff_batch>();
    h->owner = ctx->owner;
    h->b = mpsg::heff_batch_from_ops(&ctx->c, v, use_graph != 0);
    *out = h.release();
  });
}

int mpsg_heff2_batch_apply(mpsg_heff_batch* b, const mpsg_tensor* const* v, mpsg_tensor** out) {
  return guarded([&] {
    need(b, "b");
    need(v, "v");
    need(out, "out");
    mpsg::HeffBatch& B = *b->b;
    mpsg::Context* c = B.ctx;
    for (int i = 0; i < B.n; ++i) {
      need(v[i], "v[i]");
      if (!v[i]->t.ctx || v[i]->t.ctx->device != c->device)
        throw mpsg::Error(mpsg::kErrArgument, "batch: tensor on another device");
      if (!mpsg::same_meta(v[i]->t.meta, B.vmeta[i]))
        throw mpsg::Error(mpsg::kErrSpaceMismatch, "batch: tensor of another structure");
    }
    for (int i = 0; i < B.n; ++i)
      MPSG_CUDA(cudaMemcpyAsync(B.vin->ptr + B.voff[i], v[i]->t.data(),
                                sizeof(double) * B.vmeta[i].total, cudaMemcpyDeviceToDevice,
                                c->stream));
    B.apply();
    for (int i = 0; i < B.n; ++i) {
      mpsg::DeviceTensor t = mpsg::new_tensor(c, B.vmeta[i], false);
      MPSG_CUDA(cudaMemcpyAsync(t.data(), B.vout->ptr + B.voff[i],
                                sizeof(double) * B.vmeta[i].total, cudaMemcpyDeviceToDevice,
                                c->stream));
      out[i] = wrap(std::move(t));
    }
  });
}

int mpsg_heff2_batch_eigsolve(mpsg_heff_batch* b, const mpsg_tensor* const* x0, int32_t krylovdim,
                              int32_t maxiter, double tol, double* eigenvalues,
                              mpsg_tensor** eigenvectors, double* normres, int32_t* numiter,
                              int32_t* numops, int32_t* converged) {
  return guarded([&] {
    need(b, "b");
    need(x0, "x0");
    need(eigenvalues, "eigenvalues");
    need(eigenvectors, "eigenvectors");
    std::vector<const mpsg::DeviceTensor*> xs;
    for (int i = 0; i < b->b->n; ++i) {
      need(x0[i], "x0[i]");
      xs.push_back(&x0[i]->t);
    }
    auto R = mpsg::eigsolve_heff2_batch(*b->b, xs, krylovdim, maxiter, tol);
    for (int i = 0; i < b->b->n; ++i) {
      eigenvalues[i] = R[i].value;
      eigenvectors[i] = wrap(std::move(R[i].vec));
      if (normres) normres[i] = R[i].normres;
      if (numiter) numiter[i] = R[i].numiter;
      if (numops) numops[i] = R[i].numops;
      if (converged) converged[i] = R[i].converged ? 1 : 0;
    }
  });
}

int mpsg_heff2_batch_info(const mpsg_heff_batch* b, double* ref_flops, int64_t* graph_kernels,
                          int64_t* applies, int32_t* tuning) {
  return guarded([&] {
    need(b, "b");
    const mpsg::HeffBatch& B = *b->b;
    if (ref_flops) *ref_flops = B.ref_flops;
    if (graph_kernels) *graph_kernels = B.exec ? B.graph_kernels : 0;
    if (applies) *applies = B.applies;
    if (tuning) {
      tuning[0] = B.t1.bn;
      tuning[1] = B.t1.order;
      tuning[2] = B.t2.bn;
      tuning[3] = B.t2.order;
    }
  });
}

int mpsg_heff2_batch_free(mpsg_heff_batch* b) {
  return guarded([&] { delete b; });
}

int mpsg_ctx_tuner(mpsg_ctx* ctx, int32_t enable, int64_t* runs, int64_t* hits) {
  return guarded([&] {
    need(ctx, "ctx");
    if (enable == 0 || enable == 1) ctx->c.autotune = enable != 0;
    if (runs) *runs = ctx->c.tune_runs;
    if (hits) *hits = ctx->c.tune_hits;
  });
}

int mpsg_ctx_set_split_tuning(mpsg_ctx* ctx, int32_t bn, int32_t order, int32_t splitk) {
  return guarded([&] {
    need(ctx, "ctx");
    if (bn < 0) {
      ctx->c.forced_bn = ctx->c.forced_order = -1;
      ctx->c.forced_splitk = 0;
      return;
    }
    if (bn != 0 && bn != 64 && bn != 128)
      throw mpsg::Error(mpsg::kErrArgument, "split GEMM N tile must be 0, 64 or 128");
    if (order != 0 && order != 1) throw mpsg::Error(mpsg::kErrArgument, "tile order must be 0 or 1");
    if (splitk != 0 && splitk != 1) throw mpsg::Error(mpsg::kErrArgument, "split-K must be 0 or 1");
    ctx->c.forced_bn = bn;
    ctx->c.forced_order = order;
    ctx->c.forced_splitk = splitk;
  });
}

int mpsg_plan_heff2_check(const mpsg_tensor* v, const mpsg_tensor* envl, const mpsg_tensor* envr,
                          const mpsg_tensor* w1, const mpsg_tensor* w2) {
  return guarded([&] {
    need(v, "v");
    need(envl, "envl");
    need(envr, "envr");
    need(w1, "w1");
    need(w2, "w2");
    mpsg::check_heff_folded(v->t.meta, envl->t.meta, envr->t.meta, w1->t.meta, w2->t.meta);
  });
}

static mpsg_tensor* meta_only(const mpsg::TensorMeta& m) {
  mpsg::DeviceTensor t;
  t.meta = m;
  return wrap(std::move(t));
}

int mpsg_meta_create(int32_t charge, int32_t nlegs, const int32_t* nsect, const int32_t* charges,
                     const int64_t* dims, const int32_t* isdual, mpsg_tensor** out) {
  return guarded([&] {
    need(out, "out");
    auto sp = parse_spaces(nlegs, nsect, charges, dims, isdual);
    *out = meta_only(mpsg::TensorMeta::build(charge, sp));
  });
}

int mpsg_plan_permutelegs(const mpsg_tensor* a, const int32_t* perm, mpsg_tensor** out) {
  return guarded([&] {
    need(a, "a");
    need(perm, "perm");
    need(out, "out");
    auto p = mpsg::plan_permutelegs(a->t.meta, ivec(perm, a->t.meta.N()));
    mpsg::validate_copy_tasks(p.tasks, a->t.meta.total, p.out.total);
    *out = meta_only(p.out);
  });
}

int mpsg_plan_fuselegs(const mpsg_tensor* a, int32_t l, int32_t n, int32_t dual,
                       mpsg_tensor** out) {
  return guarded([&] {
    need(a, "a");
    need(out, "out");
    auto p = mpsg::plan_fuselegs(a->t.meta, l, n, dual != 0);
    mpsg::validate_copy_tasks(p.tasks, a->t.meta.total, p.out.total);
    *out = meta_only(p.out);
  });
}

int mpsg_plan_splitleg(const mpsg_tensor* a, int32_t l, int32_t nspaces, const int32_t* nsect,
                       const int32_t* charges, const int64_t* dims, const int32_t* isdual,
                       mpsg_tensor** out) {
  return guarded([&] {
    need(a, "a");
    need(out, "out");
    auto sp = parse_spaces(nspaces, nsect, charges, dims, isdual);
    auto p = mpsg::plan_splitleg(a->t.meta, l, sp);
    mpsg::validate_copy_tasks(p.tasks, a->t.meta.total, p.out.total);
    *out = meta_only(p.out);
  });
}

int mpsg_plan_symmatrix(const mpsg_tensor* a, int32_t nrows, const int32_t* rows, int32_t ncols,
                        const int32_t* cols, mpsg_tensor** out) {
  return guarded([&] {
    need(a, "a");
    need(out, "out");
    if (nrows < 0 || ncols < 0) throw mpsg::Error(mpsg::kErrArgument, "negative count");
    std::vector<int> r = nrows ? ivec(rows, nrows) : std::vector<int>();
    std::vector<int> c = ncols ? ivec(cols, ncols) : std::vector<int>();
    auto p = mpsg::plan_symmatrix(a->t.meta, r, c);
    mpsg::validate_copy_tasks(p.tasks, a->t.meta.total, p.out.total);
    *out = meta_only(p.out);
  });
}

int mpsg_plan_matmul(const mpsg_tensor* a, const mpsg_tensor* b, mpsg_tensor** out,
                     double* flops) {
  return guarded([&] {
    need(a, "a");
    need(b, "b");
    need(out, "out");
    auto p = mpsg::plan_matmul(a->t.meta, b->t.meta);
    mpsg::validate_gemms(p.gemms, a->t.meta.total, b->t.meta.total, p.out.total);
    if (flops) *flops = p.flops;
    *out = meta_only(p.out);
  });
}

int mpsg_plan_contract(const mpsg_tensor* a, const int32_t* idxa, const mpsg_tensor* b,
                       const int32_t* idxb, mpsg_tensor** out, double* flops) {
  return guarded([&] {
    need(a, "a");
    need(b, "b");
    need(idxa, "idxa");
    need(idxb, "idxb");
    need(out, "out");
    auto p = mpsg::plan_contract(a->t.meta, ivec(idxa, a->t.meta.N()), b->t.meta,
                                 ivec(idxb, b->t.meta.N()));
    mpsg::validate_contract(*p, a->t.meta, b->t.meta);
    if (flops) *flops = p->flops;
    *out = p->scalar ? nullptr : meta_only(p->split.out);
  });
}

int mpsg_plan_contract_gemms(const mpsg_tensor* a, const int32_t* idxa, const mpsg_tensor* b,
                             const int32_t* idxb, int64_t* count, int64_t* mnk) {
  return guarded([&] {
    need(a, "a");
    need(b, "b");
    need(idxa, "idxa");
    need(idxb, "idxb");
    need(count, "count");
    auto p = mpsg::plan_contract(a->t.meta, ivec(idxa, a->t.meta.N()), b->t.meta,
                                 ivec(idxb, b->t.meta.N()));
    *count = (int64_t)p->mm.gemms.size();
    if (mnk)
      for (size_t i = 0; i < p->mm.gemms.size(); ++i) {
        mnk[3 * i] = p->mm.gemms[i].M;
        mnk[3 * i + 1] = p->mm.gemms[i].N;
        mnk[3 * i + 2] = p->mm.gemms[i].K;
      }
  });
}

int mpsg_plan_contract_tasks(const mpsg_tensor* a, const int32_t* idxa, const mpsg_tensor* b,
                             const int32_t* idxb, int64_t* copy_tasks, int64_t* gemm_tasks) {
  return guarded([&] {
    need(a, "a");
    need(b, "b");
    need(idxa, "idxa");
    need(idxb, "idxb");
    auto p = mpsg::plan_contract(a->t.meta, ivec(idxa, a->t.meta.N()), b->t.meta,
                                 ivec(idxb, b->t.meta.N()));
    if (copy_tasks)
      *copy_tasks = (int64_t)(p->fa.tasks.size() + p->fb.tasks.size() + p->split.tasks.size());
    if (gemm_tasks) *gemm_tasks = (int64_t)p->mm.gemms.size();
  });
}

int mpsg_fill(mpsg_ctx* ctx, mpsg_tensor* a, double x) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    mpsg::launch_fill(&ctx->c, a->t.data(), a->t.meta.total, x);
  });
}

int mpsg_rmul(mpsg_ctx* ctx, mpsg_tensor* a, double alpha) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    mpsg::launch_scale(&ctx->c, a->t.meta.total, alpha, a->t.data(), a->t.data());
  });
}

int mpsg_mul(mpsg_ctx* ctx, mpsg_tensor* b, const mpsg_tensor* a, double alpha) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(b, "b");
    mpsg::require_similar(a->t, b->t, "oops");
    mpsg::launch_scale(&ctx->c, a->t.meta.total, alpha, a->t.data(), b->t.data());
  });
}

int mpsg_axpy(mpsg_ctx* ctx, double alpha, const mpsg_tensor* a, mpsg_tensor* b) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(b, "b");
    mpsg::require_similar(a->t, b->t, "axpy! The two matrices are not simliar!");
    mpsg::launch_axpby(&ctx->c, a->t.meta.total, alpha, a->t.data(), 1.0, b->t.data());
  });
}

int mpsg_axpby(mpsg_ctx* ctx, double alpha, const mpsg_tensor* a, double beta, mpsg_tensor* b) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(b, "b");
    mpsg::require_similar(a->t, b->t, "axpy! The two matrices are not simliar!");
    mpsg::launch_axpby(&ctx->c, a->t.meta.total, alpha, a->t.data(), beta, b->t.data());
  });
}

int mpsg_dots(mpsg_ctx* ctx, int32_t n, const mpsg_tensor* const* a,
              const mpsg_tensor* const* b, double* out) {
  return guarded([&] {
    need(ctx, "ctx");
    if (n < 0) throw mpsg::Error(mpsg::kErrArgument, "negative count");
    if (n == 0) return;
    need(a, "a");
    need(b, "b");
    need(out, "out");
    std::vector<mpsg::VecPair> pairs((size_t)n);
    for (int32_t i = 0; i < n; ++i) {
      need(a[i], "a[i]");
      need(b[i], "b[i]");
      mpsg::require_similar(a[i]->t, b[i]->t, "The two SymTensors have to be similar to dot!");
      pairs[i] = {a[i]->t.data(), b[i]->t.data(), a[i]->t.meta.total};
    }
    mpsg::dots_host(&ctx->c, pairs, out);
  });
}

int mpsg_lincomb(mpsg_ctx* ctx, int32_t n, const double* c, const mpsg_tensor* const* x,
                 mpsg_tensor* out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(out, "out");
    if (n < 0) throw mpsg::Error(mpsg::kErrArgument, "negative count");
    std::vector<const double*> xs((size_t)n);
    std::vector<double> cs((size_t)n);
    if (n) {
      need(c, "c");
      need(x, "x");
    }
    for (int32_t i = 0; i < n; ++i) {
      need(x[i], "x[i]");
      mpsg::require_similar(x[i]->t, out->t, "lincomb: the tensors are not similar!");
      xs[i] = x[i]->t.data();
      cs[i] = c[i];
    }
    mpsg::launch_lincomb(&ctx->c, out->t.meta.total, xs, cs, out->t.data());
  });
}

int mpsg_dot(mpsg_ctx* ctx, const mpsg_tensor* a, const mpsg_tensor* b, double* out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(b, "b");
    need(out, "out");
    mpsg::require_similar(a->t, b->t, "The two SymTensors have to be similar to dot!");
    *out = mpsg::dot(&ctx->c, a->t, b->t);
  });
}

int mpsg_norm(mpsg_ctx* ctx, const mpsg_tensor* a, double* out) {
  return guarded([&] {
    need(ctx, "ctx");
    need(a, "a");
    need(out, "out");
    *out = std::sqrt(mpsg::dot(&ctx->c, a->t, a->t));
  });
}

}  // extern "C"
