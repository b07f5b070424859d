// Thick-restart Lanczos on device-resident tensors (the KrylovKit.eigsolve call of
// src/dmrg.jl:77-82).  Krylov vectors, reorthogonalisation dot products and vector updates are
// FP64 kernels on the context stream; the host keeps only the small projected matrix.
#include <algorithm>
#include <cmath>

#include "linalg.hpp"
#include "small_eigh.cuh"

namespace mpsg {

void small_eigh(int n, const double* A, double* evals, double* evecs) {
  std::vector<double> a(A, A + n * n), v(n * n, 0.0);
  for (int i = 0; i < n; ++i) v[i * n + i] = 1.0;
  auto at = [&](int i, int j) -> double& { return a[i + n * j]; };
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) (i == j ? diag : off) += at(i, j) * at(i, j);
    if (off <= 1e-32 * std::max(diag, 1e-300)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = at(p, q);
        if (apq == 0.0) continue;
        double theta = (at(q, q) - at(p, p)) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // rotate columns p, q
          double akp = at(k, p), akq = at(k, q);
          at(k, p) = c * akp - s * akq;
          at(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // rotate rows p, q
          double apk = at(p, k), aqk = at(q, k);
          at(p, k) = c * apk - s * aqk;
          at(q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double vkp = v[k + n * p], vkq = v[k + n * q];
          v[k + n * p] = c * vkp - s * vkq;
          v[k + n * q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int x, int y) { return at(x, x) < at(y, y); });
  for (int i = 0; i < n; ++i) {
    evals[i] = at(order[i], order[i]);
    for (int k = 0; k < n; ++k) evecs[k + n * i] = v[k + n * order[i]];
  }
}

namespace {

__global__ void small_eigh_kernel(const double* __restrict__ H, int ld, int K,
                                  double* __restrict__ D, double* __restrict__ U) {
  warp_eigh(H, ld, K, D, U);
}

// One pass of the orthogonalisation, after its dot products dots[j] = <V_j, w> (j < K): the
// coefficients of w <- w - sum_j dots[j] V_j ([1, -dots...]) and H(K-1, K-1) += dots[K-1], the
// projection on the newest basis vector.
__global__ void orth_coef_kernel(const double* __restrict__ dots, int K, double* __restrict__ coef,
                                 double* __restrict__ hkk) {
  const int j = threadIdx.x;
  if (j == 0) coef[0] = 1.0;
  if (j < K) coef[1 + j] = -dots[j];
  if (j == K - 1) *hkk += dots[j];
}

__global__ void set_sym_kernel(double* __restrict__ H, int ld, int i, int j, double x) {
  H[i + (int64_t)ld * j] = x;
  H[j + (int64_t)ld * i] = x;
}

// Restart: H <- 0, H(i, i) = D(i), H(keep, i) = H(i, keep) = beta U(K-1, i) for i < keep.
__global__ void restart_h_kernel(double* __restrict__ H, int ld, int keep, int K,
                                 const double* __restrict__ D, const double* __restrict__ U,
                                 double beta) {
  for (int e = threadIdx.x; e < ld * ld; e += blockDim.x) H[e] = 0.0;
  __syncthreads();
  const int i = threadIdx.x;
  if (i < keep) {
    H[i + (int64_t)ld * i] = D[i];
    const double b = beta * U[(K - 1) + (int64_t)K * i];
    H[keep + (int64_t)ld * i] = b;
    H[i + (int64_t)ld * keep] = b;
  }
}

// Device scratch of one Lanczos solve: the projected matrix, its eigen-decomposition, dot and
// linear-combination tables.  Everything the recurrence needs stays on the device; the host
// reads one norm per Krylov step and two numbers per restart.
struct LanczosWork {
  Context* ctx;
  int kd, ld;
  std::shared_ptr<Buffer> buf;  // H, D, U, dots, coef, partial sums (doubles)
  double *H, *D, *U, *dots, *coef, *part;
  VecPair* pairs = nullptr;
  const double** xs = nullptr;
  int64_t n;
  LanczosWork(Context* c, int kd_, int64_t n_) : ctx(c), kd(kd_), ld(kd_ + 1), n(n_) {
    const int g = dots_grid(ctx, std::max<int64_t>(n, 1));
    const int64_t nh = (int64_t)ld * ld, nd = kd, nu = (int64_t)kd * kd;
    const int64_t total = nh + nd + nu + (kd + 1) + (kd + 2) + (int64_t)(kd + 1) * g;
    buf = alloc_buffer(ctx, total);
    H = buf->ptr;
    D = H + nh;
    U = D + nd;
    dots = U + nu;
    coef = dots + (kd + 1);
    part = coef + (kd + 2);
    MPSG_CUDA(cudaMallocAsync((void**)&pairs, sizeof(VecPair) * (kd + 1), ctx->stream));
    MPSG_CUDA(cudaMallocAsync((void**)&xs, sizeof(double*) * (kd + 2), ctx->stream));
    MPSG_CUDA(cudaMemsetAsync(H, 0, sizeof(double) * nh, ctx->stream));
  }
  ~LanczosWork() {
    cudaFreeAsync(pairs, ctx->stream);
    cudaFreeAsync(xs, ctx->stream);
  }
  // y <- sum_i c[i] x_i with the coefficients already on the device (c)
  void lincomb(const std::vector<const double*>& x, const double* c, double* y) {
    MPSG_CUDA(cudaMemcpyAsync(xs, x.data(), sizeof(double*) * x.size(), cudaMemcpyHostToDevice,
                              ctx->stream));
    launch_lincomb_device(ctx, n, (int)x.size(), xs, c, y);
  }
  // classical Gram-Schmidt against V applied twice, on the device; H(K-1, K-1) gets the summed
  // projection on the newest vector
  void orthogonalize(DeviceTensor& w, const std::vector<DeviceTensor>& V) {
    const int K = (int)V.size();
    std::vector<VecPair> pr(K);
    std::vector<const double*> x(K + 1);
    x[0] = w.data();
    for (int j = 0; j < K; ++j) {
      pr[j] = VecPair{V[j].data(), w.data(), n};
      x[1 + j] = V[j].data();
    }
    MPSG_CUDA(cudaMemcpyAsync(pairs, pr.data(), sizeof(VecPair) * K, cudaMemcpyHostToDevice,
                              ctx->stream));
    for (int pass = 0; pass < 2; ++pass) {
      launch_dots_device(ctx, pairs, K, n, part, dots);
      orth_coef_kernel<<<1, 32, 0, ctx->stream>>>(dots, K, coef, H + (K - 1) + (int64_t)ld * (K - 1));
      ctx->kernel_launches++;
      lincomb(x, coef, w.data());
    }
  }
  // K x K eigen-decomposition of the projected matrix; returns (lowest value, U(K-1, 0))
  std::pair<double, double> eig(int K) {
    small_eigh_kernel<<<1, 32, 0, ctx->stream>>>(H, ld, K, D, U);
    MPSG_CUDA(cudaGetLastError());
    ctx->kernel_launches++;
    MPSG_CUDA(cudaMemcpyAsync(ctx->h_pinned, D, sizeof(double), cudaMemcpyDeviceToHost,
                              ctx->stream));
    MPSG_CUDA(cudaMemcpyAsync(ctx->h_pinned + 1, U + (K - 1), sizeof(double),
                              cudaMemcpyDeviceToHost, ctx->stream));
    MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
    return {ctx->h_pinned[0], ctx->h_pinned[1]};
  }
};

DeviceTensor scaled(Context* ctx, const DeviceTensor& a, double alpha) {
  DeviceTensor t = new_tensor(ctx, a.meta, false);
  launch_scale(ctx, a.meta.total, alpha, a.data(), t.data());
  return t;
}

}  // namespace

EigResult eigsolve_heff2(Context* ctx, const DeviceTensor& x0, const DeviceTensor& envL,
                         const DeviceTensor& envR, const DeviceTensor& W1, const DeviceTensor& W2,
                         int krylovdim, int maxiter, double tol, int precision) {
  if (krylovdim < 2) throw Error(kErrArgument, "krylovdim must be at least 2");
  if (krylovdim > 32) throw Error(kErrArgument, "krylovdim must be at most 32");
  if (maxiter < 1) throw Error(kErrArgument, "maxiter must be at least 1");
  auto op = heff_create(ctx, x0.meta, envL, envR, W1, W2, precision);
  auto f = [&](const DeviceTensor& x) { return heff_apply(*op, x); };
  const int kd = krylovdim;
  LanczosWork Wk(ctx, kd, x0.meta.total);
  EigResult R;
  double beta0 = std::sqrt(dot(ctx, x0, x0));
  if (!(beta0 > 0)) throw Error(kErrArgument, "eigsolve: zero start vector");
  std::vector<DeviceTensor> V;
  V.push_back(scaled(ctx, x0, 1.0 / beta0));
  DeviceTensor w = f(V[0]);
  int numops = 1, numiter = 1;
  Wk.orthogonalize(w, V);
  double beta = std::sqrt(dot(ctx, w, w));
  bool arrow = false;
  for (;;) {
    int K = (int)V.size();
    if (K == kd || beta <= tol) {
      const auto ev = Wk.eig(K);  // on the device; the host reads two numbers
      const double normres = std::fabs(beta * ev.second);
      const bool converged = normres <= tol;
      if (converged || beta <= tol || numiter >= maxiter) {
        std::vector<const double*> xv(K);
        for (int j = 0; j < K; ++j) xv[j] = V[j].data();
        DeviceTensor x = new_tensor(ctx, V[0].meta, false);
        Wk.lincomb(xv, Wk.U, x.data());  // sum_j U(j, 0) V_j
        double nx = std::sqrt(dot(ctx, x, x));
        launch_scale(ctx, x.meta.total, 1.0 / nx, x.data(), x.data());
        R.value = ev.first;
        R.vec = x;
        R.normres = normres;
        R.numiter = numiter;
        R.numops = numops;
        R.converged = converged;
        return R;
      }
      int keep = std::max(1, (3 * kd + 2 * (converged ? 1 : 0)) / 5);
      std::vector<const double*> xv(K);
      for (int j = 0; j < K; ++j) xv[j] = V[j].data();
      std::vector<DeviceTensor> Vn;
      for (int i = 0; i < keep; ++i) {
        Vn.push_back(new_tensor(ctx, V[0].meta, false));
        Wk.lincomb(xv, Wk.U + (int64_t)K * i, Vn.back().data());
      }
      restart_h_kernel<<<1, 64, 0, ctx->stream>>>(Wk.H, Wk.ld, keep, K, Wk.D, Wk.U, beta);
      MPSG_CUDA(cudaGetLastError());
      ctx->kernel_launches++;
      V = std::move(Vn);
      ++numiter;
      arrow = true;
      K = keep;
    }
    DeviceTensor v = scaled(ctx, w, 1.0 / beta);
    if (arrow) {
      arrow = false;
    } else {
      set_sym_kernel<<<1, 1, 0, ctx->stream>>>(Wk.H, Wk.ld, K, K - 1, beta);
      ctx->kernel_launches++;
    }
    V.push_back(v);
    w = f(v);
    ++numops;
    Wk.orthogonalize(w, V);
    beta = std::sqrt(dot(ctx, w, w));
  }
}

}  // namespace mpsg
