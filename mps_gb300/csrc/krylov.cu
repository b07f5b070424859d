// Thick-restart Lanczos on device-resident tensors (the KrylovKit.eigsolve call of
// src/dmrg.jl:77-82).  Krylov vectors, reorthogonalisation dot products and vector updates are
// FP64 kernels on the context stream; the host keeps only the small projected matrix.
#include <algorithm>
#include <cmath>

#include "linalg.hpp"

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

DeviceTensor scaled(Context* ctx, const DeviceTensor& a, double alpha) {
  DeviceTensor t = new_tensor(ctx, a.meta, false);
  launch_scale(ctx, a.meta.total, alpha, a.data(), t.data());
  return t;
}

DeviceTensor lincomb(Context* ctx, const std::vector<DeviceTensor>& V, const double* c) {
  DeviceTensor t = scaled(ctx, V[0], c[0]);
  for (size_t j = 1; j < V.size(); ++j)
    launch_axpby(ctx, t.meta.total, c[j], V[j].data(), 1.0, t.data());
  return t;
}

// classical Gram-Schmidt applied twice; returns the summed coefficients
std::vector<double> orthogonalize(Context* ctx, DeviceTensor& w, const std::vector<DeviceTensor>& V) {
  std::vector<double> h(V.size(), 0.0);
  for (int pass = 0; pass < 2; ++pass) {
    std::vector<double> c(V.size());
    for (size_t j = 0; j < V.size(); ++j) c[j] = dot(ctx, V[j], w);
    for (size_t j = 0; j < V.size(); ++j) {
      launch_axpby(ctx, w.meta.total, -c[j], V[j].data(), 1.0, w.data());
      h[j] += c[j];
    }
  }
  return h;
}

}  // namespace

EigResult eigsolve_heff2(Context* ctx, const DeviceTensor& x0, const DeviceTensor& envL,
                         const DeviceTensor& envR, const DeviceTensor& W1, const DeviceTensor& W2,
                         int krylovdim, int maxiter, double tol, int precision) {
  if (krylovdim < 2) throw Error(kErrArgument, "krylovdim must be at least 2");
  if (maxiter < 1) throw Error(kErrArgument, "maxiter must be at least 1");
  auto op = heff_create(ctx, x0.meta, envL, envR, W1, W2, precision);
  auto f = [&](const DeviceTensor& x) { return heff_apply(*op, x); };
  const int kd = krylovdim;
  std::vector<double> H((kd + 1) * (kd + 1), 0.0);
  auto Hat = [&](int i, int j) -> double& { return H[i + (kd + 1) * j]; };
  EigResult R;
  double beta0 = std::sqrt(dot(ctx, x0, x0));
  if (!(beta0 > 0)) throw Error(kErrArgument, "eigsolve: zero start vector");
  std::vector<DeviceTensor> V;
  V.push_back(scaled(ctx, x0, 1.0 / beta0));
  DeviceTensor w = f(V[0]);
  int numops = 1, numiter = 1;
  std::vector<double> h = orthogonalize(ctx, w, V);
  Hat(0, 0) = h[0];
  double beta = std::sqrt(dot(ctx, w, w));
  bool arrow = false;
  std::vector<double> D(kd), U(kd * kd), Hk(kd * kd);
  for (;;) {
    int K = (int)V.size();
    if (K == kd || beta <= tol) {
      for (int j = 0; j < K; ++j)
        for (int i = 0; i < K; ++i) Hk[i + K * j] = Hat(i, j);
      small_eigh(K, Hk.data(), D.data(), U.data());
      double normres = std::fabs(beta * U[(K - 1) + K * 0]);
      bool converged = normres <= tol;
      if (converged || beta <= tol || numiter >= maxiter) {
        DeviceTensor x = lincomb(ctx, V, &U[0]);
        double nx = std::sqrt(dot(ctx, x, x));
        launch_scale(ctx, x.meta.total, 1.0 / nx, x.data(), x.data());
        R.value = D[0];
        R.vec = x;
        R.normres = normres;
        R.numiter = numiter;
        R.numops = numops;
        R.converged = converged;
        return R;
      }
      int keep = std::max(1, (3 * kd + 2 * (converged ? 1 : 0)) / 5);
      std::vector<DeviceTensor> Vn;
      for (int i = 0; i < keep; ++i) Vn.push_back(lincomb(ctx, V, &U[K * i]));
      std::fill(H.begin(), H.end(), 0.0);
      for (int i = 0; i < keep; ++i) {
        Hat(i, i) = D[i];
        Hat(keep, i) = Hat(i, keep) = beta * U[(K - 1) + K * i];
      }
      V = std::move(Vn);
      ++numiter;
      arrow = true;
      K = keep;
    }
    DeviceTensor v = scaled(ctx, w, 1.0 / beta);
    if (arrow) arrow = false;
    else Hat(K, K - 1) = Hat(K - 1, K) = beta;
    V.push_back(v);
    w = f(v);
    ++numops;
    h = orthogonalize(ctx, w, V);
    Hat(K, K) = h[K];
    beta = std::sqrt(dot(ctx, w, w));
  }
}

}  // namespace mpsg
