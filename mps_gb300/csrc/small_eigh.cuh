// Small symmetric eigenproblems on the device (the projected matrices of the Lanczos solvers).
#pragma once

namespace mpsg {

// Symmetric eigen-decomposition of the leading K x K block of H (leading dimension ld, K <= 32)
// by cyclic Jacobi in one warp (lane k owns row / column k of each rotation), FP64, the same
// sweep order and stopping rule as small_eigh; ascending eigenvalues in D, eigenvectors in the
// columns of U (K x K, column-major).
__device__ __forceinline__ void warp_eigh(const double* __restrict__ H, int ld, int K,
                                          double* __restrict__ D, double* __restrict__ U) {
  __shared__ double a[32][33], v[32][33];
  __shared__ int order[32];
  const int k = threadIdx.x;
  for (int j = 0; j < K; ++j) {
    if (k < K) {
      a[k][j] = H[k + (int64_t)ld * j];
      v[k][j] = k == j ? 1.0 : 0.0;
    }
  }
  __syncwarp();
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, diag = 0.0;
    if (k < K)
      for (int j = 0; j < K; ++j) (k == j ? diag : off) += a[k][j] * a[k][j];
    for (int o = 16; o; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      diag += __shfl_xor_sync(0xffffffffu, diag, o);
    }
    if (off <= 1e-32 * fmax(diag, 1e-300)) break;
    for (int p = 0; p < K - 1; ++p)
      for (int q = p + 1; q < K; ++q) {
        const double apq = a[p][q];
        if (apq == 0.0) continue;
        const double theta = (a[q][q] - a[p][p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
        __syncwarp();
        if (k < K) {  // columns p, q
          const double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - sn * akq;
          a[k][q] = sn * akp + c * akq;
        }
        __syncwarp();
        if (k < K) {  // rows p, q
          const double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - sn * aqk;
          a[q][k] = sn * apk + c * aqk;
          const double vkp = v[k][p], vkq = v[k][q];
          v[k][p] = c * vkp - sn * vkq;
          v[k][q] = sn * vkp + c * vkq;
        }
        __syncwarp();
      }
  }
  if (k == 0) {  // stable selection order by ascending diagonal
    for (int i = 0; i < K; ++i) order[i] = i;
    for (int i = 1; i < K; ++i)
      for (int j = i; j > 0 && a[order[j]][order[j]] < a[order[j - 1]][order[j - 1]]; --j) {
        const int x = order[j];
        order[j] = order[j - 1];
        order[j - 1] = x;
      }
  }
  __syncwarp();
  if (k < K) {
    D[k] = a[order[k]][order[k]];
    for (int i = 0; i < K; ++i) U[k + (int64_t)K * i] = v[k][order[i]];
  }
}

}  // namespace mpsg
