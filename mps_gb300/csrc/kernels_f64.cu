// Plain FP64 path: grouped block GEMM (one persistent launch over every sector GEMM of a
// contraction) and the FP64 vector operations of the Krylov solver.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so the GEMM is a register-blocked
// DFMA kernel whose only job is to keep the FP64 pipe busy: 64x64 output tile per CTA, 4x4
// accumulators per thread, K staged through shared memory in steps of 16.
#include "runtime.hpp"

namespace mpsg {

namespace {

constexpr int BM = 64, BN = 64, BK = 16;

__global__ void __launch_bounds__(256) gemm_f64_grouped_kernel(
    const GemmTask* __restrict__ tasks, const int64_t* __restrict__ prefix, int ntasks,
    int64_t ntiles, const double* __restrict__ A, const double* __restrict__ B,
    double* __restrict__ C) {
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  __shared__ GemmTask g;
  __shared__ int64_t first;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    if (tid == 0) {
      int lo = 0, hi = ntasks - 1;
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= t) lo = mid;
        else hi = mid - 1;
      }
      g = tasks[lo];
      first = prefix[lo];
    }
    __syncthreads();
    const int64_t tm = (g.M + BM - 1) / BM;
    const int64_t lt = t - first;
    const int64_t m0 = (lt % tm) * BM, n0 = (lt / tm) * BN;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
    const double* Ab = A + g.offA;
    const double* Bb = B + g.offB;
    for (int64_t k0 = 0; k0 < g.K; k0 += BK) {
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        int m = tid & 63, k = (tid >> 6) + 4 * r;
        int64_t gm = m0 + m, gk = k0 + k;
        As[k][m] = (gm < g.M && gk < g.K) ? __ldg(Ab + gm + gk * g.lda) : 0.0;
        int kb = tid & 15, n = (tid >> 4) + 16 * r;
        int64_t gkb = k0 + kb, gn = n0 + n;
        Bs[kb][n] = (gkb < g.K && gn < g.N) ? __ldg(Bb + gkb + gn * g.ldb) : 0.0;
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < BK; ++k) {
        double a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[k][tx + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = Bs[k][ty + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
      __syncthreads();
    }
    double* Cb = C + g.offC;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int64_t gn = n0 + ty + 16 * j;
      if (gn >= g.N) continue;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        int64_t gm = m0 + tx + 16 * i;
        if (gm < g.M) Cb[gm + gn * g.ldc] = acc[i][j];
      }
    }
    __syncthreads();
  }
}

// Thin sector GEMMs (the MPO steps and W folds: K and one of M, N at most kThin) are memory-
// or DFMA-bound; padding them to 64 x 64 x 16 tiles wastes most of the FP64 pipe. One thread
// computes one output row (N thin) or one output column (M thin); the thin operand is the same
// for every thread of a task and reaches a warp as cache broadcasts.
constexpr int kThin = 32;

__device__ __forceinline__ int find_task(const int64_t* __restrict__ prefix, int n, int64_t u) {
  int lo = 0, hi = n - 1;  // largest t with prefix[t] <= u
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(prefix + mid) <= u) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Bodies with the contraction length as a template parameter: exactly K FMAs per output (an
// unrolled loop to kThin with a k < K guard would make the compiler issue all kThin of them, and
// FP64 issue rate is what bounds these kernels).
template <int K>
__device__ __forceinline__ void thin_row(const GemmTask& g, int64_t m, const double* __restrict__ A,
                                         const double* __restrict__ B, double* __restrict__ C) {
  double a[K > 0 ? K : 1];
#pragma unroll
  for (int k = 0; k < K; ++k) a[k] = __ldg(A + g.offA + m + k * g.lda);
  for (int64_t j = 0; j < g.N; ++j) {
    const double* b = B + g.offB + j * g.ldb;
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < K; ++k) acc = fma(a[k], __ldg(b + k), acc);
    C[g.offC + m + j * g.ldc] = acc;
  }
}

template <int K>
__device__ __forceinline__ void thin_col(const GemmTask& g, int64_t j, const double* __restrict__ A,
                                         const double* __restrict__ B, double* __restrict__ C) {
  double b[K > 0 ? K : 1];
#pragma unroll
  for (int k = 0; k < K; ++k) b[k] = __ldg(B + g.offB + k + j * g.ldb);
  for (int64_t m = 0; m < g.M; ++m) {
    const double* a = A + g.offA + m;
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < K; ++k) acc = fma(__ldg(a + k * g.lda), b[k], acc);
    C[g.offC + m + j * g.ldc] = acc;
  }
}

#define MPSG_THIN_CASES(F, g, i, A, B, C)                                                      \
  switch ((int)(g).K) {                                                                        \
    case 0: F<0>(g, i, A, B, C); break;   case 1: F<1>(g, i, A, B, C); break;                 \
    case 2: F<2>(g, i, A, B, C); break;   case 3: F<3>(g, i, A, B, C); break;                 \
    case 4: F<4>(g, i, A, B, C); break;   case 5: F<5>(g, i, A, B, C); break;                 \
    case 6: F<6>(g, i, A, B, C); break;   case 7: F<7>(g, i, A, B, C); break;                 \
    case 8: F<8>(g, i, A, B, C); break;   case 9: F<9>(g, i, A, B, C); break;                 \
    case 10: F<10>(g, i, A, B, C); break; case 11: F<11>(g, i, A, B, C); break;               \
    case 12: F<12>(g, i, A, B, C); break; case 13: F<13>(g, i, A, B, C); break;               \
    case 14: F<14>(g, i, A, B, C); break; case 15: F<15>(g, i, A, B, C); break;               \
    case 16: F<16>(g, i, A, B, C); break; case 17: F<17>(g, i, A, B, C); break;               \
    case 18: F<18>(g, i, A, B, C); break; case 19: F<19>(g, i, A, B, C); break;               \
    case 20: F<20>(g, i, A, B, C); break; case 21: F<21>(g, i, A, B, C); break;               \
    case 22: F<22>(g, i, A, B, C); break; case 23: F<23>(g, i, A, B, C); break;               \
    case 24: F<24>(g, i, A, B, C); break; case 25: F<25>(g, i, A, B, C); break;               \
    case 26: F<26>(g, i, A, B, C); break; case 27: F<27>(g, i, A, B, C); break;               \
    case 28: F<28>(g, i, A, B, C); break; case 29: F<29>(g, i, A, B, C); break;               \
    case 30: F<30>(g, i, A, B, C); break; case 31: F<31>(g, i, A, B, C); break;               \
    default: F<32>(g, i, A, B, C); break;                                                      \
  }

__global__ void __launch_bounds__(256) gemm_f64_rows_kernel(
    const GemmTask* __restrict__ tasks, const int64_t* __restrict__ prefix, int ntasks,
    int64_t nunits, const double* __restrict__ A, const double* __restrict__ B,
    double* __restrict__ C) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < nunits;
       u += (int64_t)gridDim.x * blockDim.x) {
    const int t = find_task(prefix, ntasks, u);
    const GemmTask g = tasks[t];
    const int64_t m = u - __ldg(prefix + t);
    MPSG_THIN_CASES(thin_row, g, m, A, B, C)
  }
}

__global__ void __launch_bounds__(256) gemm_f64_cols_kernel(
    const GemmTask* __restrict__ tasks, const int64_t* __restrict__ prefix, int ntasks,
    int64_t nunits, const double* __restrict__ A, const double* __restrict__ B,
    double* __restrict__ C) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < nunits;
       u += (int64_t)gridDim.x * blockDim.x) {
    const int t = find_task(prefix, ntasks, u);
    const GemmTask g = tasks[t];
    const int64_t j = u - __ldg(prefix + t);
    MPSG_THIN_CASES(thin_col, g, j, A, B, C)
  }
}

__global__ void fill_kernel(double* __restrict__ x, int64_t n, double v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = v;
}

__global__ void axpby_kernel(int64_t n, double a, const double* __restrict__ x, double b,
                             double* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = fma(a, x[i], b * y[i]);
}

__global__ void scale_kernel(int64_t n, double a, const double* __restrict__ x,
                             double* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i];
}

__device__ inline double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += sh[i];
  return r;
}

// Pass 1: fixed-grid partial sums; pass 2: one CTA sums the partials in a fixed order.
__global__ void __launch_bounds__(256) dot_partial_kernel(int64_t n, const double* __restrict__ x,
                                                          const double* __restrict__ y,
                                                          double* __restrict__ partial) {
  __shared__ double sh[8];
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    v = fma(x[i], y[i], v);
  double r = block_sum(v, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

__global__ void __launch_bounds__(256) sum_partials_kernel(int np, const double* __restrict__ p,
                                                           double* __restrict__ out) {
  __shared__ double sh[8];
  double v = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) v += p[i];
  double r = block_sum(v, sh);
  if (threadIdx.x == 0) *out = r;
}

// Batched dot products: blockIdx.y selects the pair; every pair gets the same fixed grid of
// partial sums and one CTA per pair adds them in a fixed order (deterministic).
__global__ void __launch_bounds__(256) dots_partial_kernel(const VecPair* __restrict__ pairs,
                                                           double* __restrict__ partial) {
  __shared__ double sh[8];
  const VecPair p = pairs[blockIdx.y];
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < p.n;
       i += (int64_t)gridDim.x * blockDim.x)
    v = fma(p.x[i], p.y[i], v);
  double r = block_sum(v, sh);
  if (threadIdx.x == 0) partial[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = r;
}

__global__ void __launch_bounds__(256) dots_sum_kernel(int np, const double* __restrict__ p,
                                                       double* __restrict__ out) {
  __shared__ double sh[8];
  double v = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) v += p[(int64_t)blockIdx.x * np + i];
  double r = block_sum(v, sh);
  if (threadIdx.x == 0) out[blockIdx.x] = r;
}

// y[e] = sum_i c[i] x_i[e]; one thread reads every operand of its element before writing it, so
// y may be one of the operands
__global__ void __launch_bounds__(256) lincomb_kernel(int64_t n, int m,
                                                      const double* const* __restrict__ xs,
                                                      const double* __restrict__ c,
                                                      double* __restrict__ y) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int i = 0; i < m; ++i) s = fma(c[i], xs[i][e], s);
    y[e] = s;
  }
}

int vec_grid(Context* ctx, int64_t n) {
  int64_t g = (n + 255) / 256;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)ctx->num_sms * 4));
}

}  // namespace

void DevGemmPlan::build_host(const std::vector<GemmTask>& g, double flops_, GemmTables& t) {
  host = g;
  flops = flops_;
  t = GemmTables();
  for (const GemmTask& x : g) {
    if (x.K <= kThin && x.N <= kThin && x.M >= x.N) t.part[kRows].push_back(x);
    else if (x.K <= kThin && x.M <= kThin) t.part[kCols].push_back(x);
    else t.part[kTiled].push_back(x);
  }
  for (int q = 0; q < 3; ++q) {
    const auto& v = t.part[q];
    auto& pre = t.prefix[q];
    pre.assign(v.size() + 1, 0);
    for (size_t k = 0; k < v.size(); ++k) {
      int64_t units = q == kTiled ? ((v[k].M + BM - 1) / BM) * ((v[k].N + BN - 1) / BN)
                      : q == kRows ? v[k].M : v[k].N;
      pre[k + 1] = pre[k] + units;
    }
    count[q] = (int)v.size();
    units[q] = pre.back();
  }
  n = count[kTiled];
  ntiles = units[kTiled];
}

void DevGemmPlan::upload(const std::vector<GemmTask>& g, double flops_, cudaStream_t st) {
  release();
  stream = st;
  GemmTables t;
  build_host(g, flops_, t);
  for (int q = 0; q < 3; ++q) {
    if (count[q] == 0) continue;
    const size_t bt = sizeof(GemmTask) * count[q], bp = sizeof(int64_t) * (count[q] + 1);
    MPSG_CUDA(cudaMallocAsync((void**)&d_part[q], bt, st));
    MPSG_CUDA(cudaMallocAsync((void**)&d_part_prefix[q], bp, st));
    MPSG_CUDA(cudaMemcpyAsync(d_part[q], t.part[q].data(), bt, cudaMemcpyHostToDevice, st));
    MPSG_CUDA(cudaMemcpyAsync(d_part_prefix[q], t.prefix[q].data(), bp, cudaMemcpyHostToDevice,
                              st));
  }
  d_tasks = d_part[kTiled];
  d_prefix = d_part_prefix[kTiled];
}

void DevGemmPlan::release() {
  for (int q = 0; q < 3; ++q) {
    if (d_part[q]) cudaFreeAsync(d_part[q], stream);
    if (d_part_prefix[q]) cudaFreeAsync(d_part_prefix[q], stream);
    d_part[q] = nullptr;
    d_part_prefix[q] = nullptr;
    count[q] = 0;
    units[q] = 0;
  }
  d_tasks = nullptr;
  d_prefix = nullptr;
  n = 0;
  ntiles = 0;
}

void launch_gemm_f64(Context* ctx, const DevGemmPlan& p, const double* A, const double* B,
                     double* C) {
  if (p.units[kTiled] + p.units[kRows] + p.units[kCols] == 0) return;
  KernelTimer timer(ctx, kKindGemmF64, p.flops);
  if (p.units[kTiled]) {
    int64_t grid = std::min<int64_t>(p.units[kTiled], (int64_t)ctx->num_sms * 4);
    gemm_f64_grouped_kernel<<<(unsigned)grid, 256, 0, ctx->stream>>>(
        p.d_part[kTiled], p.d_part_prefix[kTiled], p.count[kTiled], p.units[kTiled], A, B, C);
    MPSG_CUDA(cudaGetLastError());
    ctx->kernel_launches++;
  }
  for (int q : {kRows, kCols}) {
    if (!p.units[q]) continue;
    int64_t grid = std::min<int64_t>((p.units[q] + 255) / 256, (int64_t)ctx->num_sms * 8);
    auto kern = q == kRows ? gemm_f64_rows_kernel : gemm_f64_cols_kernel;
    kern<<<(unsigned)grid, 256, 0, ctx->stream>>>(p.d_part[q], p.d_part_prefix[q], p.count[q],
                                                  p.units[q], A, B, C);
    MPSG_CUDA(cudaGetLastError());
    ctx->kernel_launches++;
  }
  ctx->gemm_flops += p.flops;
}

void launch_fill(Context* ctx, double* x, int64_t n, double v) {
  if (n == 0) return;
  fill_kernel<<<vec_grid(ctx, n), 256, 0, ctx->stream>>>(x, n, v);
  MPSG_CUDA(cudaGetLastError());
  ctx->kernel_launches++;
}

void launch_axpby(Context* ctx, int64_t n, double a, const double* x, double b, double* y) {
  if (n == 0) return;
  axpby_kernel<<<vec_grid(ctx, n), 256, 0, ctx->stream>>>(n, a, x, b, y);
  MPSG_CUDA(cudaGetLastError());
  ctx->kernel_launches++;
}

void launch_scale(Context* ctx, int64_t n, double a, const double* x, double* y) {
  if (n == 0) return;
  scale_kernel<<<vec_grid(ctx, n), 256, 0, ctx->stream>>>(n, a, x, y);
  MPSG_CUDA(cudaGetLastError());
  ctx->kernel_launches++;
}

int dots_grid(Context* ctx, int64_t nmax) { return std::min(vec_grid(ctx, nmax), 64); }

void dots_host(Context* ctx, const std::vector<VecPair>& pairs, double* out) {
  const int np = (int)pairs.size();
  if (np == 0) return;
  int64_t nmax = 1;
  for (const VecPair& p : pairs) nmax = std::max(nmax, p.n);
  const int g = dots_grid(ctx, nmax);
  cudaStream_t st = ctx->stream;
  VecPair* d_pairs = nullptr;
  double* d_part = nullptr;
  MPSG_CUDA(cudaMallocAsync((void**)&d_pairs, sizeof(VecPair) * np, st));
  MPSG_CUDA(cudaMallocAsync((void**)&d_part, sizeof(double) * ((int64_t)np * g + np), st));
  MPSG_CUDA(cudaMemcpyAsync(d_pairs, pairs.data(), sizeof(VecPair) * np, cudaMemcpyHostToDevice,
                            st));
  double* d_out = d_part + (int64_t)np * g;
  dots_partial_kernel<<<dim3((unsigned)g, (unsigned)np), 256, 0, st>>>(d_pairs, d_part);
  dots_sum_kernel<<<(unsigned)np, 256, 0, st>>>(g, d_part, d_out);
  MPSG_CUDA(cudaGetLastError());
  ctx->kernel_launches += 2;
  MPSG_CUDA(cudaMemcpyAsync(out, d_out, sizeof(double) * np, cudaMemcpyDeviceToHost, st));
  MPSG_CUDA(cudaFreeAsync(d_pairs, st));
  MPSG_CUDA(cudaFreeAsync(d_part, st));
  MPSG_CUDA(cudaStreamSynchronize(st));
}

void launch_lincomb(Context* ctx, int64_t n, const std::vector<const double*>& xs,
                    const std::vector<double>& c, double* y) {
  const int m = (int)xs.size();
  if (n == 0) return;
  cudaStream_t st = ctx->stream;
  const double** d_xs = nullptr;
  double* d_c = nullptr;
  MPSG_CUDA(cudaMallocAsync((void**)&d_xs, sizeof(double*) * std::max(m, 1), st));
  MPSG_CUDA(cudaMallocAsync((void**)&d_c, sizeof(double) * std::max(m, 1), st));
  if (m) {
    MPSG_CUDA(cudaMemcpyAsync(d_xs, xs.data(), sizeof(double*) * m, cudaMemcpyHostToDevice, st));
    MPSG_CUDA(cudaMemcpyAsync(d_c, c.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st));
  }
  lincomb_kernel<<<vec_grid(ctx, n), 256, 0, st>>>(n, m, d_xs, d_c, y);
  MPSG_CUDA(cudaGetLastError());
  ctx->kernel_launches++;
  MPSG_CUDA(cudaFreeAsync(d_xs, st));
  MPSG_CUDA(cudaFreeAsync(d_c, st));
}

void launch_dots_device(Context* ctx, const VecPair* d_pairs, int np, int64_t nmax,
                        double* d_part, double* d_out) {
  if (np == 0) return;
  const int g = dots_grid(ctx, nmax);
  dots_partial_kernel<<<dim3((unsigned)g, (unsigned)np), 256, 0, ctx->stream>>>(d_pairs, d_part);
  dots_sum_kernel<<<(unsigned)np, 256, 0, ctx->stream>>>(g, d_part, d_out);
  MPSG_CUDA(cudaGetLastError());
  ctx->kernel_launches += 2;
}

void launch_lincomb_device(Context* ctx, int64_t n, int m, const double* const* d_xs,
                           const double* d_c, double* y) {
  if (n == 0) return;
  lincomb_kernel<<<vec_grid(ctx, n), 256, 0, ctx->stream>>>(n, m, d_xs, d_c, y);
  MPSG_CUDA(cudaGetLastError());
  ctx->kernel_launches++;
}

void launch_dot(Context* ctx, int64_t n, const double* x, const double* y, double* d_out) {
  if (n == 0) {
    launch_fill(ctx, d_out, 1, 0.0);
    return;
  }
  int g = vec_grid(ctx, n);
  dot_partial_kernel<<<g, 256, 0, ctx->stream>>>(n, x, y, ctx->d_partials);
  sum_partials_kernel<<<1, 256, 0, ctx->stream>>>(g, ctx->d_partials, d_out);
  MPSG_CUDA(cudaGetLastError());
  ctx->kernel_launches += 2;
}

}  // namespace mpsg
