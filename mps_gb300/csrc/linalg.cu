// Per-sector SVD with greedy truncation (src/symtools.jl:1-35, src/mpsutils.jl:89-179) and the
// thick-restart Lanczos eigensolver that drives the two-site effective Hamiltonian (the role of
// KrylovKit.eigsolve at src/dmrg.jl:77-82).  Everything stays FP64 on the GPU; the host only
// sees singular values (for the truncation choice) and the small projected matrix.
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <exception>
#include <functional>
#include <thread>

#include "linalg.hpp"

namespace mpsg {

#define MPSG_SOLVER(call)                                                                   \
  do {                                                                                      \
    cusolverStatus_t s_ = (call);                                                           \
    if (s_ != CUSOLVER_STATUS_SUCCESS)                                                      \
      throw ::mpsg::Error(::mpsg::kErrCuda, std::string(#call) + " failed: " + std::to_string((int)s_)); \
  } while (0)

#define MPSG_BLAS(call)                                                                     \
  do {                                                                                      \
    cublasStatus_t s_ = (call);                                                             \
    if (s_ != CUBLAS_STATUS_SUCCESS)                                                        \
      throw ::mpsg::Error(::mpsg::kErrCuda, std::string(#call) + " failed: " + std::to_string((int)s_)); \
  } while (0)

namespace {

constexpr int kLanes = 8;  // solver lanes created per context; MPSG_SOLVER_LANES of them used

// Lanes a call spreads its blocks over: MPSG_SOLVER_LANES (1..8), default 4.
int active_lanes() {
  const char* e = std::getenv("MPSG_SOLVER_LANES");
  const int n = e ? std::atoi(e) : 4;
  return std::max(1, std::min(kLanes, n));
}

// Side streams with their own cuSOLVER and cuBLAS handles. The per-sector factorisations of one
// call are independent, so they run concurrently on these lanes, forked from the context stream
// by an event and joined back into it before anything downstream (or the host) reads them.
struct SolverLanes {
  cudaStream_t st[kLanes] = {};
  cusolverDnHandle_t sol[kLanes] = {};
  cublasHandle_t blas[kLanes] = {};
  cudaEvent_t fork = nullptr;
  cudaEvent_t join[kLanes] = {};
  ~SolverLanes() {
    for (int i = 0; i < kLanes; ++i) {
      if (st[i]) cudaStreamSynchronize(st[i]);
      if (sol[i]) cusolverDnDestroy(sol[i]);
      if (blas[i]) cublasDestroy(blas[i]);
      if (join[i]) cudaEventDestroy(join[i]);
      if (st[i]) cudaStreamDestroy(st[i]);
    }
    if (fork) cudaEventDestroy(fork);
  }
};

SolverLanes& lanes(Context* ctx) {
  if (!ctx->solver) {
    auto* L = new SolverLanes();
    ctx->solver = L;
    ctx->solver_destroy = [](void* p) { delete (SolverLanes*)p; };
    MPSG_CUDA(cudaEventCreateWithFlags(&L->fork, cudaEventDisableTiming));
    for (int i = 0; i < kLanes; ++i) {
      MPSG_CUDA(cudaStreamCreateWithFlags(&L->st[i], cudaStreamNonBlocking));
      MPSG_CUDA(cudaEventCreateWithFlags(&L->join[i], cudaEventDisableTiming));
      MPSG_SOLVER(cusolverDnCreate(&L->sol[i]));
      MPSG_SOLVER(cusolverDnSetStream(L->sol[i], L->st[i]));
      MPSG_BLAS(cublasCreate(&L->blas[i]));
      MPSG_BLAS(cublasSetStream(L->blas[i], L->st[i]));
    }
  }
  return *(SolverLanes*)ctx->solver;
}

// dst[i + ld*i] = s[i] on a zeroed k x k block
__global__ void set_diag_kernel(double* __restrict__ dst, const double* __restrict__ s, int64_t k) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < k;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i + k * i] = s[i];
}

// dst (r x n, column-major) = first r columns of src (n x k, column-major) transposed
__global__ void transpose_prefix_kernel(double* __restrict__ dst, const double* __restrict__ src,
                                        int64_t r, int64_t n) {
  __shared__ double t[32][33];
  const int64_t i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  for (int y = threadIdx.y; y < 32; y += 8) {
    int64_t i = i0 + y, j = j0 + threadIdx.x;  // read src(j, i): column i of src
    if (i < r && j < n) t[y][threadIdx.x] = src[j + n * i];
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += 8) {
    int64_t j = j0 + y, i = i0 + threadIdx.x;  // write dst(i, j)
    if (i < r && j < n) dst[i + r * j] = t[threadIdx.x][y];
  }
}

// The k largest eigenpairs of an n x n Gram matrix in descending order: X[:, i] = Q[:, n-1-i] and
// S[i] = sqrt(max(w[n-1-i], 0)), where (w, Q) is the ascending eigen-decomposition.
__global__ void top_eigpairs_kernel(double* __restrict__ X, double* __restrict__ S,
                                    const double* __restrict__ Q, const double* __restrict__ w,
                                    int64_t n, int64_t k) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * k;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / n, r = t - i * n;
    X[t] = Q[r + n * (n - 1 - i)];
    if (r == 0) S[i] = sqrt(fmax(w[n - 1 - i], 0.0));
  }
}

// S[i] = |Y[:, i]| (one warp per column, FP64), then S[i] = min(S[i], S[i-1]) over i (one
// thread, after the norms): the singular values of A as the column norms of A^T U (or A V) for
// the Gram eigenvectors U (V). Their absolute error is about eps * max(S), where sqrt of the
// Gram eigenvalue is off by about eps * max(S)^2 / S for small values. The running minimum keeps
// the order where round-off ties neighbouring values.
__global__ void col_norms_kernel(const double* __restrict__ Y, double* __restrict__ S,
                                 int64_t rows, int64_t k) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = warp; c < k; c += nwarps) {
    const double* y = Y + c * rows;
    double acc = 0.0;
    for (int64_t r = lane; r < rows; r += 32) acc = fma(y[r], y[r], acc);
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) S[c] = sqrt(acc);
  }
}

__global__ void running_min_kernel(double* __restrict__ S, int64_t k) {
  if (blockIdx.x == 0 && threadIdx.x == 0)
    for (int64_t i = 1; i < k; ++i) S[i] = fmin(S[i], S[i - 1]);
}

// X[:, i] /= S[i] (columns with S[i] == 0 become zero)
__global__ void scale_cols_inv_kernel(double* __restrict__ X, const double* __restrict__ S,
                                      int64_t rows, int64_t k) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < rows * k;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double s = S[t / rows];
    X[t] = s > 0.0 ? X[t] / s : 0.0;
  }
}

unsigned grid_for(int64_t n) { return (unsigned)std::min<int64_t>((n + 255) / 256, 1184); }

// Runs work(lane, b) for every block, largest cost first, each block on the least loaded of the
// solver lanes; the lanes are forked from and joined back into the context stream. Each lane's
// list is issued by its own host thread: cuSOLVER's eigen- and SVD solvers block the calling
// thread on large blocks, which would otherwise serialise the lanes.
void run_on_lanes(Context* ctx, SolverLanes& L, size_t nb, const std::function<double(size_t)>& cost,
                  const std::function<void(int, size_t)>& work) {
  std::vector<size_t> order(nb);
  for (size_t b = 0; b < nb; ++b) order[b] = b;
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t x, size_t y) { return cost(x) > cost(y); });
  std::vector<size_t> list[kLanes];
  double load[kLanes] = {0, 0, 0, 0, 0, 0, 0, 0};
  const int nl = active_lanes();
  for (size_t b : order) {
    int lane = 0;
    for (int i = 1; i < nl; ++i)
      if (load[i] < load[lane]) lane = i;
    load[lane] += cost(b);
    list[lane].push_back(b);
  }
  MPSG_CUDA(cudaEventRecord(L.fork, ctx->stream));
  for (int i = 0; i < kLanes; ++i)
    if (!list[i].empty()) MPSG_CUDA(cudaStreamWaitEvent(L.st[i], L.fork, 0));
  std::exception_ptr failure[kLanes];
  auto run_lane = [&](int i) {
    try {
      MPSG_CUDA(cudaSetDevice(ctx->device));  // the current device is per host thread
      for (size_t b : list[i]) work(i, b);
    } catch (...) {
      failure[i] = std::current_exception();
    }
  };
  std::vector<std::thread> threads;
  for (int i = 1; i < kLanes; ++i)
    if (!list[i].empty()) threads.emplace_back(run_lane, i);
  run_lane(0);
  for (auto& t : threads) t.join();
  for (int i = 0; i < kLanes; ++i) {
    if (list[i].empty()) continue;
    MPSG_CUDA(cudaEventRecord(L.join[i], L.st[i]));
    MPSG_CUDA(cudaStreamWaitEvent(ctx->stream, L.join[i], 0));
  }
  for (int i = 0; i < kLanes; ++i)
    if (failure[i]) std::rethrow_exception(failure[i]);
}

// Complex block assembled from its real and imaginary planes (rows x cols, column-major):
// dst = A, or A^T when trans, with the imaginary part multiplied by imsign (-1: conjugate).
__global__ void interleave_kernel(double2* __restrict__ dst, const double* __restrict__ re,
                                  const double* __restrict__ im, double imsign, int64_t rows,
                                  int64_t cols, int trans) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < rows * cols;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = t / rows, i = t - j * rows;
    const int64_t d = trans ? j + cols * i : t;
    dst[d] = make_double2(re[t], imsign * im[t]);
  }
}

// dst (rows x cols, column-major, split into planes) = op(src)(i, j): src[i + ld j], or
// src[j + ld i] when trans; conjugated when conj.
__global__ void cplx_extract_kernel(double* __restrict__ dre, double* __restrict__ dim,
                                    const double2* __restrict__ src, int64_t rows, int64_t cols,
                                    int64_t ld, int trans, int conj) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < rows * cols;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = t / rows, i = t - j * rows;
    const double2 s = trans ? src[j + ld * i] : src[i + ld * j];
    dre[t] = s.x;
    dim[t] = conj ? -s.y : s.y;
  }
}

struct BlockSVD {
  int c1, c2;
  int64_t M, N, k;
  std::shared_ptr<Buffer> U, S, V;  // U: M x k, S: k, V: N x k (all column-major)
  std::shared_ptr<Buffer> work, aux, wbuf;  // temporaries, kept until the lanes are joined
  std::shared_ptr<Buffer> ref;              // second-level Gram workspace (density matrix)
  int lwork = 0;
  int64_t refined = 0;                      // eigenvectors recomputed by the second level
};

// Second level of the density-matrix factorisation: Gram eigenvalues below 1e-11 times the
// largest of the block (singular values below about 3e-6 of the block's largest) have
// eigenvectors fixed only to eps * lambda_max / gap by the first eigen-decomposition, which at
// a DMRG truncation cut mixes kept and discarded directions. Their subspace is decomposed
// again through its own Gram matrix, whose entries are of the size of those eigenvalues, so the
// second decomposition resolves them to eps relative to the largest of them.
constexpr double kRefineDefault = 1e-11;
double refine_threshold() {  // MPSG_GRAM_REFINE overrides it (0: no second level)
  const char* e = std::getenv("MPSG_GRAM_REFINE");
  return e ? std::atof(e) : kRefineDefault;
}

// Exact thin SVD of one column-major M x N block with cuSOLVER's QR-iteration SVD (gesvd, the
// method of the reference's fallback, src/symtools.jl:14-19). gesvd wants M >= N, so a wide
// block is factorised through its transpose. Buffers are allocated by the caller (prepare_exact)
// on the context stream; this only enqueues work on the lane's stream.
void prepare_exact(Context* ctx, cusolverDnHandle_t h, BlockSVD& B) {
  const int64_t M = B.M, N = B.N, k = B.k;
  B.U = alloc_buffer(ctx, M * k);
  B.S = alloc_buffer(ctx, k);
  B.V = alloc_buffer(ctx, N * k);
  B.work = alloc_buffer(ctx, M * N);
  B.aux = alloc_buffer(ctx, k * k);
  const int64_t m = std::max(M, N), n = std::min(M, N);
  MPSG_SOLVER(cusolverDnDgesvd_bufferSize(h, (int)m, (int)n, &B.lwork));
  B.wbuf = alloc_buffer(ctx, std::max(B.lwork, 1));
}

void run_exact(Context* ctx, cudaStream_t st, cusolverDnHandle_t h, const double* A, BlockSVD& B,
               int* dinfo) {
  const int64_t M = B.M, N = B.N, k = B.k;
  if (M >= N) {
    MPSG_CUDA(cudaMemcpyAsync(B.work->ptr, A, sizeof(double) * M * N, cudaMemcpyDeviceToDevice,
                              st));
    // A = U S VT with VT (N x N) in aux; V = VT^T
    MPSG_SOLVER(cusolverDnDgesvd(h, 'S', 'S', (int)M, (int)N, B.work->ptr, (int)M, B.S->ptr,
                                 B.U->ptr, (int)M, B.aux->ptr, (int)N, B.wbuf->ptr, B.lwork,
                                 nullptr, dinfo));
    dim3 g((unsigned)((N + 31) / 32), (unsigned)((N + 31) / 32));
    transpose_prefix_kernel<<<g, dim3(32, 8), 0, st>>>(B.V->ptr, B.aux->ptr, N, N);
  } else {
    // A^T (N x M) = U' S V'^T  =>  A = V' S U'^T: V = U' (N x M), U = V'^T^T from aux (M x M)
    dim3 g((unsigned)((N + 31) / 32), (unsigned)((M + 31) / 32));
    transpose_prefix_kernel<<<g, dim3(32, 8), 0, st>>>(B.work->ptr, A, N, M);
    MPSG_SOLVER(cusolverDnDgesvd(h, 'S', 'S', (int)N, (int)M, B.work->ptr, (int)N, B.S->ptr,
                                 B.V->ptr, (int)N, B.aux->ptr, (int)M, B.wbuf->ptr, B.lwork,
                                 nullptr, dinfo));
    dim3 g2((unsigned)((M + 31) / 32), (unsigned)((M + 31) / 32));
    transpose_prefix_kernel<<<g2, dim3(32, 8), 0, st>>>(B.U->ptr, B.aux->ptr, M, M);
  }
  MPSG_CUDA(cudaGetLastError());
  (void)k;
}

// Jacobi SVD of one block on the context stream: the second method tried when QR iteration
// reports non-convergence.
void run_jacobi(Context* ctx, const double* A, BlockSVD& B) {
  cusolverDnHandle_t h = lanes(ctx).sol[0];
  const int64_t M = B.M, N = B.N, k = B.k;
  cudaStream_t st = lanes(ctx).st[0];
  MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
  auto work = alloc_buffer(ctx, M * N);
  MPSG_CUDA(cudaMemcpyAsync(work->ptr, A, sizeof(double) * M * N, cudaMemcpyDeviceToDevice,
                            ctx->stream));
  MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
  gesvdjInfo_t params;
  MPSG_SOLVER(cusolverDnCreateGesvdjInfo(&params));
  int lwork = 0;
  MPSG_SOLVER(cusolverDnDgesvdj_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, 1, (int)M, (int)N,
                                           work->ptr, (int)M, B.S->ptr, B.U->ptr, (int)M,
                                           B.V->ptr, (int)N, &lwork, params));
  auto wbuf = alloc_buffer(ctx, std::max(lwork, 1));
  int* dinfo = nullptr;
  MPSG_CUDA(cudaMallocAsync((void**)&dinfo, sizeof(int), ctx->stream));
  MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
  MPSG_SOLVER(cusolverDnDgesvdj(h, CUSOLVER_EIG_MODE_VECTOR, 1, (int)M, (int)N, work->ptr,
                                (int)M, B.S->ptr, B.U->ptr, (int)M, B.V->ptr, (int)N, wbuf->ptr,
                                lwork, dinfo, params));
  int info = 0;
  MPSG_CUDA(cudaMemcpyAsync(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, st));
  MPSG_CUDA(cudaStreamSynchronize(st));
  cusolverDnDestroyGesvdjInfo(params);
  cudaFreeAsync(dinfo, ctx->stream);
  if (info != 0) throw Error(kErrNoConvergence, "block SVD did not converge");
  (void)k;
}

// Density-matrix factorisation of one block: the eigen-decomposition of the Gram matrix on the
// side whose factor must be orthonormal. Left: A A^T = U S^2 U^T, then V = A^T U S^-1. Right:
// A^T A = V S^2 V^T, then U = A V S^-1. The orthonormal factor is exact to rounding; the other
// satisfies U S V^T = U U^T A (left) or A V V^T (right) exactly, i.e. the product is the
// projection of A on the kept singular subspace, which is all a sweep uses of it.
void prepare_gram(Context* ctx, cusolverDnHandle_t h, BlockSVD& B, bool left) {
  const int64_t M = B.M, N = B.N, k = B.k, n = left ? M : N;
  B.U = alloc_buffer(ctx, M * k);
  B.S = alloc_buffer(ctx, k);
  B.V = alloc_buffer(ctx, N * k);
  B.work = alloc_buffer(ctx, n * n);
  B.aux = alloc_buffer(ctx, n);
  MPSG_SOLVER(cusolverDnDsyevd_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                          (int)n, B.work->ptr, (int)n, B.aux->ptr, &B.lwork));
  int lwork2 = 0;  // the second level decomposes at most k x k
  MPSG_SOLVER(cusolverDnDsyevd_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                          (int)k, B.work->ptr, (int)k, B.aux->ptr, &lwork2));
  B.lwork = std::max(B.lwork, lwork2);
  B.wbuf = alloc_buffer(ctx, std::max(B.lwork, 1));
  const int64_t rows = left ? N : M;  // rows of the other factor
  B.ref = alloc_buffer(ctx, rows * k + 2 * k * k + n * k + 2 * k);
}

void run_gram(Context* ctx, cudaStream_t st, cusolverDnHandle_t h, cublasHandle_t bl,
              const double* A, BlockSVD& B, bool left, int* dinfo) {
  const int64_t M = B.M, N = B.N, k = B.k, n = left ? M : N;
  const double one = 1.0, zero = 0.0;
  double* G = B.work->ptr;
  if (left)
    MPSG_BLAS(cublasDsyrk(bl, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, (int)M, (int)N, &one, A,
                          (int)M, &zero, G, (int)M));
  else
    MPSG_BLAS(cublasDsyrk(bl, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, (int)N, (int)M, &one, A,
                          (int)M, &zero, G, (int)N));
  MPSG_SOLVER(cusolverDnDsyevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, (int)n, G,
                               (int)n, B.aux->ptr, B.wbuf->ptr, B.lwork, dinfo));
  double* X = left ? B.U->ptr : B.V->ptr;  // orthonormal factor
  double* Y = left ? B.V->ptr : B.U->ptr;  // the other one
  top_eigpairs_kernel<<<grid_for(n * k), 256, 0, st>>>(X, B.S->ptr, G, B.aux->ptr, n, k);
  const int64_t rows = left ? N : M;
  // second level: the eigenvalues decide how many trailing columns of X to redo
  std::vector<double> w(n);
  int info = 0;
  MPSG_CUDA(cudaMemcpyAsync(w.data(), B.aux->ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  MPSG_CUDA(cudaMemcpyAsync(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, st));
  MPSG_CUDA(cudaStreamSynchronize(st));
  int64_t p = 0;
  const double thr = refine_threshold();
  if (info == 0 && n > 0 && w[n - 1] > 0 && thr > 0)
    for (int64_t i = 0; i < k; ++i)
      if (w[n - 1 - i] < thr * w[n - 1]) ++p;
  if (p >= 2) {
    double* Xs = X + n * (k - p);  // the trailing p columns (smallest eigenvalues of the top k)
    double* Ys = B.ref->ptr;       // rows x p
    double* Gs = Ys + rows * k;    // p x p
    double* Rs = Gs + k * k;       // p x p, descending
    double* Xt = Rs + k * k;       // n x p
    double* ws = Xt + n * k;       // p eigenvalues, p square roots (unused)
    if (left)  // Ys = A^T Xs
      MPSG_BLAS(cublasDgemm(bl, CUBLAS_OP_T, CUBLAS_OP_N, (int)N, (int)p, (int)M, &one, A, (int)M,
                            Xs, (int)M, &zero, Ys, (int)N));
    else  // Ys = A Xs
      MPSG_BLAS(cublasDgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, (int)M, (int)p, (int)N, &one, A, (int)M,
                            Xs, (int)N, &zero, Ys, (int)M));
    MPSG_BLAS(cublasDsyrk(bl, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, (int)p, (int)rows, &one, Ys,
                          (int)rows, &zero, Gs, (int)p));
    MPSG_SOLVER(cusolverDnDsyevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, (int)p, Gs,
                                 (int)p, ws, B.wbuf->ptr, B.lwork, dinfo));
    top_eigpairs_kernel<<<grid_for(p * p), 256, 0, st>>>(Rs, ws + k, Gs, ws, p, p);
    MPSG_BLAS(cublasDgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, (int)n, (int)p, (int)p, &one, Xs, (int)n,
                          Rs, (int)p, &zero, Xt, (int)n));
    MPSG_CUDA(cudaMemcpyAsync(Xs, Xt, sizeof(double) * n * p, cudaMemcpyDeviceToDevice, st));
    B.refined = p;
  }
  if (left)  // V (N x k) = A^T U
    MPSG_BLAS(cublasDgemm(bl, CUBLAS_OP_T, CUBLAS_OP_N, (int)N, (int)k, (int)M, &one, A, (int)M,
                          X, (int)M, &zero, Y, (int)N));
  else  // U (M x k) = A V
    MPSG_BLAS(cublasDgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, (int)M, (int)k, (int)N, &one, A, (int)M,
                          X, (int)N, &zero, Y, (int)M));
  col_norms_kernel<<<(unsigned)std::min<int64_t>((k + 7) / 8, 1184), 256, 0, st>>>(Y, B.S->ptr,
                                                                                 rows, k);
  running_min_kernel<<<1, 1, 0, st>>>(B.S->ptr, k);
  scale_cols_inv_kernel<<<grid_for(rows * k), 256, 0, st>>>(Y, B.S->ptr, rows, k);
  MPSG_CUDA(cudaGetLastError());
}

}  // namespace

std::vector<int64_t> truncatedsizes(const std::vector<std::vector<double>>& S, int64_t maxdim,
                                    double tol, double tieband) {
  const size_t n = S.size();
  std::vector<int64_t> ptr(n, 0);
  std::vector<double> c(n, 0.0);
  int64_t total = 0;
  double cmax = 0.0;
  for (size_t i = 0; i < n; ++i) {
    c[i] = S[i].empty() ? 0.0 : S[i][0];
    total += (int64_t)S[i].size();
    cmax = std::max(cmax, c[i]);
  }
  const double band = tieband > 0 ? tieband * cmax : 0.0;
  const int64_t steps = std::min(maxdim, total);
  for (int64_t it = 1; it <= steps; ++it) {
    size_t index = 0;
    double m = c[0];
    for (size_t i = 1; i < n; ++i)  // first maximum, like Julia's findmax
      if (c[i] > m) {
        m = c[i];
        index = i;
      }
    if (band > 0) {
      for (size_t i = 0; i < n; ++i)
        if (c[i] >= m - band) {
          index = i;
          m = c[i];
          break;
        }
    }
    if (m < tol) {
      if (it == 1)
        throw Error(kErrTolerance, "The largest singular value is smaller than tol!");
      break;
    }
    if (ptr[index] + 1 >= (int64_t)S[index].size()) {
      // exhausted sector: the reference sets 0.0 (below any tol > 0); -1 also keeps a tol <= 0
      // walk from stepping past the sector's last value
      ptr[index] += 1;
      c[index] = -1.0;
    } else {
      ptr[index] += 1;
      c[index] = S[index][ptr[index]];
    }
  }
  return ptr;
}

SVDResult svd_blocks(Context* ctx, const DeviceTensor& A, bool truncate, int64_t maxdim,
                     double tol, double tieband, int method) {
  if (A.meta.N() != 2) throw Error(kErrArgument, "svd needs a rank-2 tensor (SymMatrix)");
  if (method != kSvdExact && method != kSvdGramLeft && method != kSvdGramRight)
    throw Error(kErrArgument, "unknown SVD method");
  const size_t nb = A.meta.nblocks();
  SolverLanes& L = lanes(ctx);
  std::vector<BlockSVD> blocks(nb);
  std::vector<std::vector<double>> S(nb);
  // all buffers first (stream-ordered on the context stream), then fork the lanes
  for (size_t b = 0; b < nb; ++b) {
    BlockSVD& B = blocks[b];
    B.c1 = A.meta.sec.labels(b)[0];
    B.c2 = A.meta.sec.labels(b)[1];
    B.M = A.meta.sec.sizes(b)[0];
    B.N = A.meta.sec.sizes(b)[1];
    B.k = std::min(B.M, B.N);
    if (method == kSvdExact) prepare_exact(ctx, L.sol[0], B);
    else prepare_gram(ctx, L.sol[0], B, method == kSvdGramLeft);
  }
  int* dinfo = nullptr;
  if (nb) {
    MPSG_CUDA(cudaMallocAsync((void**)&dinfo, sizeof(int) * nb, ctx->stream));
    MPSG_CUDA(cudaMemsetAsync(dinfo, 0, sizeof(int) * nb, ctx->stream));
  }
  auto cost = [&](size_t b) {
    const double m = (double)std::max(blocks[b].M, blocks[b].N);
    const double n = (double)blocks[b].k;
    return m * n * n + n * n * n;
  };
  run_on_lanes(ctx, L, nb, cost, [&](int lane, size_t b) {
    const double* Ab = A.data() + A.meta.off[b];
    if (method == kSvdExact) run_exact(ctx, L.st[lane], L.sol[lane], Ab, blocks[b], dinfo + b);
    else run_gram(ctx, L.st[lane], L.sol[lane], L.blas[lane], Ab, blocks[b],
                  method == kSvdGramLeft, dinfo + b);
  });
  ctx->kernel_launches += (int64_t)nb * (method == kSvdExact ? 1 : 4);
  std::vector<int> info(nb, 0);
  if (nb)
    MPSG_CUDA(cudaMemcpyAsync(info.data(), dinfo, sizeof(int) * nb, cudaMemcpyDeviceToHost,
                              ctx->stream));
  for (size_t b = 0; b < nb; ++b) {
    S[b].resize(blocks[b].k);
    MPSG_CUDA(cudaMemcpyAsync(S[b].data(), blocks[b].S->ptr, sizeof(double) * blocks[b].k,
                              cudaMemcpyDeviceToHost, ctx->stream));
  }
  MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (dinfo) cudaFreeAsync(dinfo, ctx->stream);
  for (size_t b = 0; b < nb; ++b) {
    if (info[b] == 0) continue;
    if (method != kSvdExact) {
      // the Gram eigensolver failed on this block: factorise it exactly instead (QR-iteration
      // SVD, then Jacobi), which also leaves u and v orthonormal with u s v = A
      BlockSVD E;
      E.c1 = blocks[b].c1;
      E.c2 = blocks[b].c2;
      E.M = blocks[b].M;
      E.N = blocks[b].N;
      E.k = blocks[b].k;
      prepare_exact(ctx, L.sol[0], E);
      int* d1 = nullptr;
      MPSG_CUDA(cudaMallocAsync((void**)&d1, sizeof(int), ctx->stream));
      MPSG_CUDA(cudaMemsetAsync(d1, 0, sizeof(int), ctx->stream));
      MPSG_CUDA(cudaEventRecord(L.fork, ctx->stream));
      MPSG_CUDA(cudaStreamWaitEvent(L.st[0], L.fork, 0));
      run_exact(ctx, L.st[0], L.sol[0], A.data() + A.meta.off[b], E, d1);
      ctx->kernel_launches += 1;
      MPSG_CUDA(cudaEventRecord(L.join[0], L.st[0]));
      MPSG_CUDA(cudaStreamWaitEvent(ctx->stream, L.join[0], 0));
      int i1 = 0;
      MPSG_CUDA(cudaMemcpyAsync(&i1, d1, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
      cudaFreeAsync(d1, ctx->stream);
      if (i1 != 0) run_jacobi(ctx, A.data() + A.meta.off[b], E);
      blocks[b].U = E.U;
      blocks[b].S = E.S;
      blocks[b].V = E.V;
    } else {
      run_jacobi(ctx, A.data() + A.meta.off[b], blocks[b]);
    }
    MPSG_CUDA(cudaMemcpy(S[b].data(), blocks[b].S->ptr, sizeof(double) * blocks[b].k,
                         cudaMemcpyDeviceToHost));
  }
  std::vector<int64_t> ns(nb);
  int64_t total = 0;
  for (size_t b = 0; b < nb; ++b) total += blocks[b].k;
  // keep-everything requests (tol <= 0, maxdim >= total) skip the greedy walk, which with
  // tol = 0 could step past an exhausted sector on zero values
  const bool keep_all = tol <= 0.0 && maxdim >= total;
  if (truncate && !keep_all) {
    ns = truncatedsizes(S, maxdim, tol, tieband);
  } else {
    for (size_t b = 0; b < nb; ++b) ns[b] = blocks[b].k;
  }
  std::vector<std::pair<int, int64_t>> pl, pr;
  SVDResult R;
  for (size_t b = 0; b < nb; ++b) {
    if (ns[b] <= 0) continue;
    pl.push_back({blocks[b].c1, ns[b]});
    pr.push_back({blocks[b].c2, ns[b]});
    R.singular_values.push_back(std::vector<double>(S[b].begin(), S[b].begin() + ns[b]));
    R.kept_sectors.push_back({blocks[b].c1, blocks[b].c2});
  }
  if (pl.empty()) throw Error(kErrTolerance, "no singular value kept");
  Space Vl = Space::make(pl, A.meta.space[0].dual);
  Space Vr = Space::make(pr, A.meta.space[1].dual);
  TensorMeta mu = TensorMeta::build(0, {A.meta.space[0], dual_space(Vl)});
  TensorMeta ms = TensorMeta::build(A.meta.charge, {Vl, Vr});
  TensorMeta mv = TensorMeta::build(0, {dual_space(Vr), A.meta.space[1]});
  R.u = new_tensor(ctx, mu, false);
  R.s = new_tensor(ctx, ms, true);
  R.s.diag = true;
  R.v = new_tensor(ctx, mv, false);
  for (size_t b = 0; b < nb; ++b) {
    const int64_t r = ns[b];
    if (r <= 0) continue;
    const BlockSVD& B = blocks[b];
    int su[2] = {B.c1, B.c1}, ss[2] = {B.c1, B.c2}, sv[2] = {B.c2, B.c2};
    long iu = mu.find(su), is = ms.find(ss), iv = mv.find(sv);
    if (iu < 0 || is < 0 || iv < 0) throw Error(kErrSpaceMismatch, "svd: output sector missing");
    // U[:, 1:r] is the contiguous prefix of the column-major U
    MPSG_CUDA(cudaMemcpyAsync(R.u.data() + mu.off[iu], B.U->ptr, sizeof(double) * B.M * r,
                              cudaMemcpyDeviceToDevice, ctx->stream));
    set_diag_kernel<<<1, 256, 0, ctx->stream>>>(R.s.data() + ms.off[is], B.S->ptr, r);
    dim3 g((unsigned)((r + 31) / 32), (unsigned)((B.N + 31) / 32));
    transpose_prefix_kernel<<<g, dim3(32, 8), 0, ctx->stream>>>(R.v.data() + mv.off[iv],
                                                               B.V->ptr, r, B.N);
    MPSG_CUDA(cudaGetLastError());
    ctx->kernel_launches += 2;
  }
  return R;
}

// Complex per-sector SVD: the blocks are (re + i im), factorised with cuSOLVER's complex
// QR-iteration SVD on the solver lanes; A = U S V^H per sector, and v holds V^H (the layout of
// the real path, where v holds V^T). A wide block is factorised through A^H = U' S V'^H, so that
// U = V' and V^H = U'^H.
CSVDResult svd_blocks_complex(Context* ctx, const DeviceTensor& Are, const DeviceTensor& Aim,
                              bool truncate, int64_t maxdim, double tol, double tieband) {
  if (Are.meta.N() != 2) throw Error(kErrArgument, "svd needs a rank-2 tensor (SymMatrix)");
  if (!same_meta(Are.meta, Aim.meta))
    throw Error(kErrSpaceMismatch, "real and imaginary parts differ in charge or spaces");
  if (Are.diag || Aim.diag) throw Error(kErrArgument, "complex svd of a diagonal tensor");
  struct CBlock {
    int c1, c2;
    int64_t M, N, k;
    std::shared_ptr<Buffer> work, U, VT, S, wbuf, rwork;
    int lwork = 0;
  };
  const size_t nb = Are.meta.nblocks();
  SolverLanes& L = lanes(ctx);
  std::vector<CBlock> blocks(nb);
  for (size_t b = 0; b < nb; ++b) {
    CBlock& B = blocks[b];
    B.c1 = Are.meta.sec.labels(b)[0];
    B.c2 = Are.meta.sec.labels(b)[1];
    B.M = Are.meta.sec.sizes(b)[0];
    B.N = Are.meta.sec.sizes(b)[1];
    B.k = std::min(B.M, B.N);
    const int64_t m = std::max(B.M, B.N), n = B.k;
    B.work = alloc_buffer(ctx, 2 * B.M * B.N);
    B.U = alloc_buffer(ctx, 2 * m * n);
    B.VT = alloc_buffer(ctx, 2 * n * n);
    B.S = alloc_buffer(ctx, n);
    B.rwork = alloc_buffer(ctx, std::max<int64_t>(n, 1));
    MPSG_SOLVER(cusolverDnZgesvd_bufferSize(L.sol[0], (int)m, (int)n, &B.lwork));
    B.wbuf = alloc_buffer(ctx, 2 * std::max(B.lwork, 1));
  }
  int* dinfo = nullptr;
  if (nb) {
    MPSG_CUDA(cudaMallocAsync((void**)&dinfo, sizeof(int) * nb, ctx->stream));
    MPSG_CUDA(cudaMemsetAsync(dinfo, 0, sizeof(int) * nb, ctx->stream));
  }
  auto cost = [&](size_t b) {
    const double m = (double)std::max(blocks[b].M, blocks[b].N), n = (double)blocks[b].k;
    return m * n * n + n * n * n;
  };
  run_on_lanes(ctx, L, nb, cost, [&](int lane, size_t b) {
    CBlock& B = blocks[b];
    cudaStream_t st = L.st[lane];
    const double* re = Are.data() + Are.meta.off[b];
    const double* im = Aim.data() + Aim.meta.off[b];
    auto* W = (cuDoubleComplex*)B.work->ptr;
    auto* U = (cuDoubleComplex*)B.U->ptr;
    auto* VT = (cuDoubleComplex*)B.VT->ptr;
    auto* WB = (cuDoubleComplex*)B.wbuf->ptr;
    const bool tall = B.M >= B.N;
    // tall: work = A (M x N); wide: work = A^H (N x M)
    interleave_kernel<<<grid_for(B.M * B.N), 256, 0, st>>>((double2*)W, re, im, tall ? 1.0 : -1.0,
                                                          B.M, B.N, tall ? 0 : 1);
    MPSG_CUDA(cudaGetLastError());
    const int m = (int)std::max(B.M, B.N), n = (int)B.k;
    MPSG_SOLVER(cusolverDnZgesvd(L.sol[lane], 'S', 'S', m, n, W, m, B.S->ptr, U, m, VT, n, WB,
                                 B.lwork, B.rwork->ptr, dinfo + b));
  });
  ctx->kernel_launches += (int64_t)nb;
  std::vector<int> info(nb, 0);
  std::vector<std::vector<double>> S(nb);
  if (nb)
    MPSG_CUDA(cudaMemcpyAsync(info.data(), dinfo, sizeof(int) * nb, cudaMemcpyDeviceToHost,
                              ctx->stream));
  for (size_t b = 0; b < nb; ++b) {
    S[b].resize(blocks[b].k);
    MPSG_CUDA(cudaMemcpyAsync(S[b].data(), blocks[b].S->ptr, sizeof(double) * blocks[b].k,
                              cudaMemcpyDeviceToHost, ctx->stream));
  }
  MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (dinfo) cudaFreeAsync(dinfo, ctx->stream);
  for (size_t b = 0; b < nb; ++b)
    if (info[b] != 0) throw Error(kErrNoConvergence, "complex block SVD did not converge");
  int64_t total = 0;
  for (size_t b = 0; b < nb; ++b) total += blocks[b].k;
  std::vector<int64_t> ns(nb);
  const bool keep_all = tol <= 0.0 && maxdim >= total;
  if (truncate && !keep_all) {
    ns = truncatedsizes(S, maxdim, tol, tieband);
  } else {
    for (size_t b = 0; b < nb; ++b) ns[b] = blocks[b].k;
  }
  std::vector<std::pair<int, int64_t>> pl, pr;
  CSVDResult R;
  for (size_t b = 0; b < nb; ++b) {
    if (ns[b] <= 0) continue;
    pl.push_back({blocks[b].c1, ns[b]});
    pr.push_back({blocks[b].c2, ns[b]});
    R.singular_values.push_back(std::vector<double>(S[b].begin(), S[b].begin() + ns[b]));
  }
  if (pl.empty()) throw Error(kErrTolerance, "no singular value kept");
  Space Vl = Space::make(pl, Are.meta.space[0].dual);
  Space Vr = Space::make(pr, Are.meta.space[1].dual);
  TensorMeta mu = TensorMeta::build(0, {Are.meta.space[0], dual_space(Vl)});
  TensorMeta ms = TensorMeta::build(Are.meta.charge, {Vl, Vr});
  TensorMeta mv = TensorMeta::build(0, {dual_space(Vr), Are.meta.space[1]});
  R.ure = new_tensor(ctx, mu, false);
  R.uim = new_tensor(ctx, mu, false);
  R.s = new_tensor(ctx, ms, true);
  R.s.diag = true;
  R.vre = new_tensor(ctx, mv, false);
  R.vim = new_tensor(ctx, mv, false);
  for (size_t b = 0; b < nb; ++b) {
    const int64_t r = ns[b];
    if (r <= 0) continue;
    const CBlock& B = blocks[b];
    int su[2] = {B.c1, B.c1}, ss[2] = {B.c1, B.c2}, sv[2] = {B.c2, B.c2};
    long iu = mu.find(su), is = ms.find(ss), iv = mv.find(sv);
    if (iu < 0 || is < 0 || iv < 0) throw Error(kErrSpaceMismatch, "svd: output sector missing");
    const auto* U = (const double2*)B.U->ptr;
    const auto* VT = (const double2*)B.VT->ptr;
    double *ure = R.ure.data() + mu.off[iu], *uim = R.uim.data() + mu.off[iu];
    double *vre = R.vre.data() + mv.off[iv], *vim = R.vim.data() + mv.off[iv];
    cudaStream_t st = ctx->stream;
    if (B.M >= B.N) {  // u = U[:, :r] (M x r); v = VT[:r, :] (r x N)
      cplx_extract_kernel<<<grid_for(B.M * r), 256, 0, st>>>(ure, uim, U, B.M, r, B.M, 0, 0);
      cplx_extract_kernel<<<grid_for(r * B.N), 256, 0, st>>>(vre, vim, VT, r, B.N, B.N, 0, 0);
    } else {  // u = (V'^H)^H[:, :r] from VT' (M x M); v = U'^H[:r, :] from U' (N x M)
      cplx_extract_kernel<<<grid_for(B.M * r), 256, 0, st>>>(ure, uim, VT, B.M, r, B.M, 1, 1);
      cplx_extract_kernel<<<grid_for(r * B.N), 256, 0, st>>>(vre, vim, U, r, B.N, B.N, 1, 1);
    }
    set_diag_kernel<<<1, 256, 0, st>>>(R.s.data() + ms.off[is], B.S->ptr, r);
    MPSG_CUDA(cudaGetLastError());
    ctx->kernel_launches += 3;
  }
  return R;
}

}  // namespace mpsg
