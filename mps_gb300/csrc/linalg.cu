// Per-sector SVD with greedy truncation (src/symtools.jl:1-35, src/mpsutils.jl:89-179) and the
// thick-restart Lanczos eigensolver that drives the two-site effective Hamiltonian (the role of
// KrylovKit.eigsolve at src/dmrg.jl:77-82).  Everything stays FP64 on the GPU; the host only
// sees singular values (for the truncation choice) and the small projected matrix.
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>

#include "linalg.hpp"

namespace mpsg {

#define MPSG_SOLVER(call)                                                                   \
  do {                                                                                      \
    cusolverStatus_t s_ = (call);                                                           \
    if (s_ != CUSOLVER_STATUS_SUCCESS)                                                      \
      throw ::mpsg::Error(::mpsg::kErrCuda, std::string(#call) + " failed: " + std::to_string((int)s_)); \
  } while (0)

namespace {

cusolverDnHandle_t solver(Context* ctx) {
  if (!ctx->solver) {
    cusolverDnHandle_t h;
    MPSG_SOLVER(cusolverDnCreate(&h));
    MPSG_SOLVER(cusolverDnSetStream(h, ctx->stream));
    ctx->solver = h;
    ctx->solver_destroy = [](void* p) { cusolverDnDestroy((cusolverDnHandle_t)p); };
  }
  return (cusolverDnHandle_t)ctx->solver;
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

struct BlockSVD {
  int c1, c2;
  int64_t M, N, k;
  std::shared_ptr<Buffer> U, S, V;  // U: M x k, S: k, V: N x k (all column-major)
};

// Thin SVD of one column-major M x N block with cuSOLVER's Jacobi SVD; on non-convergence it
// falls back to the QR-iteration SVD, as the reference falls back to LAPACK QRIteration
// (src/symtools.jl:14-19).
void block_svd(Context* ctx, const double* A, BlockSVD& out) {
  auto h = solver(ctx);
  const int64_t M = out.M, N = out.N, k = std::min(M, N);
  out.k = k;
  out.U = alloc_buffer(ctx, M * k);
  out.S = alloc_buffer(ctx, k);
  out.V = alloc_buffer(ctx, N * k);
  auto work = alloc_buffer(ctx, M * N);  // gesvdj overwrites its input
  MPSG_CUDA(cudaMemcpyAsync(work->ptr, A, sizeof(double) * M * N, cudaMemcpyDeviceToDevice,
                            ctx->stream));
  gesvdjInfo_t params;
  MPSG_SOLVER(cusolverDnCreateGesvdjInfo(&params));
  int lwork = 0;
  MPSG_SOLVER(cusolverDnDgesvdj_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, 1, (int)M, (int)N,
                                           work->ptr, (int)M, out.S->ptr, out.U->ptr, (int)M,
                                           out.V->ptr, (int)N, &lwork, params));
  auto wbuf = alloc_buffer(ctx, std::max(lwork, 1));
  int* dinfo = nullptr;
  MPSG_CUDA(cudaMallocAsync((void**)&dinfo, sizeof(int), ctx->stream));
  MPSG_SOLVER(cusolverDnDgesvdj(h, CUSOLVER_EIG_MODE_VECTOR, 1, (int)M, (int)N, work->ptr,
                                (int)M, out.S->ptr, out.U->ptr, (int)M, out.V->ptr, (int)N,
                                wbuf->ptr, lwork, dinfo, params));
  int info = 0;
  MPSG_CUDA(cudaMemcpyAsync(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
  cusolverDnDestroyGesvdjInfo(params);
  if (info != 0) {
    // QR-iteration fallback (needs M >= N: run on the transpose otherwise)
    MPSG_CUDA(cudaMemcpyAsync(work->ptr, A, sizeof(double) * M * N, cudaMemcpyDeviceToDevice,
                              ctx->stream));
    if (M >= N) {
      auto vt = alloc_buffer(ctx, N * N);
      MPSG_SOLVER(cusolverDnDgesvd_bufferSize(h, (int)M, (int)N, &lwork));
      auto w2 = alloc_buffer(ctx, std::max(lwork, 1));
      MPSG_SOLVER(cusolverDnDgesvd(h, 'S', 'S', (int)M, (int)N, work->ptr, (int)M, out.S->ptr,
                                   out.U->ptr, (int)M, vt->ptr, (int)N, w2->ptr, lwork, nullptr,
                                   dinfo));
      // V = VT^T
      dim3 g((unsigned)((N + 31) / 32), (unsigned)((N + 31) / 32));
      transpose_prefix_kernel<<<g, dim3(32, 8), 0, ctx->stream>>>(out.V->ptr, vt->ptr, N, N);
    } else {
      auto at = alloc_buffer(ctx, M * N);
      dim3 g((unsigned)((N + 31) / 32), (unsigned)((M + 31) / 32));
      // at (N x M) = A^T : rows of at = columns of A
      transpose_prefix_kernel<<<g, dim3(32, 8), 0, ctx->stream>>>(at->ptr, A, N, M);
      auto vt = alloc_buffer(ctx, M * M);
      MPSG_SOLVER(cusolverDnDgesvd_bufferSize(h, (int)N, (int)M, &lwork));
      auto w2 = alloc_buffer(ctx, std::max(lwork, 1));
      // A^T = U' S V'^T  =>  A = V' S U'^T: U = V' (M x M), V = U' (N x M)
      MPSG_SOLVER(cusolverDnDgesvd(h, 'S', 'S', (int)N, (int)M, at->ptr, (int)N, out.S->ptr,
                                   out.V->ptr, (int)N, vt->ptr, (int)M, w2->ptr, lwork, nullptr,
                                   dinfo));
      dim3 g2((unsigned)((M + 31) / 32), (unsigned)((M + 31) / 32));
      transpose_prefix_kernel<<<g2, dim3(32, 8), 0, ctx->stream>>>(out.U->ptr, vt->ptr, M, M);
    }
    MPSG_CUDA(cudaMemcpyAsync(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (info != 0) {
      cudaFreeAsync(dinfo, ctx->stream);
      throw Error(kErrNoConvergence, "block SVD did not converge");
    }
  }
  cudaFreeAsync(dinfo, ctx->stream);
  ctx->kernel_launches += 1;
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
      ptr[index] += 1;
      c[index] = 0.0;
    } else {
      ptr[index] += 1;
      c[index] = S[index][ptr[index]];
    }
  }
  return ptr;
}

SVDResult svd_blocks(Context* ctx, const DeviceTensor& A, bool truncate, int64_t maxdim,
                     double tol, double tieband) {
  if (A.meta.N() != 2) throw Error(kErrArgument, "svd needs a rank-2 tensor (SymMatrix)");
  const size_t nb = A.meta.nblocks();
  std::vector<BlockSVD> blocks(nb);
  std::vector<std::vector<double>> S(nb);
  for (size_t b = 0; b < nb; ++b) {
    blocks[b].c1 = A.meta.sec.labels(b)[0];
    blocks[b].c2 = A.meta.sec.labels(b)[1];
    blocks[b].M = A.meta.sec.sizes(b)[0];
    blocks[b].N = A.meta.sec.sizes(b)[1];
    block_svd(ctx, A.data() + A.meta.off[b], blocks[b]);
    S[b].resize(blocks[b].k);
    MPSG_CUDA(cudaMemcpyAsync(S[b].data(), blocks[b].S->ptr, sizeof(double) * blocks[b].k,
                              cudaMemcpyDeviceToHost, ctx->stream));
  }
  MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int64_t> ns(nb);
  if (truncate) {
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

}  // namespace mpsg
