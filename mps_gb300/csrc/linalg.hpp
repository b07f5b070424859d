// FP64 per-sector SVD / truncation and the Lanczos eigensolver (see linalg.cu, krylov.cu).
#pragma once

#include "ops.hpp"

namespace mpsg {

// Greedy global truncation (src/mpsutils.jl:89-112): the maxdim largest values above the
// absolute tol, ties to the first sector; tieband > 0 widens "equal" to tieband * max(S).
std::vector<int64_t> truncatedsizes(const std::vector<std::vector<double>>& S, int64_t maxdim,
                                    double tol, double tieband);

struct SVDResult {
  DeviceTensor u, s, v;  // s stored as dense diagonal blocks (diag flag set)
  std::vector<std::vector<double>> singular_values;  // kept values per kept sector
  std::vector<std::pair<int, int>> kept_sectors;
};

// Per-block factorisation methods. Exact: thin SVD (QR iteration). Gram left / right: the
// density-matrix truncation, eigen-decomposition of A A^T (u orthonormal) or A^T A (v
// orthonormal); the other factor carries S^-1 times the projection of A, so u s v^T equals the
// projection of A on the kept singular subspace.
enum SvdMethod { kSvdExact = 0, kSvdGramLeft = 1, kSvdGramRight = 2 };

// _svd_ (truncate=false, src/symtools.jl:1-35) and svdtrunc (src/mpsutils.jl:116-179).
SVDResult svd_blocks(Context* ctx, const DeviceTensor& A, bool truncate, int64_t maxdim,
                     double tol, double tieband, int method = kSvdExact);

// Complex per-sector SVD of (re + i im): A = u s v with u (re, im) isometric, s real diagonal
// and v = V^H per sector; same truncation rule and output spaces as svd_blocks.
struct CSVDResult {
  DeviceTensor ure, uim, s, vre, vim;
  std::vector<std::vector<double>> singular_values;
};
CSVDResult svd_blocks_complex(Context* ctx, const DeviceTensor& Are, const DeviceTensor& Aim,
                              bool truncate, int64_t maxdim, double tol, double tieband);

struct EigResult {
  double value = 0;
  DeviceTensor vec;
  double normres = 0;
  int numiter = 0, numops = 0;
  bool converged = false;
};

// Lowest eigenpair of v -> _applymps2site(v, envL, envR, W1, W2) from x0 (thick-restart Lanczos
// with full reorthogonalisation; KrylovKit eigsolve(..., 1, :SR, ishermitian=true) semantics).
EigResult eigsolve_heff2(Context* ctx, const DeviceTensor& x0, const DeviceTensor& envL,
                         const DeviceTensor& envR, const DeviceTensor& W1, const DeviceTensor& W2,
                         int krylovdim, int maxiter, double tol, int precision);

// Symmetric eigen-decomposition of a small dense matrix (cyclic Jacobi, FP64), ascending.
void small_eigh(int n, const double* A, double* evals, double* evecs);

}  // namespace mpsg
