// Host-side sector planner: U(1) charges, graded leg spaces, sector enumeration and the copy/GEMM
// task lists that realise permutelegs / fuselegs / splitleg / SymMatrix / block GEMM / split on
// the device.  Pure C++ (no CUDA), so every table can be checked on a CPU.
//
// Conventions follow the SymTensors layer of amiragha/mps:
//   * a sector is a tuple of raw charge labels, one per leg, ordered column-major
//     (last leg slowest: src/sector.jl:35-36);
//   * a leg with isdual=true contributes -label to the tensor charge (src/sector.jl:14-20);
//   * a tensor stores every allowed sector (src/sector.jl:69-92) as a column-major block, blocks
//     concatenated in sector order in one flat buffer.
#pragma once

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace mpsg {

constexpr int kMaxLegs = 16;   // legs per tensor (MPO chains fused in tests reach 10)
constexpr int kMaxTaskDims = 16;

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// Status codes returned across the C ABI (0 = success).
enum Status : int {
  kOk = 0,
  kErrArgument = 1,      // invalid argument (null pointer, bad leg index, ...)
  kErrSpaceMismatch = 2, // spaces/sectors that do not fit (reference: SpaceMismatch/SectorMismatch)
  kErrCuda = 3,          // a CUDA runtime or library call failed
  kErrNoConvergence = 4, // an iterative solver stopped without convergence (result still valid)
  kErrUnsupported = 5,   // operation the reference does not define either
  kErrTolerance = 6,     // largest singular value below tol (reference: error in truncatedsizes)
};

inline int eff(int label, bool isdual) { return isdual ? -label : label; }

// Graded space: sorted charges with positive dims and a dual flag (src/vspace.jl:5-18).
struct Space {
  std::vector<int> ch;
  std::vector<int64_t> dm;
  bool dual = false;

  int64_t dim(int c) const;
  int64_t total() const;
  int size() const { return (int)ch.size(); }
  bool operator==(const Space& o) const { return dual == o.dual && ch == o.ch && dm == o.dm; }
  bool operator!=(const Space& o) const { return !(*this == o); }
  static Space make(std::vector<std::pair<int, int64_t>> pairs, bool dual);  // validates + sorts
};

Space dual_space(const Space& V);
bool isdual_pair(const Space& a, const Space& b);
// Tensor product of spaces, fused right to left (src/vspace.jl:109-138).
Space fuse(bool dual, const std::vector<Space>& Vs);

// A list of sectors of N legs: labels (n*N) and block sizes (n*N).
struct SectorList {
  int N = 0;
  std::vector<int> lab;
  std::vector<int64_t> sz;
  size_t count() const { return N ? lab.size() / N : 0; }
  const int* labels(size_t i) const { return lab.data() + i * N; }
  const int64_t* sizes(size_t i) const { return sz.data() + i * N; }
  int64_t numel(size_t i) const {
    int64_t n = 1;
    for (int k = 0; k < N; ++k) n *= sz[i * N + k];
    return n;
  }
};

// All sectors of Vs adding up to `charge`, in sorted order (src/sector.jl:69-92).
SectorList allsectorsandsizes(int charge, const std::vector<Space>& Vs);

// Column-major sector order (reversed tuple compare).
bool sector_less(const int* a, const int* b, int N);

struct TensorMeta {
  int charge = 0;
  std::vector<Space> space;
  SectorList sec;
  std::vector<int64_t> off;   // block offsets (elements) in the flat buffer
  int64_t total = 0;

  int N() const { return (int)space.size(); }
  size_t nblocks() const { return sec.count(); }
  // Block index of a sector, -1 when absent (binary search in sector order).
  long find(const int* labels) const;
  static TensorMeta build(int charge, std::vector<Space> space);  // every allowed sector
};

bool same_meta(const TensorMeta& a, const TensorMeta& b);  // same charge and spaces

// One strided N-d copy: dst[doff + sum i_k*dstr_k] = src[soff + sum i_k*sstr_k] over the extents.
struct CopyTask {
  int nd = 0;
  int64_t ext[kMaxTaskDims];
  int64_t sstr[kMaxTaskDims];
  int64_t dstr[kMaxTaskDims];
  int64_t soff = 0, doff = 0;
  int64_t numel() const {
    int64_t n = 1;
    for (int i = 0; i < nd; ++i) n *= ext[i];
    return n;
  }
  void simplify();  // drop unit extents, merge axes contiguous in both src and dst
};

// One block GEMM: C[M x N] = A[M x K] * B[K x N], all column-major with the given leading
// dimensions; K == 0 writes zeros (an allowed sector without partner blocks, contract.jl:292-294).
struct GemmTask {
  int64_t M, N, K;
  int64_t offA, offB, offC;
  int64_t lda, ldb, ldc;
};

// SymMatrix(A, rows, cols) (contract.jl:112-171): fused meta + copy tasks A -> fused.
struct FusePlan {
  TensorMeta out;
  std::vector<CopyTask> tasks;
  bool identity = false;  // fused buffer is bit-identical to A's buffer
};
FusePlan plan_symmatrix(const TensorMeta& A, const std::vector<int>& rows1,
                        const std::vector<int>& cols1);

// A * B on rank-2 tensors (contract.jl:234-298).
struct MatmulPlan {
  TensorMeta out;
  std::vector<GemmTask> gemms;
  double flops = 0;
};
MatmulPlan plan_matmul(const TensorMeta& A, const TensorMeta& B);

// permutelegs (symreleg.jl:34-51), 1-based perm.
struct RelegPlan {
  TensorMeta out;
  std::vector<CopyTask> tasks;
  bool identity = false;
};
RelegPlan plan_permutelegs(const TensorMeta& A, const std::vector<int>& perm1);
RelegPlan plan_fuselegs(const TensorMeta& A, int l1, int n, bool dual);          // symreleg.jl:79-146
RelegPlan plan_splitleg(const TensorMeta& A, int l1, const std::vector<Space>& sp); // symreleg.jl:160-214
// SymTensor(C, rlegs, clegs) followed by permutelegs(., perm1) (contract.jl:187-224, 45-46).
RelegPlan plan_split_permute(const TensorMeta& C, const std::vector<Space>& rlegs,
                             const std::vector<Space>& clegs, const std::vector<int>& perm1);

// Affine map of one block of an intermediate tensor X, in X's own (column-major) axis order:
// element i of the block sits at off + sum_k i_k * str[k] of the other buffer.
struct BlockMap {
  int64_t off = 0;
  int64_t str[kMaxLegs] = {0};
};
// Same plans, also recording per X block where it comes from (split: fused C -> X) or where it
// goes (symmatrix: X -> fused matrix).
RelegPlan plan_split_permute_rec(const TensorMeta& C, const std::vector<Space>& rlegs,
                                 const std::vector<Space>& clegs, const std::vector<int>& perm1,
                                 std::vector<BlockMap>* src_of_x);
FusePlan plan_symmatrix_rec(const TensorMeta& X, const std::vector<int>& rows1,
                            const std::vector<int>& cols1, std::vector<BlockMap>* dst_of_x);
// Compose "split C into X" with "fuse X into a matrix" into one copy list C -> matrix, so X is
// never materialised.  X is the output structure of the split plan.
std::vector<CopyTask> compose_through(const TensorMeta& X, const std::vector<BlockMap>& src_of_x,
                                      const std::vector<BlockMap>& dst_of_x);

// _contract_index_perm (contract.jl:82-99): 1-based positions.
void contract_index_perm(const std::vector<int>& idx, std::vector<int>& rems,
                         std::vector<int>& cons, std::vector<int>& tofinals);

// Full contract(A, idxA, B, idxB) plan (contract.jl:11-47).
struct ContractPlan {
  FusePlan fa, fb;
  MatmulPlan mm;
  RelegPlan split;
  bool scalar = false;  // every leg contracted: result is a number
  double flops = 0;
  // arguments of the pieces, kept to compose plans of chained contractions
  std::vector<int> rowsA, colsA, rowsB, colsB;  // SymMatrix index lists (1-based)
  std::vector<Space> rlegs, clegs;              // legs of the split
  std::vector<int> perm;                        // final permutation (1-based)
};

// Host check of a composed plan: moves element indices through the two-step plan and through
// the composed list and compares (used by tests; throws Error on mismatch).
void check_composition(const std::vector<CopyTask>& step1, int64_t n_src, int64_t n_mid,
                       const std::vector<CopyTask>& step2, int64_t n_dst,
                       const std::vector<CopyTask>& composed);
std::shared_ptr<ContractPlan> plan_contract(const TensorMeta& A, const std::vector<int>& idxA,
                                            const TensorMeta& B, const std::vector<int>& idxB);

// Serialised key of a tensor's structure (charge + spaces), used by the plan cache.
std::string meta_key(const TensorMeta& m);

// Host self-checks of task lists (run by tests before anything reaches a GPU): every source and
// destination address in range, every destination element written exactly once, every GEMM
// operand window inside its buffer.  Throw Error on the first violation.
void validate_copy_tasks(const std::vector<CopyTask>& tasks, int64_t src_total,
                         int64_t dst_total);
void validate_gemms(const std::vector<GemmTask>& g, int64_t a_total, int64_t b_total,
                    int64_t c_total);
void validate_contract(const ContractPlan& p, const TensorMeta& A, const TensorMeta& B);

}  // namespace mpsg
