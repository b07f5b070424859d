// Tensor-level operations built from the planner and the kernel launchers.
#pragma once

#include "runtime.hpp"
#include "split.hpp"

namespace mpsg {

void context_init(Context* ctx, int device);

DeviceTensor new_tensor(Context* ctx, const TensorMeta& meta, bool zero);
DeviceTensor copy_tensor(Context* ctx, const DeviceTensor& t);
DeviceTensor dual_view(const DeviceTensor& t);
void require_similar(const DeviceTensor& a, const DeviceTensor& b, const char* msg);

DeviceTensor permutelegs(Context* ctx, const DeviceTensor& a, const std::vector<int>& perm1);
DeviceTensor fuselegs(Context* ctx, const DeviceTensor& a, int l1, int n, bool dual);
DeviceTensor splitleg(Context* ctx, const DeviceTensor& a, int l1, const std::vector<Space>& sp);
DeviceTensor symmatrix(Context* ctx, const DeviceTensor& a, const std::vector<int>& rows,
                       const std::vector<int>& cols);
DeviceTensor matmul(Context* ctx, const DeviceTensor& a, const DeviceTensor& b, int precision);

// The GEMM part of a contraction (operand fusion + block products): the result in the plan's
// fused output layout, before the final split / permutation.
std::shared_ptr<Buffer> contract_gemm(Context* ctx, DevContract& p, const DeviceTensor& a,
                                      const DeviceTensor& b, int precision);
std::shared_ptr<DevContract> get_contract_plan(Context* ctx, const TensorMeta& A,
                                               const std::vector<int>& idxA,
                                               const TensorMeta& B,
                                               const std::vector<int>& idxB);
// Returns an empty tensor (no buffer, no legs) and sets *scalar when every leg is contracted.
DeviceTensor contract(Context* ctx, const DeviceTensor& a, const std::vector<int>& idxA,
                      const DeviceTensor& b, const std::vector<int>& idxB, int precision,
                      double* scalar);

DeviceTensor applymps2site(Context* ctx, const DeviceTensor& v, const DeviceTensor& envL,
                           const DeviceTensor& envR, const DeviceTensor& W1,
                           const DeviceTensor& W2, int precision);
double applymps2site_flops(Context* ctx, const TensorMeta& v, const TensorMeta& envL,
                           const TensorMeta& envR, const TensorMeta& W1, const TensorMeta& W2);
DeviceTensor mpsupdateleft(Context* ctx, const DeviceTensor& env, const DeviceTensor& A,
                           const DeviceTensor& W, int precision);
DeviceTensor mpsupdateright(Context* ctx, const DeviceTensor& env, const DeviceTensor& A,
                            const DeviceTensor& W, int precision);

double dot(Context* ctx, const DeviceTensor& a, const DeviceTensor& b);

// Two-site effective Hamiltonian prepared for repeated application.
//  * precision 0: the reference's four contractions (src/apply.jl:99-103) in FP64.
//  * precision S >= 2: W1 folded into envL and W2 into envR once (FP64), so that every
//    application is two large block GEMMs on the tensor cores:
//      X(l,s1',m',s2,r)  = envLW(l',s1,l,m',s1') . v(l',s1,s2,r)        over (l', s1)
//      v'(l,s1',s2',r')  = X . envRW(r,m',s2,s2',r')                      over (m', s2, r)
//    with the constant operands fused and sliced once.
// The structure-only part of a prepared split-precision H_eff: the two GEMM contraction plans
// (with their split-GEMM plans, which also hold the packed constant operands) and the composed
// copy list. Building it is host work (planning, table uploads, tensor maps); the context keeps
// idle ones by structure and precision so that the next operator of the same structure (the
// same bond in a later sweep, repeated reference-style calls) skips it. One live operator owns
// an entry at a time.
struct HeffPlans {
  std::shared_ptr<DevContract> c1, c2;
  DevCopyPlan x2a;                   // fused X of GEMM 1 -> fused A of GEMM 2 (X never built)
  std::vector<CopyTask> x2a_host;    // its host task list (batched operators concatenate it)
  DevCopyPlan lw2a, rw2b;            // fold outputs -> GEMM 1's A / GEMM 2's B (composed)
  size_t bytes = 0;                  // device storage held, for the cache budget
  ~HeffPlans() {
    x2a.release();
    lw2a.release();
    rw2b.release();
  }
};

struct HeffOp {
  Context* ctx = nullptr;
  int precision = 0;
  DeviceTensor envL, envR, W1, W2;   // precision 0

  TensorMeta vmeta;
  std::shared_ptr<HeffPlans> plans;  // precision >= 2
  std::string plan_key;
  std::shared_ptr<Buffer> fusedA1, fusedB2;
  // prepared for a batch (heff_prepare): the FP64 fused constant operands kept, no split plans
  // of its own; it cannot be applied alone
  bool batch_only = false;
  double ref_flops = 0;  // algorithmic flops of the reference contraction order
  // algorithmic bytes per application (precision >= 2): block-permute copies (8 read + 8 written
  // per element) and operand packing (exponent pass 8 read, slice pass 8 read + 2 S written)
  double copy_bytes = 0, pack_bytes = 0;
  ~HeffOp();             // hands `plans` back to the context's cache
};

// Host plans of the W-folded H_eff: the two folding contractions, the two GEMM contractions and
// the composed copy list from GEMM 1's fused output to GEMM 2's fused A operand.
struct FoldedHeffPlans {
  std::shared_ptr<ContractPlan> lw, rw, c1, c2;
  std::vector<CopyTask> x2a;
  // the folds' fused GEMM outputs moved straight into GEMM 1's A / GEMM 2's B operands
  // (envLW and envRW are never materialised)
  std::vector<CopyTask> lw2a, rw2b;
};
FoldedHeffPlans plan_heff_folded(const TensorMeta& v, const TensorMeta& envL,
                                 const TensorMeta& envR, const TensorMeta& W1,
                                 const TensorMeta& W2);
// Host self-check of those plans (bounds, coverage, composition == two steps).
void check_heff_folded(const TensorMeta& v, const TensorMeta& envL, const TensorMeta& envR,
                       const TensorMeta& W1, const TensorMeta& W2);
// The structure-only parts of a W-folded H_eff at `precision` slices: its plans (taken from the
// context's idle cache or built, without split-GEMM plans) and the two fold contractions.
struct HeffParts {
  std::shared_ptr<HeffPlans> plans;
  std::string key;  // cache key of `plans`
  std::shared_ptr<DevContract> plw, prw;
};
HeffParts heff_parts(Context* ctx, const TensorMeta& vmeta, const DeviceTensor& envL,
                     const DeviceTensor& envR, const DeviceTensor& W1, const DeviceTensor& W2,
                     int precision);
// The W folds in FP64, written straight into GEMM 1's fused A (dstA1, c1 fa layout) and GEMM
// 2's fused B (dstB2, c2 fb layout); each waits for its event first when one is given.
void heff_fold(Context* ctx, HeffParts& H, const DeviceTensor& envL, const DeviceTensor& envR,
               const DeviceTensor& W1, const DeviceTensor& W2, double* dstA1, double* dstB2,
               cudaEvent_t wait_left = nullptr, cudaEvent_t wait_right = nullptr);
// Hands idle plans back to the context's cache (LRU, a share of 8 GiB per process).
void heff_plans_return(Context* ctx, const std::string& key, std::shared_ptr<HeffPlans> plans);
// Split-GEMM kernel configuration for a task list at S slices: the tuner's cached choice for
// this shape class, tuning it first when the context's autotuning is on (batch.cu), else the
// defaults.
split::Tuning choose_tuning(Context* ctx, const std::vector<GemmTask>& g, int S);
// wait_left / wait_right: events the left / right W fold waits for (inputs still arriving)
std::shared_ptr<HeffOp> heff_create(Context* ctx, const TensorMeta& vmeta, const DeviceTensor& envL,
                                    const DeviceTensor& envR, const DeviceTensor& W1,
                                    const DeviceTensor& W2, int precision,
                                    cudaEvent_t wait_left = nullptr,
                                    cudaEvent_t wait_right = nullptr);
// _applymps2site from host arrays (v, envL, envR, W1, W2 in host_in, into the given device
// tensors) to a host array: the uploads run on a copy stream, each W fold starts as soon as its
// two inputs have arrived, and the result is downloaded before returning.
DeviceTensor applymps2site_host(Context* ctx, const DeviceTensor& v, const DeviceTensor& envL,
                                const DeviceTensor& envR, const DeviceTensor& W1,
                                const DeviceTensor& W2, const double* const host_in[5],
                                int precision, double* host_out);
DeviceTensor heff_apply(HeffOp& op, const DeviceTensor& v);
// The part of a batched H_eff that belongs to one chain, done on that chain's context: plans,
// and the W folds into FP64 fused operands kept in the operator (batch_only).
std::shared_ptr<HeffOp> heff_prepare(Context* ctx, const TensorMeta& vmeta,
                                     const DeviceTensor& envL, const DeviceTensor& envR,
                                     const DeviceTensor& W1, const DeviceTensor& W2, int precision);

// One host<->device copy on the context's copy stream, started after the work queued so far on
// the context stream. It holds the tensor's device buffer, so the tensor may be released at once;
// destroying an unfinished copy waits for it on the host.
struct AsyncCopy {
  std::shared_ptr<Context> owner;
  std::shared_ptr<Buffer> buf;
  cudaEvent_t done = nullptr;
  ~AsyncCopy();
};
void ensure_copy_stream(Context* ctx);
std::unique_ptr<AsyncCopy> copy_async(Context* ctx, const DeviceTensor& t, double* host,
                                      bool to_host);

}  // namespace mpsg
