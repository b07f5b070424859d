// Many prepared two-site effective Hamiltonians applied as one (independent DMRG chains on one
// GPU), the lock-step Lanczos solver over them, and the tuner of the split-precision GEMM.
#pragma once

#include "linalg.hpp"
#include "ops.hpp"
#include "split.hpp"

namespace mpsg {

// Two-site H_eff of n chains (any structures, one slice count S >= 2) prepared together. Every
// phase of an application is ONE launch over all chains: the per-chain copy lists, packing
// tables and sector GEMM problem lists are concatenated, with every chain's data in its own
// segment of shared device buffers, and the two split GEMMs run as one persistent grouped
// launch each over the problems of all chains (tiles dealt largest K first across chains).
// The application (vin -> vout, 5 copy / pack / GEMM stages) is captured once in a CUDA graph
// and replayed. Operands and start vectors may belong to other contexts of the same device
// (one per chain): their producers must have finished (the caller synchronises those contexts)
// before they are passed in, and they must stay alive until the call returns.
struct HeffBatch {
  Context* ctx = nullptr;
  int S = 0, n = 0;
  bool use_graph = true;
  std::vector<TensorMeta> vmeta;
  std::vector<std::string> keys;                 // plan cache keys, handed back on destruction
  std::vector<std::shared_ptr<HeffPlans>> plans;
  std::vector<int64_t> voff;                     // chain i's segment of vin / vout (elements)
  int64_t vtot = 0;                              // length of vin / vout (segments 32-aligned)
  double ref_flops = 0;                          // reference 4-step flops of one application
  std::shared_ptr<Buffer> vin, vout, B1, C1, A2, C2;
  DevCopyPlan cin, cx2a, cout;
  split::SplitPlan g1, g2;
  split::Tuning t1, t2;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t graph_kernels = 0;  // kernels of one replay
  int64_t applies = 0;
  void run_launches();
  void apply();  // vin -> vout on the context stream
  ~HeffBatch();
};

std::unique_ptr<HeffBatch> heff_batch_create(Context* ctx, const std::vector<TensorMeta>& vmeta,
                                             const std::vector<const DeviceTensor*>& envL,
                                             const std::vector<const DeviceTensor*>& envR,
                                             const std::vector<const DeviceTensor*>& W1,
                                             const std::vector<const DeviceTensor*>& W2,
                                             int precision, bool use_graph);

// The same batch from operators prepared by heff_prepare on the chains' own contexts (same
// device, same precision; their preparation must have finished): the batch copies their fused
// constant operands and reads their host task lists, and keeps no reference to them.
std::unique_ptr<HeffBatch> heff_batch_from_ops(Context* ctx, const std::vector<const HeffOp*>& ops,
                                               bool use_graph);

// Lowest eigenpair of every chain's H_eff from its start vector, by the thick-restart Lanczos
// of eigsolve_heff2 run for all chains in lock step: one batched application per Krylov step
// (a graph replay), and the recurrence (reorthogonalisation dots, vector updates, the projected
// eigenproblems, restarts) as a fixed handful of launches over all chains. Chains that finish
// early drop out of the recurrence; their segments of the application are not read.
std::vector<EigResult> eigsolve_heff2_batch(HeffBatch& B, const std::vector<const DeviceTensor*>& x0,
                                            int krylovdim, int maxiter, double tol);

// Tuner of the split-precision grouped GEMM: the shape class of a problem list (slice count
// and histogram of problem shapes in factor-4 buckets) -> the fastest configuration among the
// N tiles and tile orders the kernel supports, measured on the device with CUDA events the
// first time the class is met and cached in the context.
std::string tune_shape_class(const std::vector<GemmTask>& g, int S);
split::Tuning tune_split(Context* ctx, const std::vector<GemmTask>& g, int S);

}  // namespace mpsg
