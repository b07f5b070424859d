// Tensor-level operations built from the planner and the kernel launchers.
#pragma once

#include "runtime.hpp"

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

}  // namespace mpsg
