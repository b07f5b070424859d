// Handle types and the error guard shared by the C ABI translation units (capi.cu, noalloc.cu).
#pragma once

#include <new>
#include <string>
#include <vector>

#include "../../include/mpsgb300.h"
#include "runtime.hpp"

// The handle holds one reference to the context; device buffers hold the others, so
// mpsg_ctx_destroy never leaves a live tensor with a dangling stream.
struct mpsg_ctx {
  std::shared_ptr<mpsg::Context> owner;
  mpsg::Context& c;
  explicit mpsg_ctx(std::shared_ptr<mpsg::Context> p) : owner(std::move(p)), c(*owner) {}
};
struct mpsg_tensor {
  mpsg::DeviceTensor t;
};

namespace mpsg_capi {

void set_last_error(const std::string& msg);  // message returned by mpsg_last_error

// Runs f and maps exceptions to status codes (0 on success).
template <class F>
int guarded(F&& f) {
  try {
    f();
    return mpsg::kOk;
  } catch (const mpsg::Error& e) {
    set_last_error(e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    return mpsg::kErrArgument;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return mpsg::kErrArgument;
  }
}

inline void need(const void* p, const char* what) {
  if (!p) throw mpsg::Error(mpsg::kErrArgument, std::string("null argument: ") + what);
}

inline std::vector<int> ivec(const int32_t* p, int n) { return std::vector<int>(p, p + n); }

}  // namespace mpsg_capi
