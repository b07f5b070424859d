// Index decoding of the block-permute engine's copy tasks, shared by the kernel and by a host
// harness: magic-number division, the plain-division reference decode the device-checked build
// compares it with, and the address span of a task.
//
// A copy task moves an N-d block: position (i_0, ..., i_{n-1}), i_j < ext[j], goes from
// soff + sum_j i_j sstr[j] to doff + sum_j i_j dstr[j].
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define MPSG_HD __host__ __device__ __forceinline__
#else
#define MPSG_HD inline
#endif

namespace mpsg {

// q = n / d for every n < 2^31 as (hi32(n * m) + n) >> s, with m and s from magic_u31(d).
inline void magic_u31(uint32_t d, uint32_t& m, uint32_t& s) {
  uint32_t l = 0;
  while (((uint64_t)1 << l) < d) ++l;
  m = (uint32_t)((((uint64_t)1 << 32) * (((uint64_t)1 << l) - d)) / d + 1);
  s = l;
}

MPSG_HD uint32_t fdiv(uint32_t n, uint32_t m, uint32_t s) {
#if defined(__CUDA_ARCH__)
  return (__umulhi(n, m) + n) >> s;
#else
  return (uint32_t)((((uint64_t)n * m) >> 32) + n) >> s;
#endif
}

// Source and destination offsets of mixed-radix position q over the axes ax[0..nax) (ax[0]
// fastest), by plain division: the reference for the magic-number decode.
MPSG_HD void ref_decode(const int64_t* ext, const int64_t* sstr, const int64_t* dstr,
                        const int* ax, int nax, int64_t q, int64_t& so, int64_t& dof) {
  for (int j = 0; j < nax; ++j) {
    const int i = ax[j];
    const int64_t ii = q % ext[i];
    q /= ext[i];
    so += ii * sstr[i];
    dof += ii * dstr[i];
  }
}

// The same decode by magic-number division (what the copy kernel runs).
MPSG_HD void fast_decode(const int64_t* ext, const int64_t* sstr, const int64_t* dstr,
                         const uint32_t* mag, const uint32_t* shf, const int* ax, int nax,
                         uint32_t q, int64_t& so, int64_t& dof) {
  for (int j = 0; j < nax; ++j) {
    const int i = ax[j];
    const uint32_t qi = fdiv(q, mag[i], shf[i]);
    const int64_t ii = (int64_t)(q - qi * (uint32_t)ext[i]);
    q = qi;
    so += ii * sstr[i];
    dof += ii * dstr[i];
  }
}

// Lowest and highest offset one side of a task touches (off + sum of the extreme steps).
MPSG_HD void task_span(const int64_t* ext, const int64_t* str, int nd, int64_t off, int64_t& lo,
                       int64_t& hi) {
  lo = hi = off;
  for (int i = 0; i < nd; ++i) {
    const int64_t step = (ext[i] > 0 ? ext[i] - 1 : 0) * str[i];
    if (step < 0) lo += step;
    else hi += step;
  }
}

}  // namespace mpsg
