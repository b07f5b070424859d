// Index decoding of the block-permute engine's copy tasks, shared by the kernel and by a host
// harness: magic-number division, the plain-division reference decode the device-checked build
// compares it with, and the address span of a task.
//
// A copy task moves an N-d block: position (i_0, ..., i_{n-1}), i_j < ext[j], goes from
// soff + sum_j i_j sstr[j] to doff + sum_j i_j dstr[j].
#pragma once

#include <cstdint>
#include <vector>

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

// One unit of the row path: element i < len (len <= the unit bound) goes from
// src + soff + i * sstr to dst + doff + i * dstr. Rows with sstr == 1 are staged through shared
// memory by bulk asynchronous copies; the others are read element by element.
struct BulkRow {
  int64_t soff, doff;
  int32_t len, sstr, dstr, pad;
};

// 16-byte-aligned interior [i0, i1) of the byte span of len doubles starting at byte address a0
// (i1 == i0 when there is none): the part of a row a bulk asynchronous copy can move. At most
// one element before i0 and one after i1 remain.
MPSG_HD void row_interior(uint64_t a0, int64_t len, uint64_t& i0, uint64_t& i1) {
  const uint64_t a1 = a0 + 8 * (uint64_t)len;
  i0 = (a0 + 15) & ~(uint64_t)15;
  i1 = a1 & ~(uint64_t)15;
  if (i1 < i0) i1 = i0;
}

// Appends the rows of a task along axis a: one row per position of the other axes (decoded by
// plain division, the first other axis fastest), each cut into ceil(ext[a] / max_elems) pieces
// of nearly equal length. Strides along a must fit in 32 bits.
inline void append_bulk_rows(int nd, const int64_t* ext, const int64_t* sstr,
                             const int64_t* dstr, int64_t soff, int64_t doff, int a,
                             int max_elems, std::vector<BulkRow>& rows) {
  int ax[16];
  int nax = 0;
  int64_t outer = 1;
  for (int i = 0; i < nd; ++i)
    if (i != a) {
      ax[nax++] = i;
      outer *= ext[i];
    }
  const int64_t len = ext[a];
  const int64_t pieces = (len + max_elems - 1) / max_elems;
  const int64_t base = len / pieces, extra = len % pieces;  // `extra` pieces get one more
  for (int64_t q = 0; q < outer; ++q) {
    int64_t so = soff, dof = doff;
    ref_decode(ext, sstr, dstr, ax, nax, q, so, dof);
    int64_t c = 0;
    for (int64_t p = 0; p < pieces; ++p) {
      const int64_t n = base + (p < extra ? 1 : 0);
      rows.push_back(BulkRow{so + c * sstr[a], dof + c * dstr[a], (int32_t)n, (int32_t)sstr[a],
                             (int32_t)dstr[a], 0});
      c += n;
    }
  }
}

}  // namespace mpsg
