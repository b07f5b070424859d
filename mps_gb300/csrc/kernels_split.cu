// Split-precision grouped block GEMM on the 5th-generation tensor cores (tcgen05 + TMEM + TMA).
//
// C (FP64) = A (FP64) * B (FP64) for every sector GEMM of a contraction, computed from bf16
// slices of the operands (an error-free splitting in the style of Ozaki et al.):
//
//   * Packing.  Every row i of A (and every column j of B) is cut into K-chunks of `chunk`
//     columns.  With e(i,c) the power-of-two bound of row i in chunk c and R(i) = max_c e(i,c),
//     the chunk is written as a fixed-point integer F with beta*S fraction bits relative to
//     2^e(i,c), and F is split into S balanced base-2^beta digits t_0..t_{S-1}
//     (|t_0| <= 2^beta, |t_p| <= 2^(beta-1)); slice p stores t_p * 2^(e(i,c)-R(i)-beta(p+1)),
//     exactly representable in bf16.  All of this is integer arithmetic on the FP64 bit
//     pattern: GB300 executes FP64 at a small fraction of its FP32 rate.
//   * MMA.  For every slice pair (p, q) with p + q < S, tcgen05.mma (M=128, N=64 or 128, K=16,
//     bf16 in, FP32 out) accumulates group g = p + q into a TMEM accumulator: its own for
//     g <= S - 3, one shared by groups S - 2 and S - 1 (exact_accs).  Within one chunk every
//     product of an exact group g is an integer multiple of one power of two and the sum stays
//     below 2^24 units (chunk * 2^12 * max(4, g + 3) <= 2^24, exact_chunk), so its FP32
//     accumulation is exact; the shared accumulator of the two smallest groups rounds at
//     2^-24 of a sum weighted 2^(-7(S-2)), below the slicing error.
//   * Epilogue.  After each chunk the epilogue warps drain the S - 1 accumulators (tcgen05.ld)
//     into a double-single (hi, lo) FP32 pair per output element (TwoSum, exact up to 2^-48),
//     release TMEM to the MMA warp (double-buffered where it fits), and after the last chunk
//     assemble (hi + lo) * 2^(R(i) + C(j)) as an FP64 number with integer instructions only.
//
// Accuracy: slicing error <= 2^(-beta*S) relative to the row/column scale, so S = 2 is the
// classic "bf16x3" (3 products), S = 3 gives about 21 bits (6 products), S = 4 about 28 bits,
// S = 6 about 42 bits and S = 7 about 49 bits (28 products), the FP64-class setting.
//
// Kernel layout: persistent, one CTA per SM, 6 warps: warp 0 = TMA producer (one elected
// thread, cp.async.bulk.tensor 3-d loads of pre-packed K-major tiles with 128B swizzle), warp 1
// = TMEM allocator + MMA issuer (one thread), warps 2-5 = epilogue (one TMEM lane per thread).
// Every mbarrier wait is bounded (clock64 budget); on timeout the kernel records an error code,
// stops issuing work, waits for its own MMAs and frees TMEM before returning.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <type_traits>

#include "split.hpp"

namespace mpsg {
namespace split {

// ------------------------------------------------------------------------------------------
// device helpers (inline PTX)
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ uint32_t mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok;
}

constexpr long long kWaitCycles = 4000000000LL;  // about 2 s at the maximum SM clock

// Bounded wait on a barrier phase; returns false (and raises the abort flag) on timeout or when
// another role already aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                          int* err, int code) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if (clock64() - t0 > kWaitCycles) {
      *abort_flag = 1;
      atomicCAS(err, 0, code);
      return false;
    }
  }
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}

// 32 consecutive FP32 columns of one TMEM lane per thread (shape 32x32b, 32 repetitions)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
        "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
        "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// 16 consecutive FP32 columns of one TMEM lane per thread (shape 32x32b, 16 repetitions)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major operand tile, 128-byte swizzle, 8-row groups 1024 B
// apart (stride byte offset), base 1024-byte aligned.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                    // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset
  d |= (uint64_t)1 << 46;                    // descriptor version
  d |= (uint64_t)2 << 61;                    // 128-byte swizzle
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, bf16 A and B, both K-major.
__host__ __device__ constexpr uint32_t make_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// (hi + lo) * 2^E as FP64 using integer instructions only (hi, lo normal or zero FP32 values
// with |lo| <= |hi|; a non-finite hi is returned as is).  Bits below 2^-62 of |hi| are
// truncated.
__device__ __forceinline__ double ds_to_f64(float hi, float lo, int E) {
  if ((__float_as_uint(hi) & 0x7f800000u) == 0x7f800000u) return (double)hi;  // NaN / Inf
  if (hi == 0.f) {
    hi = lo;
    lo = 0.f;
    if (hi == 0.f) return 0.0;
  }
  const uint32_t uh = __float_as_uint(hi), ul = __float_as_uint(lo);
  const int eh = (int)((uh >> 23) & 0xff);
  const int el = (int)((ul >> 23) & 0xff);
  long long mh = (long long)((uh & 0x7fffffu) | (eh ? 0x800000u : 0u));
  if (uh >> 31) mh = -mh;
  long long I = mh << 38;  // value = I * 2^(eh - 150 - 38)
  if (lo != 0.f) {
    long long ml = (long long)((ul & 0x7fffffu) | (el ? 0x800000u : 0u));
    if (ul >> 31) ml = -ml;
    const int d = 38 - (eh - el);
    if (d >= 0) I += ml << d;
    else if (d > -63) I += ml >> (-d);
  }
  if (I == 0) return 0.0;
  const unsigned long long sign = I < 0 ? (1ull << 63) : 0ull;
  unsigned long long A = I < 0 ? (unsigned long long)(-I) : (unsigned long long)I;
  const int lz = __clzll((long long)A);
  A <<= lz;  // bit 63 set
  unsigned long long mant = A >> 11;
  const unsigned long long rest = A & 0x7ffull;
  if ((rest > 0x400ull) || (rest == 0x400ull && (mant & 1ull))) mant += 1;  // round to nearest
  int shift = 0;
  if (mant >> 53) {
    mant >>= 1;
    shift = 1;
  }
  // value = mant * 2^(63 - lz - 52 + shift) * 2^(eh - 188 + E - 11 + 11)
  const long long bexp = (long long)63 - lz + shift + (eh - 188) + E + 1023;
  if (bexp <= 0) return 0.0;  // below the normal range: negligible at this accuracy
  if (bexp >= 2047) return __longlong_as_double((long long)(sign | (0x7ffull << 52)));
  return __longlong_as_double(
      (long long)(sign | ((unsigned long long)bexp << 52) | (mant & ((1ull << 52) - 1))));
}

__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  const float s = __fadd_rn(hi, x);
  const float bv = __fsub_rn(s, hi);
  const float av = __fsub_rn(s, bv);
  const float err = __fadd_rn(__fsub_rn(hi, av), __fsub_rn(x, bv));
  hi = s;
  lo = __fadd_rn(lo, err);
}

__device__ __forceinline__ int find_problem(const int64_t* __restrict__ prefix, int n, int64_t t) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// ------------------------------------------------------------------------------------------
// packing kernels
// ------------------------------------------------------------------------------------------
// Operand view: element (r, k) of problem p at base[off + r*rs + k*ks]; A uses rows = M,
// (rs, ks) = (1, lda); B uses rows = N, (rs, ks) = (ldb, 1).
__device__ __forceinline__ void operand_geom(const Problem& P, int is_b, int64_t& rows,
                                             int64_t& off, int64_t& rs, int64_t& ks) {
  if (!is_b) {
    rows = P.M;
    off = P.offA;
    rs = 1;
    ks = P.lda;
  } else {
    rows = P.N;
    off = P.offB;
    rs = P.ldb;
    ks = 1;
  }
}

__device__ __forceinline__ int exp_bound(unsigned long long absbits) {
  // smallest e with |x| < 2^e for the largest |x| (0 when every value is 0)
  if (absbits == 0) return 0;
  const int eb = (int)(absbits >> 52);
  return (eb == 0 ? -1022 : eb - 1023) + 1;
}

constexpr int kNoExponent = (int)0x80808080;  // byte pattern of the reset: "row entirely zero"
constexpr unsigned long long kNonFinite = 0x7ff0000000000000ull;  // |bits| of Inf; NaN above

// One CTA per (problem, block of operand rows, K chunk): chunk exponents e(r,c), and the row
// reference R(r) = max_c e(r,c) by atomicMax (R is reset to kNoExponent before the pass).
// Loads are coalesced along whichever operand axis is contiguous. Row blocks of 32 rows: for A
// operands (row-contiguous) 32 rows x 8 K groups per CTA, for B operands (K-contiguous) one
// warp per row, four rows per warp.
constexpr int kExpRowsA = 32, kExpRowsB = 32;

__global__ void __launch_bounds__(256) pack_exponents_kernel(
    const Problem* __restrict__ probs, const int64_t* __restrict__ item_prefix, int nprob,
    int64_t nitems, int is_b, int chunk, int write_e, const double* __restrict__ X,
    int16_t* __restrict__ E,
    int32_t* __restrict__ R) {
  __shared__ unsigned long long red[8][33];
  const int t = threadIdx.x;
  const int rb = is_b ? kExpRowsB : kExpRowsA;
  for (int64_t it = blockIdx.x; it < nitems; it += gridDim.x) {
    const int p = find_problem(item_prefix, nprob, it);
    const Problem P = probs[p];
    const int64_t lt = it - item_prefix[p];
    int64_t rows, off, rs, ks;
    operand_geom(P, is_b, rows, off, rs, ks);
    const int64_t nrb = (rows + rb - 1) / rb;
    const int64_t r0 = (lt % nrb) * rb;
    const int c = (int)(lt / nrb);
    const int64_t k0 = (int64_t)c * chunk, k1 = min(k0 + chunk, P.K);
    const int64_t rbase = is_b ? P.rB : P.rA;
    const int64_t ebase = is_b ? P.eB : P.eA;
    if (rs == 1) {
      // 32 consecutive rows per warp-row of the CTA, 8 interleaved K groups
      const int r = t & 31, kg = t >> 5;
      unsigned long long m = 0;
      if (r0 + r < rows)
        for (int64_t k = k0 + kg; k < k1; k += 8) {
          unsigned long long b =
              (unsigned long long)__double_as_longlong(X[off + (r0 + r) + k * ks]) &
              0x7fffffffffffffffull;
          if (b >= kNonFinite) b = 0;  // NaN / Inf: packed as NaN slices, not a scale
          m = b > m ? b : m;
        }
      red[kg][r] = m;
      __syncthreads();
      if (t < 32 && r0 + t < rows) {
        unsigned long long mm = 0;
#pragma unroll
        for (int g = 0; g < 8; ++g) mm = red[g][t] > mm ? red[g][t] : mm;
        const int e = exp_bound(mm);
        if (write_e) E[ebase + (r0 + t) * P.nch + c] = (int16_t)e;
        if (mm) atomicMax(&R[rbase + r0 + t], e);
      }
      __syncthreads();
    } else {
      // one row per warp, lanes along the contiguous K axis
      const int lane = t & 31, w = t >> 5;
      for (int rr = w; rr < rb; rr += 8) {
        const int64_t r = r0 + rr;
        if (r >= rows) break;
        unsigned long long m = 0;
        for (int64_t k = k0 + lane; k < k1; k += 32) {
          unsigned long long b =
              (unsigned long long)__double_as_longlong(X[off + r * rs + k]) & 0x7fffffffffffffffull;
          if (b >= kNonFinite) b = 0;
          m = b > m ? b : m;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const unsigned long long q = __shfl_xor_sync(0xffffffffu, m, o);
          m = q > m ? q : m;
        }
        if (lane == 0) {
          const int e = exp_bound(m);
          if (write_e) E[ebase + r * P.nch + c] = (int16_t)e;
          if (m) atomicMax(&R[rbase + r], e);
        }
      }
    }
  }
}

// One CTA per packed tile (rows_per_tile x 64 K).  Writes S slices, row-major 128-byte rows.
// A thread owns 8 consecutive K of one row and reads them straight from global memory (no
// shared-memory staging, no barrier).
template <int S>
__global__ void __launch_bounds__(256) pack_slices_kernel(
    const Problem* __restrict__ probs, const int64_t* __restrict__ tile_prefix, int nprob,
    int64_t ntiles, int is_b, int chunk, int use_r, int rows_per_tile, int64_t rows_total,
    const double* __restrict__ X, const int16_t* __restrict__ E, const int32_t* __restrict__ R,
    __nv_bfloat16* __restrict__ out) {
  constexpr int kBeta = kSliceBits;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int p = find_problem(tile_prefix, nprob, t);
    const Problem P = probs[p];
    const int64_t lt = t - tile_prefix[p];
    const int64_t ri = lt / P.nks, kstep = lt % P.nks;
    int64_t rows, off, rs, ks;
    operand_geom(P, is_b, rows, off, rs, ks);
    const int64_t k0 = kstep * 64;
    const int64_t rbase = is_b ? P.rB : P.rA;
    const int64_t ebase = is_b ? P.eB : P.eA;
    const int c = (int)(k0 / chunk);
    const int64_t tile_row0 = (is_b ? P.tB : P.tA) * rows_per_tile + lt * rows_per_tile;
    {
      const int64_t r0 = ri * rows_per_tile;
      const int h0 = 0;
      for (int i = threadIdx.x; i < rows_per_tile * 8; i += 256) {
        // 8 threads along one row: their slice stores form one contiguous 128-byte row; loads
        // are 64 contiguous bytes per thread (K-contiguous) or 4 rows x 32 bytes per column
        // across the warp (row-contiguous), full sectors either way
        const int g8 = i & 7, rr = i >> 3;
        const int64_t r = r0 + rr;
        double xv[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int64_t k = k0 + g8 * 8 + j;
          xv[j] = (r < rows && k < P.K) ? __ldg(X + off + r * rs + k * ks) : 0.0;
        }
        int e = 0, Rr = 0;
        if (r < rows) {
          e = use_r ? R[rbase + r] : E[ebase + r * P.nch + c];
          Rr = R[rbase + r];
          if (Rr == kNoExponent) Rr = e;  // the whole row is zero: every slice is zero
        }
        // per-row slice scales 2^(e - R - beta (q+1)) (0 below the float range: negligible)
        float scale[S];
#pragma unroll
        for (int q = 0; q < S; ++q) {
          const int k = e - Rr - kBeta * (q + 1);
          scale[q] = k >= -126 ? __uint_as_float((uint32_t)(k + 127) << 23) : 0.f;
        }
        // F = round(x * 2^(beta S - e)) needs at most beta*S + 1 bits. Up to 4 slices (<= 29
        // bits) that is 32-bit integer work on the top 32 bits of the significand (hi word 20
        // bits, lo word 11, implicit 1); with more slices, 64-bit work on all 53 bits.
        constexpr bool kWide = kBeta * S + 1 > 31;
        using IntF = typename std::conditional<kWide, long long, int>::type;
        const int sbase = 1054 + e - kBeta * S;  // F = m32 >> (sbase - eb), rounded
        uint32_t packed[S][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const double x = xv[j];
          const int hw = __double2hiint(x);
          const uint32_t lw = (uint32_t)__double2loint(x);
          const int eb = (hw >> 20) & 0x7ff;
          IntF F = 0;
          if constexpr (!kWide) {
            const uint32_t m32 = (((uint32_t)hw << 11) | (lw >> 21)) | 0x80000000u;
            const int s = sbase - eb;  // >= 32 - beta*S > 0 for every element of the row chunk
            if (eb != 0 && eb != 0x7ff && s <= 32 && r < rows) {
              F = (int)(((m32 >> (s - 1)) + 1u) >> 1);  // round half up
              if (hw < 0) F = -F;
            }
          } else {
            const uint64_t m53 = ((uint64_t)(((uint32_t)hw & 0xfffffu) | 0x100000u) << 32) | lw;
            const int s = sbase + 21 - eb;  // >= 53 - beta*S >= 4 for up to 7 slices
            if (eb != 0 && eb != 0x7ff && s <= 54 && r < rows) {
              F = (long long)(((m53 >> (s - 1)) + 1ull) >> 1);  // round half up
              if (hw < 0) F = -F;
            }
          }
          const bool nonfinite = eb == 0x7ff && r < rows;  // propagates as NaN through the MMA
#pragma unroll
          for (int q = 0; q < S; ++q) {
            const int shq = kBeta * (S - 1 - q);
            int tq = (int)F;
            if (shq > 0) {
              const IntF t = (F + ((IntF)1 << (shq - 1))) >> shq;
              F -= t * ((IntF)1 << shq);
              tq = (int)t;
            }
            const float v = (float)tq * scale[q];  // exact: |tq| <= 2^beta
            const uint16_t h =
                nonfinite ? (uint16_t)0x7fc0u : __bfloat16_as_ushort(__float2bfloat16_rn(v));
            if (j & 1) packed[q][j >> 1] |= (uint32_t)h << 16;
            else packed[q][j >> 1] = (uint32_t)h;
          }
        }
#pragma unroll
        for (int q = 0; q < S; ++q) {
          uint4 w = make_uint4(packed[q][0], packed[q][1], packed[q][2], packed[q][3]);
          const int64_t idx = ((int64_t)q * rows_total + tile_row0 + h0 + rr) * 64 + g8 * 8;
          *reinterpret_cast<uint4*>(out + idx) = w;
        }
      }
    }
  }
}

// ------------------------------------------------------------------------------------------
// the GEMM kernel
// ------------------------------------------------------------------------------------------
// K-major tile with 64-byte swizzle (rows of 32 bf16), 8-row groups 512 B apart
__device__ __forceinline__ uint64_t sw64_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                    // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;           // stride byte offset: 8 rows x 64 B
  d |= (uint64_t)1 << 46;                    // descriptor version
  d |= (uint64_t)4 << 61;                    // 64-byte swizzle
  return d;
}

// Exact mode. The K step is 64 (128-byte swizzle) up to 3 slices; with 4..7 slices it is 32
// (64-byte swizzle) so that a pipeline stage holding all S slices of both operands fits 2 to 4
// times in shared memory. A chunk (the K range between exact FP32 flushes, exact_chunk) is a
// multiple of 64. BN (the N tile) is exact_bn(S) or 64.
template <int S, int BN = exact_bn(S)>
struct Cfg {
  static constexpr int kBK = S <= 3 ? 64 : 32;
  static constexpr int kPerRow = 64 / kBK;  // K steps per 64-wide packed row
  static constexpr int kPairs = S * (S + 1) / 2;
  static constexpr int kChunk = exact_chunk(S);
  static constexpr int kChunkSteps = kChunk / kBK;
  static constexpr int kBN = BN;
  static constexpr int kABytes = BM * kBK * 2;
  static constexpr int kBBytes = kBN * kBK * 2;
  static constexpr int kStageBytes = S * (kABytes + kBBytes);
  static constexpr int kStages = (220 * 1024) / kStageBytes > 4 ? 4 : (220 * 1024) / kStageBytes;
  static constexpr int kAccs = exact_accs(S);
  static constexpr int kAccCols = kAccs * kBN;
  static constexpr int kBufs = (2 * kAccCols <= 512) ? 2 : 1;
  static constexpr int kTmemCols = (kBufs * kAccCols <= 128) ? 128
                                   : (kBufs * kAccCols <= 256) ? 256 : 512;
  static constexpr int kSmemBytes = kStages * kStageBytes + 1024 + 256;
  // epilogue: four warps per TMEM lane quarter, each draining a quarter of the tile's columns
  static constexpr int kEpiWarps = 16;
  static constexpr int kEpiCols = kBN * 4 / kEpiWarps;
  static constexpr int kThreads = 32 * (2 + kEpiWarps);
};
constexpr int kExactThreads = 576;  // Cfg<S, BN>::kThreads (launch bound of the exact kernel)

// Static schedule shared by the three roles: the host sorts output tiles by decreasing K and the
// CTAs deal them out in snake order (b, 2G-1-b, 2G+b, ...), which balances ragged sectors.
__device__ __forceinline__ int64_t sched_pos(int64_t i, int G, int b) {
  return i * G + ((i & 1) ? (G - 1 - b) : b);
}

// 18 warps put 5 warps on one SM sub-partition (16K registers), which caps a thread at 96
// registers; the epilogue drains TMEM in 16-column pieces to stay close to that
template <int S, int BN>
__global__ void __launch_bounds__(kExactThreads, 1) split_gemm_kernel(
    const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
    const Problem* __restrict__ probs, const int4* __restrict__ tiles, int64_t ntiles,
    const int32_t* __restrict__ RA, const int32_t* __restrict__ CB, double* __restrict__ C,
    int* __restrict__ err) {
  using CF = Cfg<S, BN>;
  static_assert(CF::kThreads == kExactThreads, "launch bound and epilogue warp count disagree");
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = (uint64_t*)(smem + CF::kStages * CF::kStageBytes);
  uint64_t* full = bars;
  uint64_t* empty = bars + CF::kStages;
  uint64_t* tfull = bars + 2 * CF::kStages;
  uint64_t* tempty = tfull + 2;
  uint64_t* drain = tempty + 2;
  uint32_t* tmem_slot = (uint32_t*)(drain + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < CF::kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 32 * CF::kEpiWarps);
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == 1) tmem_alloc(tmem_slot, CF::kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      for (int64_t i = 0; !*abort_flag; ++i) {
        const int64_t pos = sched_pos(i, gridDim.x, blockIdx.x);
        if (pos >= ntiles) break;
        const int4 tr = tiles[pos];
        const int nks = probs[tr.x].nks;
        const int64_t baseA = (probs[tr.x].tA + (int64_t)tr.y * nks) * BM;
        const int64_t baseB = (probs[tr.x].tB + (int64_t)tr.z * nks) * CF::kBN;
        // K steps [kb, ke) of 64 columns (the whole K unless split-K halved this tile)
        const int kb = tr.w & 0xffff, ke = (int)((unsigned)tr.w >> 16);
        for (int ks = kb * CF::kPerRow; ks < ke * CF::kPerRow; ++ks) {
          if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag, err, 1)) break;
          uint8_t* sA = smem + stage * CF::kStageBytes;
          uint8_t* sB = sA + S * CF::kABytes;
          mbar_expect_tx(&full[stage], CF::kStageBytes);
          const int x = (ks % CF::kPerRow) * CF::kBK;
          const int rowA = (int)(baseA + (int64_t)(ks / CF::kPerRow) * BM);
          const int rowB = (int)(baseB + (int64_t)(ks / CF::kPerRow) * CF::kBN);
#pragma unroll
          for (int s = 0; s < S; ++s) tma_load_3d(sA + s * CF::kABytes, &tmA, &full[stage], x, rowA, s);
#pragma unroll
          for (int s = 0; s < S; ++s) tma_load_3d(sB + s * CF::kBBytes, &tmB, &full[stage], x, rowB, s);
          if (++stage == CF::kStages) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      constexpr uint32_t idesc = make_idesc(BM, CF::kBN);
      int stage = 0;
      uint32_t phase = 0;
      int64_t use = 0;
      bool issued = false;
      for (int64_t i = 0; !*abort_flag; ++i) {
        const int64_t pos = sched_pos(i, gridDim.x, blockIdx.x);
        if (pos >= ntiles) break;
        const int tw = tiles[pos].w;
        const int nsteps = (int)((unsigned)tw >> 16) * CF::kPerRow;
        for (int c0 = (tw & 0xffff) * CF::kPerRow; c0 < nsteps && !*abort_flag;
             c0 += CF::kChunkSteps) {
          const int buf = (int)(use % CF::kBufs);
          const uint32_t bph = (uint32_t)((use / CF::kBufs) & 1);
          if (!mbar_wait(&tempty[buf], bph ^ 1, abort_flag, err, 2)) break;
          tc_fence_after();
          uint32_t init = 0;  // bit g: accumulator g already written in this chunk
          const int c1 = min(nsteps, c0 + CF::kChunkSteps);
          for (int ks = c0; ks < c1; ++ks) {
            if (!mbar_wait(&full[stage], phase, abort_flag, err, 3)) break;
            tc_fence_after();
            const uint32_t sA = smem_u32(smem + stage * CF::kStageBytes);
            const uint32_t sB = sA + S * CF::kABytes;
#pragma unroll
            for (int pa = 0; pa < S; ++pa) {
#pragma unroll
              for (int qb = 0; qb < S - pa; ++qb) {
                const int g = pa + qb < CF::kAccs ? pa + qb : CF::kAccs - 1;  // accumulator
                const uint32_t dcol = tmem_base + (uint32_t)((buf * CF::kAccs + g) * CF::kBN);
                const uint64_t ad = CF::kBK == 64 ? sw128_desc(sA + pa * CF::kABytes)
                                                  : sw64_desc(sA + pa * CF::kABytes);
                const uint64_t bd = CF::kBK == 64 ? sw128_desc(sB + qb * CF::kBBytes)
                                                  : sw64_desc(sB + qb * CF::kBBytes);
#pragma unroll
                for (int kk = 0; kk < CF::kBK / 16; ++kk) {
                  umma_bf16(dcol, ad + 2 * kk, bd + 2 * kk, idesc, (init >> g) & 1u);
                  init |= 1u << g;
                }
              }
            }
            umma_commit(&empty[stage]);
            issued = true;
            if (++stage == CF::kStages) {
              stage = 0;
              phase ^= 1;
            }
          }
          umma_commit(&tfull[buf]);
          ++use;
        }
      }
      if (issued) {  // make sure every MMA has retired before TMEM is released
        umma_commit(drain);
        volatile int no_abort = 0;
        mbar_wait(drain, 0, &no_abort, err, 4);
      }
    }
  } else {
    // ---------------- epilogue: warps 2..(2 + kEpiWarps - 1) ----------------
    // warp w reads TMEM lanes 32 (w % 4) .. + 31 (its lane quarter = 32 tile rows); the warps
    // of one quarter split the tile's columns
    constexpr int NC = CF::kEpiCols;
    const int lrow = 32 * (warp & 3) + lane;
    const int col0 = ((warp - 2) >> 2) * NC;
    const uint32_t lane_addr = (uint32_t)(32 * (warp & 3)) << 16;
    int64_t use = 0;
    for (int64_t i = 0;; ++i) {
      const int64_t pos = sched_pos(i, gridDim.x, blockIdx.x);
      if (pos >= ntiles) break;
      const int4 tr = tiles[pos];
      const Problem P = probs[tr.x];
      const int64_t mi = tr.y, ni = tr.z;
      float hi[NC], lo[NC];
#pragma unroll
      for (int j = 0; j < NC; ++j) {
        hi[j] = 0.f;
        lo[j] = 0.f;
      }
      bool ok = true;
      const int kb = tr.w & 0xffff, ke = (int)((unsigned)tr.w >> 16);
      const bool part = kb != 0 || ke != P.nks;  // one of two split-K halves
      for (int c0 = kb * CF::kPerRow; c0 < ke * CF::kPerRow; c0 += CF::kChunkSteps) {
        const int buf = (int)(use % CF::kBufs);
        const uint32_t bph = (uint32_t)((use / CF::kBufs) & 1);
        if (!mbar_wait(&tfull[buf], bph, abort_flag, err, 5)) {
          ok = false;
          break;
        }
        tc_fence_after();
        static_assert(NC % 16 == 0, "epilogue column groups are multiples of 16");
#pragma unroll
        for (int h = 0; h < NC / 16; ++h) {  // 16-column pieces keep few registers live
#pragma unroll
          for (int g = 0; g < CF::kAccs; ++g) {
            uint32_t v[16];
            tmem_ld16(tmem_base + lane_addr +
                          (uint32_t)((buf * CF::kAccs + g) * CF::kBN + col0 + h * 16),
                      v);
#pragma unroll
            for (int j = 0; j < 16; ++j) two_sum_acc(hi[h * 16 + j], lo[h * 16 + j], __uint_as_float(v[j]));
          }
        }
        tc_fence_before();
        mbar_arrive(&tempty[buf]);
        ++use;
      }
      if (!ok) break;
      const int64_t row = mi * BM + lrow;
      if (row < P.M) {
        const int Rr = RA[P.rA + row];
        double* Cp = C + P.offC + row;
#pragma unroll
        for (int j = 0; j < NC; ++j) {
          const int64_t col = ni * CF::kBN + col0 + j;
          if (col < P.N) {
            const int Cc = CB[P.rB + col];
            // a zero row or column (no exponent) contributes exact zeros
            const int E = (Rr == kNoExponent || Cc == kNoExponent) ? 0 : Rr + Cc;
            if (part)  // zeroed output, exactly two partial sums: order-independent
              atomicAdd(Cp + col * P.ldc, ds_to_f64(hi[j], lo[j], E));
            else
              Cp[col * P.ldc] = ds_to_f64(hi[j], lo[j], E);
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem_base, CF::kTmemCols);
  }
}

// ------------------------------------------------------------------------------------------
// fast mode (S <= 3): one FP32 accumulator, per-row scale over the whole K, 128 x 256 tiles
// ------------------------------------------------------------------------------------------
// Every slice already carries its true scale 2^(e(i) - R(i) - beta(p+1)), so the products of
// all pairs (p, q) with p + q < S can share one FP32 accumulator: FP32 rounding (2^-24) stays
// below the 2^(-7 S) slicing error for S <= 3.  Without chunk flushes the epilogue is one TMEM
// read, one exponent shift and one FP64 store per element, which lets the tile grow to
// 128 x 256 (double-buffered: 2 x 256 TMEM columns) and the K step shrink to 32 (64-byte
// swizzle), doubling the MMA work per byte staged in shared memory.
constexpr int BNF = 256, BKF = 32;

// v * 2^E as FP64 from the FP32 bit pattern (integer instructions only)
__device__ __forceinline__ double f32_to_f64_scaled(float v, int E) {
  const uint32_t u = __float_as_uint(v);
  const int ef = (int)((u >> 23) & 0xff);
  if (ef == 0) return 0.0;  // zero (FP32 denormals are far below the accuracy of this path)
  if (ef == 0xff) return (double)v;  // NaN / Inf stay non-finite
  const long long be = (long long)ef - 127 + 1023 + E;
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  if (be <= 0) return 0.0;
  if (be >= 2047) return __longlong_as_double((long long)(sign | (0x7ffull << 52)));
  return __longlong_as_double(
      (long long)(sign | ((unsigned long long)be << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
}

template <int S>
struct FastCfg {
  static constexpr int kABytes = BM * BKF * 2;   // 8 KB
  static constexpr int kBBytes = BNF * BKF * 2;  // 16 KB
  static constexpr int kStageBytes = S * (kABytes + kBBytes);
  static constexpr int kStages = (220 * 1024) / kStageBytes > 6 ? 6 : (220 * 1024) / kStageBytes;
  static constexpr int kTmemCols = 2 * BNF;
  static constexpr int kSmemBytes = kStages * kStageBytes + 1024 + 256;
};

template <int S>
__global__ void __launch_bounds__(192, 1) split_gemm_fast_kernel(
    const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
    const Problem* __restrict__ probs, const int4* __restrict__ tiles, int64_t ntiles,
    const int32_t* __restrict__ RA, const int32_t* __restrict__ CB, double* __restrict__ C,
    int* __restrict__ err) {
  using CF = FastCfg<S>;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = (uint64_t*)(smem + CF::kStages * CF::kStageBytes);
  uint64_t* full = bars;
  uint64_t* empty = bars + CF::kStages;
  uint64_t* tfull = bars + 2 * CF::kStages;
  uint64_t* tempty = tfull + 2;
  uint64_t* drain = tempty + 2;
  uint32_t* tmem_slot = (uint32_t*)(drain + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < CF::kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 128);
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == 1) tmem_alloc(tmem_slot, CF::kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      for (int64_t i = 0; !*abort_flag; ++i) {
        const int64_t pos = sched_pos(i, gridDim.x, blockIdx.x);
        if (pos >= ntiles) break;
        const int4 tr = tiles[pos];
        const int nks = probs[tr.x].nks;
        const int64_t baseA = (probs[tr.x].tA + (int64_t)tr.y * nks) * BM;
        const int64_t baseB = (probs[tr.x].tB + (int64_t)tr.z * nks) * BNF;
        for (int kb = 0; kb < 2 * nks; ++kb) {
          if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag, err, 1)) break;
          uint8_t* sA = smem + stage * CF::kStageBytes;
          uint8_t* sB = sA + S * CF::kABytes;
          mbar_expect_tx(&full[stage], CF::kStageBytes);
          const int x = (kb & 1) * BKF;
          const int rowA = (int)(baseA + (int64_t)(kb >> 1) * BM);
          const int rowB = (int)(baseB + (int64_t)(kb >> 1) * BNF);
#pragma unroll
          for (int s = 0; s < S; ++s) tma_load_3d(sA + s * CF::kABytes, &tmA, &full[stage], x, rowA, s);
#pragma unroll
          for (int s = 0; s < S; ++s) tma_load_3d(sB + s * CF::kBBytes, &tmB, &full[stage], x, rowB, s);
          if (++stage == CF::kStages) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      constexpr uint32_t idesc = make_idesc(BM, BNF);
      int stage = 0;
      uint32_t phase = 0;
      int64_t use = 0;
      bool issued = false;
      for (int64_t i = 0; !*abort_flag; ++i) {
        const int64_t pos = sched_pos(i, gridDim.x, blockIdx.x);
        if (pos >= ntiles) break;
        const int nks = probs[tiles[pos].x].nks;
        if (nks == 0) continue;
        const int buf = (int)(use & 1);
        const uint32_t bph = (uint32_t)((use >> 1) & 1);
        if (!mbar_wait(&tempty[buf], bph ^ 1, abort_flag, err, 2)) break;
        tc_fence_after();
        const uint32_t dcol = tmem_base + (uint32_t)(buf * BNF);
        uint32_t acc = 0;
        for (int kb = 0; kb < 2 * nks; ++kb) {
          if (!mbar_wait(&full[stage], phase, abort_flag, err, 3)) break;
          tc_fence_after();
          const uint32_t sA = smem_u32(smem + stage * CF::kStageBytes);
          const uint32_t sB = sA + S * CF::kABytes;
#pragma unroll
          for (int pa = 0; pa < S; ++pa) {
#pragma unroll
            for (int qb = 0; qb < S - pa; ++qb) {
              const uint64_t ad = sw64_desc(sA + pa * CF::kABytes);
              const uint64_t bd = sw64_desc(sB + qb * CF::kBBytes);
#pragma unroll
              for (int kk = 0; kk < BKF / 16; ++kk) {
                umma_bf16(dcol, ad + 2 * kk, bd + 2 * kk, idesc, acc);
                acc = 1;
              }
            }
          }
          umma_commit(&empty[stage]);
          issued = true;
          if (++stage == CF::kStages) {
            stage = 0;
            phase ^= 1;
          }
        }
        umma_commit(&tfull[buf]);
        ++use;
      }
      if (issued) {
        umma_commit(drain);
        volatile int no_abort = 0;
        mbar_wait(drain, 0, &no_abort, err, 4);
      }
    }
  } else {
    // ---------------- epilogue: warps 2..5, one TMEM lane (= output row) per thread --------
    const int lrow = 32 * (warp & 3) + lane;
    const uint32_t lane_addr = (uint32_t)(32 * (warp & 3)) << 16;
    int64_t use = 0;
    for (int64_t i = 0;; ++i) {
      const int64_t pos = sched_pos(i, gridDim.x, blockIdx.x);
      if (pos >= ntiles) break;
      const int4 tr = tiles[pos];
      const Problem P = probs[tr.x];
      const int64_t row = (int64_t)tr.y * BM + lrow;
      const int64_t col0 = (int64_t)tr.z * BNF;
      double* Cp = C + P.offC + row;
      if (P.nks == 0) {  // allowed sector without partner blocks: zeros
        if (row < P.M)
          for (int j = 0; j < BNF && col0 + j < P.N; ++j) Cp[(col0 + j) * P.ldc] = 0.0;
        continue;
      }
      const int buf = (int)(use & 1);
      const uint32_t bph = (uint32_t)((use >> 1) & 1);
      if (!mbar_wait(&tfull[buf], bph, abort_flag, err, 5)) break;
      tc_fence_after();
      const int Rr = row < P.M ? RA[P.rA + row] : 0;
#pragma unroll 1
      for (int h = 0; h < BNF / 32; ++h) {
        uint32_t v[32];
        tmem_ld32(tmem_base + lane_addr + (uint32_t)(buf * BNF + h * 32), v);
        if (row < P.M) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int64_t col = col0 + h * 32 + j;
            if (col < P.N) {
              const int Cc = CB[P.rB + col];
              const int E = (Rr == kNoExponent || Cc == kNoExponent) ? 0 : Rr + Cc;
              Cp[col * P.ldc] = f32_to_f64_scaled(__uint_as_float(v[j]), E);
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&tempty[buf]);
      ++use;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem_base, CF::kTmemCols);
  }
}

// ------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    MPSG_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                               cudaEnableDefault, &q));
    if (!p || q != cudaDriverEntryPointSuccess)
      throw Error(kErrCuda, "cuTensorMapEncodeTiled is not available");
    fn = (EncodeTiledFn)p;
  }
  return fn;
}

// Packed operand [S][rows_total][64] bf16; box = box_x K-columns x box_rows rows of one slice.
static void make_map(CUtensorMap* map, void* base, int64_t rows_total, int S, int box_rows,
                     int box_x) {
  cuuint64_t gdim[3] = {64, (cuuint64_t)rows_total, (cuuint64_t)S};
  cuuint64_t gstride[2] = {128, (cuuint64_t)rows_total * 128};
  cuuint32_t box[3] = {(cuuint32_t)box_x, (cuuint32_t)box_rows, 1};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = encode_fn()(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, gdim, gstride, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE,
                           box_x == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(kErrCuda, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

int chunk_for(int S) { return exact_chunk(S); }

}  // namespace split

size_t DevGemmPlan::device_bytes() const {
  size_t b = 0;
  for (const auto& sp : splitp)
    if (sp) b += (size_t)sp->S * (size_t)(sp->rowsA + sp->rowsB) * 128;
  return b;
}

namespace split {

void SplitPlan::build(Context* ctx, const std::vector<GemmTask>& g, int S_, Tuning tune) {
  release();
  S = S_;
  if (S < 2 || S > kMaxSlices)
    throw Error(kErrUnsupported, "split precision supports 2..7 slices");
  const char* ex = std::getenv("MPSG_SPLIT_EXACT");
  fast = S <= 3 && !(ex && ex[0] == '1');
  if (tune.bn != 0 && tune.bn != 64 && tune.bn != exact_bn(S))
    throw Error(kErrArgument, "split GEMM N tile must be 64 or " + std::to_string(exact_bn(S)));
  if (tune.order != kOrderK && tune.order != kOrderProblem)
    throw Error(kErrArgument, "unknown split GEMM tile order");
  bn = fast ? BNF : (tune.bn ? tune.bn : exact_bn(S));
  order = tune.order;
  chunk = fast ? (1 << 30) : chunk_for(S);
  seg = fast ? 256 : chunk;
  probs.clear();
  int64_t tA = 0, tB = 0, rA = 0, rB = 0, eA = 0, eB = 0;
  std::vector<int64_t> tile_prefix(1, 0), packA_prefix(1, 0), packB_prefix(1, 0),
      rowA_prefix(1, 0), rowB_prefix(1, 0);
  flops = 0;
  for (const GemmTask& t : g) {
    Problem P;
    P.M = t.M;
    P.N = t.N;
    P.K = t.K;
    P.offA = t.offA;
    P.offB = t.offB;
    P.offC = t.offC;
    P.lda = t.lda;
    P.ldb = t.ldb;
    P.ldc = t.ldc;
    P.mt = (int)((t.M + BM - 1) / BM);
    P.nt = (int)((t.N + bn - 1) / bn);
    P.nks = (int)((t.K + BK - 1) / BK);
    P.nch = (int)(((int64_t)t.K + chunk - 1) / chunk);
    P.tA = tA;
    P.tB = tB;
    P.rA = rA;
    P.rB = rB;
    P.eA = eA;
    P.eB = eB;
    tA += (int64_t)P.mt * P.nks;
    tB += (int64_t)P.nt * P.nks;
    rA += (int64_t)P.mt * BM;
    rB += (int64_t)P.nt * bn;
    eA += (int64_t)P.mt * BM * std::max(P.nch, 1);
    eB += (int64_t)P.nt * bn * std::max(P.nch, 1);
    tile_prefix.push_back(tile_prefix.back() + (int64_t)P.mt * P.nt);
    packA_prefix.push_back(packA_prefix.back() + (int64_t)P.mt * P.nks);
    packB_prefix.push_back(packB_prefix.back() + (int64_t)P.nt * P.nks);
    // exponent work items: (32-row block, K chunk) pairs
    // (in fast mode the K range is only split for parallelism: segments of `seg` columns)
    const int64_t nseg = fast ? ((int64_t)t.K + seg - 1) / seg : P.nch;
    rowA_prefix.push_back(rowA_prefix.back() +
                          (P.nks ? ((P.M + kExpRowsA - 1) / kExpRowsA) * nseg : 0));
    rowB_prefix.push_back(rowB_prefix.back() +
                          (P.nks ? ((P.N + kExpRowsB - 1) / kExpRowsB) * nseg : 0));
    flops += 2.0 * t.M * t.N * t.K;
    probs.push_back(P);
  }
  nprob = (int)probs.size();
  ntiles = tile_prefix.back();
  // output tiles problem by problem (N tile, then M tile), for the snake schedule by decreasing
  // K (ties keep that order) unless the tuning asks for the problem order
  // w = K steps [kb, ke) of the tile: kb | ke << 16 (split-K halves cover part of K)
  std::vector<int4> tl;
  tl.reserve(ntiles);
  for (int p = 0; p < nprob; ++p) {
    if (probs[p].nks > 0x7fff) throw Error(kErrUnsupported, "split GEMM: K too long");
    for (int ni = 0; ni < probs[p].nt; ++ni)
      for (int mi = 0; mi < probs[p].mt; ++mi)
        tl.push_back(make_int4(p, mi, ni, probs[p].nks << 16));
  }
  auto work = [](const int4& t) { return (int)((unsigned)t.w >> 16) - (t.w & 0xffff); };
  std::vector<char> zero_prob(nprob, 0);
  nsplit = (tune.splitk && !fast)
               ? split_k_tiles(tl, probs, chunk / 64, 2 * (int64_t)ctx->num_sms, zero_prob)
               : 0;
  ntiles = (int64_t)tl.size();
  if (order == kOrderK)
    std::stable_sort(tl.begin(), tl.end(),
                     [&](const int4& a, const int4& b) { return work(a) > work(b); });
  tilesA = tA;
  tilesB = tB;
  rowsA = tA * BM;
  rowsB = tB * bn;
  nrowsA = rowA_prefix.back();
  nrowsB = rowB_prefix.back();
  rowsRA = std::max<int64_t>(rA, 1);
  rowsCB = std::max<int64_t>(rB, 1);
  if (nprob == 0) return;
  // stream-ordered allocation on the context's stream: no device-wide synchronisation, so
  // contexts sharing the GPU do not serialise on plan builds (pageable sources are staged
  // before the copy calls return)
  cudaStream_t st = ctx->stream;
  stream = st;
  auto alloc = [st](void** d, size_t bytes) {
    MPSG_CUDA(cudaMallocAsync(d, std::max<size_t>(bytes, 16), st));
  };
  auto up = [&](void** d, const void* h, size_t bytes) {
    alloc(d, bytes);
    if (bytes) MPSG_CUDA(cudaMemcpyAsync(*d, h, bytes, cudaMemcpyHostToDevice, st));
  };
  auto zero = [st](void* d, size_t bytes) { MPSG_CUDA(cudaMemsetAsync(d, 0, bytes, st)); };
  up((void**)&d_probs, probs.data(), sizeof(Problem) * nprob);
  up((void**)&d_tile_prefix, tile_prefix.data(), sizeof(int64_t) * (nprob + 1));
  up((void**)&d_tiles, tl.data(), sizeof(int4) * tl.size());
  std::vector<int> zl;
  for (int p = 0; p < nprob; ++p)
    if (zero_prob[p]) zl.push_back(p);
  nzero = (int)zl.size();
  if (nzero) up((void**)&d_zero, zl.data(), sizeof(int) * zl.size());
  up((void**)&d_packA_prefix, packA_prefix.data(), sizeof(int64_t) * (nprob + 1));
  up((void**)&d_packB_prefix, packB_prefix.data(), sizeof(int64_t) * (nprob + 1));
  up((void**)&d_rowA_prefix, rowA_prefix.data(), sizeof(int64_t) * (nprob + 1));
  up((void**)&d_rowB_prefix, rowB_prefix.data(), sizeof(int64_t) * (nprob + 1));
  alloc((void**)&d_RA, sizeof(int32_t) * std::max<int64_t>(rA, 1));
  alloc((void**)&d_CB, sizeof(int32_t) * std::max<int64_t>(rB, 1));
  zero(d_RA, sizeof(int32_t) * std::max<int64_t>(rA, 1));
  zero(d_CB, sizeof(int32_t) * std::max<int64_t>(rB, 1));
  alloc((void**)&d_EA, sizeof(int16_t) * std::max<int64_t>(eA, 1));
  alloc((void**)&d_EB, sizeof(int16_t) * std::max<int64_t>(eB, 1));
  zero(d_EA, sizeof(int16_t) * std::max<int64_t>(eA, 1));
  zero(d_EB, sizeof(int16_t) * std::max<int64_t>(eB, 1));
  alloc((void**)&d_packA, std::max<int64_t>(S * rowsA * 64 * 2, 128 * 128));
  alloc((void**)&d_packB, std::max<int64_t>(S * rowsB * 64 * 2, 128 * 128));
  alloc((void**)&d_err, sizeof(int));
  zero(d_err, sizeof(int));
  const int box_x = (fast || S > 3) ? 32 : BK;  // K step of the kernel that reads the slices
  make_map(&tmA, d_packA, std::max<int64_t>(rowsA, BM), S, BM, box_x);
  make_map(&tmB, d_packB, std::max<int64_t>(rowsB, bn), S, bn, box_x);
}

void SplitPlan::release() {
  void* ptrs[] = {d_probs, d_tile_prefix, d_packA_prefix, d_packB_prefix, d_rowA_prefix,
                  d_rowB_prefix, d_RA, d_CB, d_EA, d_EB, d_packA, d_packB, d_err, d_tiles,
                  d_zero};
  for (void* p : ptrs)
    if (p) cudaFreeAsync(p, stream);
  d_probs = nullptr;
  d_tiles = nullptr;
  d_tile_prefix = d_packA_prefix = d_packB_prefix = d_rowA_prefix = d_rowB_prefix = nullptr;
  d_RA = d_CB = nullptr;
  d_EA = d_EB = nullptr;
  d_packA = d_packB = nullptr;
  d_err = nullptr;
  d_zero = nullptr;
  nzero = 0;
  nsplit = 0;
  nprob = 0;
}

// Zeroes the output blocks of the problems listed in `list` (those with split-K tiles, whose
// halves add into the output); blockIdx.y selects the problem, blockIdx.x strides over it.
__global__ void zero_outputs_kernel(const Problem* __restrict__ probs, const int* __restrict__ list,
                                    double* __restrict__ C) {
  const Problem P = probs[list[blockIdx.y]];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < P.M * P.N;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / P.M, i = e - j * P.M;
    C[P.offC + i + j * P.ldc] = 0.0;
  }
}

// The exact kernel at N tile BN (the fast kernel when the plan is in fast mode).
template <int S, int BN>
static void launch_gemm_t(Context* ctx, SplitPlan& sp, double* C) {
  using CF = Cfg<S, BN>;
  using FCF = FastCfg<S <= 3 ? S : 3>;
  // per device, slice count and N tile (one flag array per instantiation of this launcher)
  static std::once_flag exact_set[kMaxDevices], fast_set[kMaxDevices];
  if (sp.fast)
    set_smem_limit_once(ctx, fast_set, split_gemm_fast_kernel<S <= 3 ? S : 3>,
                        (int)FCF::kSmemBytes);
  else
    set_smem_limit_once(ctx, exact_set, split_gemm_kernel<S, BN>, (int)CF::kSmemBytes);
  const int grid = (int)std::min<int64_t>(sp.ntiles, (int64_t)ctx->num_sms);
  if (sp.nzero) {
    zero_outputs_kernel<<<dim3(64, (unsigned)sp.nzero), 256, 0, ctx->stream>>>(sp.d_probs,
                                                                              sp.d_zero, C);
    MPSG_CUDA(cudaGetLastError());
    ctx->kernel_launches++;
  }
  KernelTimer timer(ctx, kKindGemmSplit, sp.flops);
  if (sp.fast) {
    if (S > 3) throw Error(kErrUnsupported, "fast split mode needs S <= 3");
    split_gemm_fast_kernel<S <= 3 ? S : 3><<<grid, 192, FCF::kSmemBytes, ctx->stream>>>(
        sp.tmA, sp.tmB, sp.d_probs, sp.d_tiles, sp.ntiles, sp.d_RA, sp.d_CB, C, sp.d_err);
  } else {
    split_gemm_kernel<S, BN><<<grid, CF::kThreads, CF::kSmemBytes, ctx->stream>>>(
        sp.tmA, sp.tmB, sp.d_probs, sp.d_tiles, sp.ntiles, sp.d_RA, sp.d_CB, C, sp.d_err);
  }
  MPSG_CUDA(cudaGetLastError());
}

template <int S>
static void launch_t(Context* ctx, SplitPlan& sp, const double* A, const double* B, double* C,
                     int what) {
  const int chunk = sp.chunk;
  for (int side = 0; side < 2; ++side) {
    if (!(what & (side ? kPackB : kPackA))) continue;
    const int64_t nitems = side ? sp.nrowsB : sp.nrowsA;
    const int64_t ntile = side ? sp.tilesB : sp.tilesA;
    const double* X = side ? B : A;
    int16_t* E = side ? sp.d_EB : sp.d_EA;
    int32_t* R = side ? sp.d_CB : sp.d_RA;
    if (nitems) {
      MPSG_CUDA(cudaMemsetAsync(R, 0x80, sizeof(int32_t) * (side ? sp.rowsCB : sp.rowsRA),
                                ctx->stream));
      KernelTimer timer(ctx, kKindPack);
      int g = (int)std::min<int64_t>(nitems, (int64_t)ctx->num_sms * 8);
      pack_exponents_kernel<<<g, 256, 0, ctx->stream>>>(
          sp.d_probs, side ? sp.d_rowB_prefix : sp.d_rowA_prefix, sp.nprob, nitems, side, sp.seg,
          sp.fast ? 0 : 1,
          X, E, R);
      MPSG_CUDA(cudaGetLastError());
      ctx->kernel_launches++;
    }
    if (ntile) {
      KernelTimer timer(ctx, kKindPackSlices);
      int g = (int)std::min<int64_t>(ntile, (int64_t)ctx->num_sms * 8);
      pack_slices_kernel<S><<<g, 256, 0, ctx->stream>>>(
          sp.d_probs, side ? sp.d_packB_prefix : sp.d_packA_prefix, sp.nprob, ntile, side, chunk,
          sp.fast ? 1 : 0,
          side ? sp.bn : BM, side ? sp.rowsB : sp.rowsA, X, E, R,
          (__nv_bfloat16*)(side ? sp.d_packB : sp.d_packA));
      MPSG_CUDA(cudaGetLastError());
      ctx->kernel_launches++;
    }
  }
  if (!(what & kRunGemm)) return;
  if (!sp.fast && sp.bn == 64 && exact_bn(S) != 64)
    launch_gemm_t<S, 64>(ctx, sp, C);
  else
    launch_gemm_t<S, exact_bn(S)>(ctx, sp, C);
  ctx->kernel_launches++;
  ctx->gemm_flops += sp.flops;
  if (ctx->debug_sync) {
    MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
    const int e = read_error(ctx, sp);
    if (e) throw Error(kErrCuda, "split GEMM: a bounded wait expired (role code " + std::to_string(e) + ")");
  }
}

void launch_split_gemm(Context* ctx, SplitPlan& sp, const double* A, const double* B, double* C,
                       int what) {
  if (sp.ntiles == 0) return;
  switch (sp.S) {
    case 2: launch_t<2>(ctx, sp, A, B, C, what); break;
    case 3: launch_t<3>(ctx, sp, A, B, C, what); break;
    case 4: launch_t<4>(ctx, sp, A, B, C, what); break;
    case 5: launch_t<5>(ctx, sp, A, B, C, what); break;
    case 6: launch_t<6>(ctx, sp, A, B, C, what); break;
    case 7: launch_t<7>(ctx, sp, A, B, C, what); break;
    default: throw Error(kErrUnsupported, "split precision supports 2..7 slices");
  }
}

int read_error(Context* ctx, SplitPlan& sp) {
  int e = 0;
  if (!sp.d_err) return 0;
  MPSG_CUDA(cudaMemcpyAsync(&e, sp.d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MPSG_CUDA(cudaStreamSynchronize(ctx->stream));
  return e;
}

}  // namespace split
}  // namespace mpsg
