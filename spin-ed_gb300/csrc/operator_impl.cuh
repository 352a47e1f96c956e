// operator_impl.cuh — device-side pieces of the matvec shared by the
// operator and eigensolver translation units (see operator.cu for the
// mathematics of the pull form and the stream form).
#pragma once

#include <type_traits>

#include "sed_internal.hpp"
#include "util.cuh"

namespace sed {

constexpr uint32_t kNull = 0xFFFFFFFFu;
constexpr unsigned kMaxCodes = 65535;

struct StreamView {
  uint64_t const* slice_ptr;
  uint32_t const* entries;
  uint16_t const* codes;  // unpacked form only
  void const* diag;       // double[D] or double2[D]
  uint8_t const* row_class;
  void const* table;      // double or double2 [n_codes]
  double const* inv_sqrt_s;
  uint32_t col_bits;
  uint32_t n_codes;
};

struct CodeView {
  uint32_t const* divisors;  // ascending divisors of |G|
  uint32_t n_div;
  uint32_t n_ph;             // 2 (real: sign) or L
  uint32_t real_phase;       // 1 if phases are encoded as sign
};

__device__ __forceinline__ uint32_t divisor_class(uint32_t S, CodeView const& C) {
  uint32_t lo = 0, hi = C.n_div;
  while (lo < hi) {
    uint32_t const mid = (lo + hi) >> 1;
    if (C.divisors[mid] < S)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

__device__ __forceinline__ uint32_t element_code(uint32_t vid, uint32_t phase, uint32_t S_j,
                                                 CodeView const& C) {
  uint32_t const ph = C.real_phase ? (phase != 0u) : phase;
  return (vid * C.n_ph + ph) * C.n_div + divisor_class(S_j, C);
}

template <class V>
__device__ __forceinline__ V load_table(void const* t, uint32_t i, bool real_table);
template <>
__device__ __forceinline__ double load_table<double>(void const* t, uint32_t i, bool) {
  return static_cast<double const*>(t)[i];
}
template <>
__device__ __forceinline__ cplx load_table<cplx>(void const* t, uint32_t i, bool real_table) {
  if (real_table) return {static_cast<double const*>(t)[i], 0.0};
  double2 const v = static_cast<double2 const*>(t)[i];
  return {v.x, v.y};
}

template <class V>
__device__ __forceinline__ V row_value(V diag_x, double f, V acc) {
  return addv(diag_x, mulv(f, acc));
}

// Number of off-diagonal elements of row r.
__device__ __forceinline__ uint32_t row_count(uint64_t r, TermsView const& T) {
  uint32_t c = 0;
  for (uint32_t u = 0; u < T.n_tuples; ++u) {
    uint32_t const tk = T.tuple_term[u];
    uint32_t const t = tk & 0xFFFFu, k = tk >> 16;
    c += T.n_off[t * 16 + local_index(r, T.tuple_sites[u], k)];
  }
  return c;
}

// Walks the elements of row r in canonical order: f(e, s, vid).
template <class F>
__device__ __forceinline__ void walk_row(uint64_t r, TermsView const& T, F&& f) {
  uint32_t e = 0;
  for (uint32_t u = 0; u < T.n_tuples; ++u) {
    uint32_t const tk = T.tuple_term[u];
    uint32_t const t = tk & 0xFFFFu, k = tk >> 16;
    uint32_t const sites = T.tuple_sites[u];
    uint32_t const a = local_index(r, sites, k);
    uint32_t const n = T.n_off[t * 16 + a];
    for (uint32_t q = 0; q < n; ++q) {
      uint32_t const a2 = T.off_col[(t * 16 + a) * 16 + q];
      uint32_t const vid = T.off_vid[(t * 16 + a) * 16 + q];
      f(e++, replace_local(r, sites, k, a2), vid);
    }
  }
}

template <class V>
__device__ __forceinline__ V row_diag(uint64_t r, TermsView const& T);
template <>
__device__ __forceinline__ double row_diag<double>(uint64_t r, TermsView const& T) {
  double d = 0.0;
  for (uint32_t u = 0; u < T.n_tuples; ++u) {
    uint32_t const tk = T.tuple_term[u];
    uint32_t const t = tk & 0xFFFFu, k = tk >> 16;
    d = __dadd_rn(d, T.diag[2 * (t * 16 + local_index(r, T.tuple_sites[u], k))]);
  }
  return d;
}
template <>
__device__ __forceinline__ cplx row_diag<cplx>(uint64_t r, TermsView const& T) {
  cplx d{0.0, 0.0};
  for (uint32_t u = 0; u < T.n_tuples; ++u) {
    uint32_t const tk = T.tuple_term[u];
    uint32_t const t = tk & 0xFFFFu, k = tk >> 16;
    uint32_t const a = local_index(r, T.tuple_sites[u], k);
    d.re = __dadd_rn(d.re, T.diag[2 * (t * 16 + a)]);
    d.im = __dadd_rn(d.im, T.diag[2 * (t * 16 + a) + 1]);
  }
  return d;
}


// ------------------------------------------ exact fixed-point accumulation --
// For a real operator with real characters (chi = +-1) the off-diagonal part
// of row i is (1/sqrt(S_i)) sum_v c_v sum_{e: value v} chi_e sqrt(S_j) x_j.
// With u_j = round(sqrt(S_j) x_j 2^F) held as int64 (one pass over x before
// the matvec, F chosen per vector from max|x_j| so that no row sum can
// overflow), the inner sums are exact integer sums of +-u_j: one integer
// accumulator per distinct value c_v, converted and scaled by c_v 2^-F once
// per row. The only rounding before the row's FP64 epilogue is that of u_j
// (half an integer step, at most 2^-61 of the largest |u|), and integer sums
// do not depend on their order, so every form of the matvec agrees bit for
// bit. The integer pipe is 64x wider than GB300's FP64 pipe, which otherwise
// bounds the matvec at one FMA per element.
constexpr unsigned kFixMaxValues = 4;   // accumulators per row
constexpr unsigned kFixMaxClasses = 256;
constexpr int64_t kFixBad = INT64_MIN;  // x held a NaN or an infinity

struct FixView {
  uint8_t const* code;   // [n_codes]: value index << 1 | character sign
  double const* sqrt_s;  // [n_div]: sqrt(S) per stabiliser class
  uint32_t n_codes;
  uint32_t n_div;
  double bound;          // (largest row count) x sqrt(largest S), rounded up
  double sqrt_s_max;     // sqrt(largest S), rounded up
  double c[kFixMaxValues];
};

// Nearest integer of a finite d with |d| < 2^62 (halves away from zero),
// from the bit pattern: integer instructions only.
__device__ __forceinline__ int64_t fix_round(double d) {
  uint64_t const b = (uint64_t)__double_as_longlong(d);
  int const e = (int)((b >> 52) & 0x7FF);
  uint64_t const m = (b & 0xFFFFFFFFFFFFFull) | (e ? (1ull << 52) : 0ull);
  int const sh = 1075 - e;  // |d| = m 2^-sh for normal d
  uint64_t mag;
  if (sh <= 0)
    mag = m << (-sh);
  else if (sh >= 64)
    mag = 0;
  else
    mag = (m + (1ull << (sh - 1))) >> sh;
  return (b >> 63) ? -(int64_t)mag : (int64_t)mag;
}

// Scale exponent F for a vector whose largest |x_j| has bit pattern
// max_bits: bound * max|x| * 2^F < 2^62, so a row's sum of at most
// (row count) terms |u_j| <= sqrt(S_max) max|x| 2^F stays below 2^62.
__device__ __forceinline__ int64_t fix_exponent(uint64_t max_bits, double bound) {
  if (max_bits >= 0x7FF0000000000000ull) return kFixBad;
  if (max_bits == 0) return 0;
  double const t = __longlong_as_double((long long)max_bits) * bound;
  int const e = (int)(((uint64_t)__double_as_longlong(t) >> 52) & 0x7FF) - 1023;  // t < 2^(e+1)
  return 61 - e;  // in [-963, 1084]: t is finite, at least 2^-1074 before the bound
}

// The same for 32-bit u (the FP32-stored form): |u_j| < 2^30, sums in int64.
__device__ __forceinline__ int64_t fix_exponent32(uint64_t max_bits, double sqrt_s_max) {
  if (max_bits >= 0x7FF0000000000000ull) return kFixBad;
  if (max_bits == 0) return 0;
  double const t = __longlong_as_double((long long)max_bits) * sqrt_s_max;
  int const e = (int)(((uint64_t)__double_as_longlong(t) >> 52) & 0x7FF) - 1023;  // t < 2^(e+1)
  int64_t F = 29 - e;
  return F > 1000 ? 1000 : (F < -1000 ? -1000 : F);
}

// 2^p for |p| <= 1000 (a normal double), built from its bits.
__device__ __forceinline__ double fix_pow2(int64_t p) {
  return __longlong_as_double((long long)((uint64_t)(1023 + p) << 52));
}

// a 2^p for any exponent F can produce (|p| <= 1100): one multiplication
// when 2^p is a normal double, else two by halves of p (each exact unless
// the result is subnormal).
__device__ __forceinline__ double fix_ldexp(double a, int64_t p) {
  if (p >= -1000 && p <= 1000) return a * fix_pow2(p);
  int64_t const h = p / 2;
  return (a * fix_pow2(h)) * fix_pow2(p - h);
}

struct OperatorTables {
  DeviceBuffer divisors;
  DeviceBuffer table;    // double[n_codes], real operators only
  DeviceBuffer table_c;  // double2[n_codes], every operator
  DeviceBuffer inv_sqrt_s;
  CodeView code{};
  uint32_t n_codes = 0;
  // fixed-point form (fix_ok: the operator qualifies)
  bool fix_ok = false;
  uint32_t fix_nv = 1;   // accumulators per row: 1, 2 or 4
  DeviceBuffer fix_code;
  DeviceBuffer fix_sqrt_s;
  FixView fix{};
};

// One row of the streamed SpMV over a SELL-32 slice (lane = row in slice).
template <class V, class X, bool RealOp, bool Packed>
__device__ __forceinline__ V stream_row_acc(StreamView const& S, void const* table, uint64_t s,
                                            uint32_t lane, X const* __restrict__ x) {
  uint64_t const base = S.slice_ptr[s];
  uint32_t const width = (uint32_t)((S.slice_ptr[s + 1] - base) >> 5);
  uint32_t const col_mask = Packed ? ((1u << S.col_bits) - 1u) : 0xFFFFFFFFu;
  V acc = zero<V>();
  uint32_t const* ent = S.entries + base + lane;
  for (uint32_t e = 0; e < width; ++e) {
    uint32_t const v = __ldcs(ent + (uint64_t)e * 32);
    if (v != kNull) {
      uint32_t const col = v & col_mask;
      uint32_t const code =
          Packed ? (v >> S.col_bits) : (uint32_t)__ldcs(S.codes + base + lane + (uint64_t)e * 32);
      mac(acc, load_table<V>(table, code, RealOp), Store<X>::load(x, col));
    }
  }
  return acc;
}

template <class V, bool RealOp>
__device__ __forceinline__ V stream_diag(StreamView const& S, uint64_t i) {
  if constexpr (std::is_same<V, double>::value) {
    return static_cast<double const*>(S.diag)[i];
  } else {
    if (RealOp) return cplx{static_cast<double const*>(S.diag)[i], 0.0};
    double2 const d2 = static_cast<double2 const*>(S.diag)[i];
    return cplx{d2.x, d2.y};
  }
}

// Stages the value table in shared memory when it fits (32 KB); returns the
// table to read from. Must be called by every thread of the block.
template <bool RealOp>
__device__ __forceinline__ void const* stage_table(StreamView const& S, unsigned char* smem) {
  bool const in_smem = S.n_codes * (RealOp ? 8u : 16u) <= 32768u;
  if (in_smem) {
    if (RealOp) {
      double* t = reinterpret_cast<double*>(smem);
      for (uint32_t c = threadIdx.x; c < S.n_codes; c += blockDim.x)
        t[c] = static_cast<double const*>(S.table)[c];
    } else {
      double2* t = reinterpret_cast<double2*>(smem);
      for (uint32_t c = threadIdx.x; c < S.n_codes; c += blockDim.x)
        t[c] = static_cast<double2 const*>(S.table)[c];
    }
    __syncthreads();
    return smem;
  }
  return S.table;
}

StreamView stream_view(OperatorData const& op);

// The fixed-point workspace of an operator (column 0), for kernels that
// prepare u and F themselves.
struct FixSlots {
  unsigned long long* max_bits;  // max |x| bit pattern (zero before use)
  int64_t* F;
  int64_t* u;
  uint8_t const* row_class;
  FixView view;
};
// True (and *out filled) when the FP64 matvec of `op` runs in fixed point
// through the stream form.
bool fix_slots(OperatorData& op, FixSlots* out);
// The matvec's pre-pass on its own: max |x|, then u and F, for x = base (+ k
// ld in Krylov mode).
int fix_prescale(OperatorData& op, double const* base, Indirect ind, cudaStream_t stream);
// FP32 streamed SpMV in Krylov-indirect mode (x = base + k ld, y = base +
// (k+1) ld); FP32 arithmetic, per-block partial sums of x_i y_i in FP64.
int operator_apply_krylov32(OperatorData& op, float* base, Indirect ind, cudaStream_t stream,
                            unsigned* blocks);
// The same SpMV on explicit FP32 vectors.
int operator_apply32(OperatorData& op, float const* x, float* y, cudaStream_t stream);
// Krylov-indirect apply (see Indirect); `blocks` receives the grid size, i.e.
// the number of partial sums written.
int operator_apply_krylov(OperatorData& op, int dtype, void* base, Indirect ind, cudaStream_t stream,
                          unsigned* blocks);
int operator_ensure_ready(OperatorData& op);

// V[:, 0..kk) <- V[:, 0..m) Y on the tensor cores (rotate_tc.cu): V FP64,
// D x m with column stride ld, Y m x kk row-major FP64, both on the device;
// *error_flag (device int) is set to 1 if a bounded wait ran out.
bool rotate_tc_eligible(uint32_t m, uint32_t kk);
int rotate_tc(double* V, uint64_t ld, uint32_t m, double const* Y, uint32_t kk, uint64_t D, cudaStream_t stream,
              int* error_flag);
// Path of the thick restart's basis rotation (sed_set_rotate_path).
extern int g_rotate_path;

}  // namespace sed
