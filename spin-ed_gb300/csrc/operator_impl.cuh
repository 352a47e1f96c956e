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


struct OperatorTables {
  DeviceBuffer divisors;
  DeviceBuffer table;    // double[n_codes], real operators only
  DeviceBuffer table_c;  // double2[n_codes], every operator
  DeviceBuffer inv_sqrt_s;
  CodeView code{};
  uint32_t n_codes = 0;
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

}  // namespace sed
