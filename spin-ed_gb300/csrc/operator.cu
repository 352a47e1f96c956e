// operator.cu — interactions, operators and the symmetry-adapted matvec
// (src/SpinED/Internal.hs:256-458).
//
// Pull form, atomic-free: row i (representative r_i) owns y_i and sums
//     y_i = diag(r_i) x_i + (1/sqrt(S_i)) sum_e V[code_e] x_{j_e}
// over the off-diagonal elements e of the local terms: s_e = r_i with the
// bits of one site tuple replaced (a -> a'), coefficient <r_i|H|s_e> =
// M[a][a'], rho_e = orbit minimum of s_e with character chi_e, j_e = index of
// rho_e, and V[code] = M[a][a'] chi_e sqrt(S_{j_e}). This is
// <r~_i|H|r~_j> = sum_s <r_i|H|s> chi(h_s) n_j / n_i with n = sqrt(S / |G|),
// which holds for any G-invariant H (no Hermiticity needed).
//
// Two forms compute the same sum in the same order, so they agree bit for
// bit:
//   on-the-fly  canonicalises every s_e per call (integer-bound);
//   stream      records (j_e, code_e) once in SELL-32 slices (32 rows per
//               warp, slot e of row lane at slice_ptr + 32 e + lane) and then
//               streams it: an HBM/FP64-bound SpMV.
#include <chrono>
#include <cmath>
#include <cstring>
#include <type_traits>

#include "operator_impl.cuh"

namespace sed {
namespace {

// ---------------------------------------------------------------- kernels --

// Per-slice maximum element count (slots = 32 * max) and element total.
// (max_width: the largest slice width, for sizing k_record's buffers.)
__global__ void k_count(uint64_t const* __restrict__ reps, uint64_t D, TermsView T,
                        uint64_t n_slices, uint64_t* __restrict__ slots,
                        uint64_t* __restrict__ elements, unsigned* __restrict__ max_width) {
  uint64_t const i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t const s = i >> 5;
  if (s >= n_slices) return;
  uint32_t const c = i < D ? row_count(reps[i], T) : 0u;
  uint32_t const m = __reduce_max_sync(0xffffffffu, c);
  uint32_t const tot = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0) {
    slots[s] = (uint64_t)m * 32;
    elements[s] = tot;
    atomicMax(max_width, m);
  }
}

constexpr unsigned kRecWarps = 4;    // warps per block of k_record
constexpr unsigned kRecBlocks = 5;   // blocks of k_record per SM the registers allow
constexpr unsigned kRecMaxElems = 80; // flattened path: elements per row at most

// k_record's shared memory for `me` element slots per row and `nc` cosets:
// sized by the operator, so that narrow rows leave room for more blocks.
size_t record_smem_bytes(unsigned me, unsigned nc) {
  return (size_t)kRecWarps * 32 * me * 4      // element descriptors
         + (size_t)kRecWarps * 32 * nc * 8    // coset images of each row
         + (size_t)nc * 64                    // bit landing positions
         + 2048 * 2;                          // row tables
}

// Records the stream form. One warp per SELL-32 slice (lane = row).
//  - Each lane applies the coset representatives to its row's representative
//    r once (Benes networks) and keeps the images in shared memory; an
//    element s = r ^ d (d: the few flipped bits) then costs
//    P_c(s) = P_c(r) ^ P_c(d), with P_c(d) assembled from the bit landing
//    table, instead of a full network per coset.
//  - When the slice is at most kRecMaxElems wide, each lane lists its row's
//    elements as (tuple, column) descriptors and the warp walks the flattened
//    (row, element) list 32 at a time, so rows of different length do not
//    leave lanes idle; wider slices fall back to one row per lane.
// Entries land in the same slots (slice_ptr + 32 e + row) either way.
template <class W, bool Real>
__global__ void __launch_bounds__(kRecWarps * 32, kRecBlocks)
    k_record(__grid_constant__ const PlanView P, IndexView I, TermsView T, CodeView C,
             uint32_t const* __restrict__ weights, uint64_t n_slices, uint64_t const* __restrict__ slice_ptr,
             uint32_t col_bits, bool packed, uint32_t* __restrict__ entries, uint16_t* __restrict__ codes,
             void* __restrict__ diag, uint8_t* __restrict__ row_class, uint32_t me, uint32_t nc) {
  extern __shared__ __align__(16) unsigned char rec_smem[];
  uint32_t* desc_all = reinterpret_cast<uint32_t*>(rec_smem);
  W* imgs_all = reinterpret_cast<W*>(rec_smem + (size_t)kRecWarps * 32 * me * 4);
  uint8_t* pos_s = rec_smem + (size_t)kRecWarps * 32 * me * 4 + (size_t)kRecWarps * 32 * nc * 8;
  uint16_t* srow = reinterpret_cast<uint16_t*>(pos_s + nc * 64);
  RowTab const RT = stage_rows(P, srow);
  bool const use_pos = P.fixed_nets != 0;
  if (use_pos) {
    for (uint32_t q = threadIdx.x; q < P.n_cosets * 64; q += blockDim.x) pos_s[q] = P.pos[q];  // n_cosets <= nc
    __syncthreads();
  }
  uint32_t const warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint64_t const s = (uint64_t)blockIdx.x * kRecWarps + warp;
  if (s >= n_slices) return;  // warp-uniform
  uint32_t* desc = desc_all + (size_t)warp * 32 * me;
  W* imgs = imgs_all + (size_t)warp * 32 * nc;
  uint64_t const i = s * 32 + lane;
  uint64_t const base = slice_ptr[s];
  uint32_t const width = (uint32_t)((slice_ptr[s + 1] - base) >> 5);
  bool const valid = i < I.D;
  uint64_t const r = valid ? I.reps[i] : 0;
  if (use_pos)
    for (uint32_t c = 0; c < P.n_cosets; ++c) imgs[lane * nc + c] = coset_apply<W>((W)r, P, c);
  __syncwarp();
  auto emit = [&](uint32_t e, uint32_t row, uint64_t r_row, uint64_t st, uint32_t vid) {
    W const x = (W)st;
    W const delta = (W)(st ^ r_row);
    auto img = [&](uint32_t c) -> W {
      if (c == 0) return x;
      if (!use_pos) return coset_apply<W>(x, P, c);
      W d = delta, pd = 0;
      while (d) {
        uint32_t const b = (uint32_t)__ffsll((long long)(uint64_t)d) - 1u;
        d &= d - 1;
        pd |= (W)1 << pos_s[c * 64 + b];
      }
      return imgs[row * nc + c] ^ pd;
    };
    auto const cz = canonicalize_img<W>(x, P, RT, img);
    int64_t const j = find_index((uint64_t)cz.rep, I);
    uint32_t ent = kNull, code = 0;
    if (j >= 0) {
      code = element_code(vid, cz.phase, weights[j], C);
      ent = packed ? ((uint32_t)j | (code << col_bits)) : (uint32_t)j;
    }
    entries[base + (uint64_t)e * 32 + row] = ent;
    if (!packed) codes[base + (uint64_t)e * 32 + row] = (uint16_t)code;
  };
  uint32_t count = 0;
  if (width <= me && T.n_tuples < 65536) {
    if (valid) {
      for (uint32_t u = 0; u < T.n_tuples; ++u) {
        uint32_t const tk = T.tuple_term[u];
        uint32_t const t = tk & 0xFFFFu, k = tk >> 16;
        uint32_t const a = local_index(r, T.tuple_sites[u], k);
        uint32_t const n = T.n_off[t * 16 + a];
        for (uint32_t q = 0; q < n; ++q)
          desc[lane * me + count++] = (q << 28) | (u << 8) | T.off_col[(t * 16 + a) * 16 + q];
      }
    }
    __syncwarp();
    // exclusive prefix of counts over the lanes
    uint32_t incl = count;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t const v = __shfl_up_sync(0xffffffffu, incl, o);
      if ((int)lane >= o) incl += v;
    }
    uint32_t const total = __shfl_sync(0xffffffffu, incl, 31);
    uint32_t const excl = incl - count;
    for (uint32_t f0 = 0; f0 < total; f0 += 32) {
      uint32_t const f = f0 + lane;
      // owning row: the largest lane whose exclusive prefix is <= f
      uint32_t row = 0;
      for (uint32_t step = 16; step > 0; step >>= 1) {
        uint32_t const probe = row + step;
        uint32_t const ex = __shfl_sync(0xffffffffu, excl, probe & 31u);
        if (probe < 32u && ex <= f) row = probe;
      }
      uint32_t const ex_row = __shfl_sync(0xffffffffu, excl, row);
      uint64_t const r_row = __shfl_sync(0xffffffffu, r, row);
      if (f < total) {
        uint32_t const e = f - ex_row;
        uint32_t const d = desc[row * me + e];
        uint32_t const u = (d >> 8) & 0xFFFFu, a2 = d & 0xFFu, q = d >> 28;
        uint32_t const tk = T.tuple_term[u];
        uint32_t const t = tk & 0xFFFFu, k = tk >> 16;
        uint32_t const sites = T.tuple_sites[u];
        uint32_t const a = local_index(r_row, sites, k);
        emit(e, row, r_row, replace_local(r_row, sites, k, a2), T.off_vid[(t * 16 + a) * 16 + q]);
      }
    }
  } else if (valid) {
    walk_row(r, T, [&](uint32_t e, uint64_t st, uint32_t vid) {
      emit(e, lane, r, st, vid);
      count = e + 1;
    });
  }
  if (valid) {
    if (Real) {
      static_cast<double*>(diag)[i] = row_diag<double>(r, T);
    } else {
      cplx const d = row_diag<cplx>(r, T);
      static_cast<double2*>(diag)[i] = make_double2(d.re, d.im);
    }
    row_class[i] = (uint8_t)divisor_class(weights[i], C);
  }
  for (uint32_t e = count; e < width; ++e) {
    entries[base + (uint64_t)e * 32 + lane] = kNull;
    if (!packed) codes[base + (uint64_t)e * 32 + lane] = 0;
  }
}

// Streamed SpMV over SELL-32 slices. RealOp selects the real table/diagonal.
// With an Indirect (Krylov) view, x = base + k ld and y = base + (k+1) ld
// with k read from device memory, and each block writes sum_i Re(x_i* y_i).
template <class X, bool RealOp, bool Packed>
__global__ void __launch_bounds__(kBlock) k_spmv(StreamView S, uint64_t D, X const* __restrict__ x,
                                                 X* __restrict__ y, Indirect ind) {
  using V = typename Store<X>::V;
  extern __shared__ unsigned char smem_raw[];
  __shared__ double red[kBlock / 32];
  if (ind.stop && *ind.stop) return;  // uniform across the grid
  if (ind.k) {
    uint64_t const k = *ind.k;
    x += k * ind.ld;
    y += (k + 1) * ind.ld;
  }
  void const* table = stage_table<RealOp>(S, smem_raw);
  uint64_t const i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t const s = i >> 5;
  double part = 0.0;
  if ((s << 5) < D) {
    V const acc = stream_row_acc<V, X, RealOp, Packed>(S, table, s, threadIdx.x & 31, x);
    if (i < D) {
      double const f = S.inv_sqrt_s[S.row_class[i]];
      V const xi = Store<X>::load(x, i);
      V const yi = row_value<V>(mulv(stream_diag<V, RealOp>(S, i), xi), f, acc);
      Store<X>::store(y, i, yi);
      part = dot_re(xi, yi);
    }
  }
  if (ind.partial) {
    double const tot = block_sum(part, red);
    if (threadIdx.x == 0) ind.partial[blockIdx.x] = tot;
  }
}

// Block form: K columns per pass, each recorded element decoded once and
// applied to all K columns (the block matvec of src/SpinED.hs:172's
// max_primme_block_size). Per column the sum and its order are those of
// k_spmv, so results are bit-identical to K single-column calls.
template <class X, bool RealOp, bool Packed, int K>
__global__ void __launch_bounds__(kBlock) k_spmv_block(StreamView S, uint64_t D, X const* __restrict__ x,
                                                       uint64_t ldx, X* __restrict__ y, uint64_t ldy) {
  using V = typename Store<X>::V;
  extern __shared__ unsigned char smem_raw[];
  void const* table = stage_table<RealOp>(S, smem_raw);
  uint64_t const i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t const s = i >> 5;
  if ((s << 5) >= D) return;
  uint32_t const lane = threadIdx.x & 31;
  uint64_t const base = S.slice_ptr[s];
  uint32_t const width = (uint32_t)((S.slice_ptr[s + 1] - base) >> 5);
  uint32_t const col_mask = Packed ? ((1u << S.col_bits) - 1u) : 0xFFFFFFFFu;
  V acc[K];
#pragma unroll
  for (int c = 0; c < K; ++c) acc[c] = zero<V>();
  uint32_t const* ent = S.entries + base + lane;
  for (uint32_t e = 0; e < width; ++e) {
    uint32_t const v = __ldcs(ent + (uint64_t)e * 32);
    if (v != kNull) {
      uint32_t const col = v & col_mask;
      uint32_t const code = Packed ? (v >> S.col_bits) : (uint32_t)__ldcs(S.codes + base + lane + (uint64_t)e * 32);
      V const t = load_table<V>(table, code, RealOp);
#pragma unroll
      for (int c = 0; c < K; ++c) mac(acc[c], t, Store<X>::load(x + c * ldx, col));
    }
  }
  if (i < D) {
    double const f = S.inv_sqrt_s[S.row_class[i]];
    V const dg = stream_diag<V, RealOp>(S, i);
#pragma unroll
    for (int c = 0; c < K; ++c)
      Store<X>::store(y + c * ldy, i, row_value<V>(mulv(dg, Store<X>::load(x + c * ldx, i)), f, acc[c]));
  }
}

// On-the-fly matvec: same sum, same order, recomputing every element.
template <class W, class X, bool RealOp>
__global__ void __launch_bounds__(kBlock)
    k_otf(__grid_constant__ const PlanView P, IndexView I, TermsView T, CodeView C, uint32_t const* __restrict__ weights,
          void const* __restrict__ table, double const* __restrict__ inv_sqrt_s,
          X const* __restrict__ x, X* __restrict__ y, Indirect ind) {
  using V = typename Store<X>::V;
  __shared__ double red[kBlock / 32];
  __shared__ uint16_t srow[2048];
  if (ind.stop && *ind.stop) return;
  RowTab const RT = stage_rows(P, srow);
  if (ind.k) {
    uint64_t const k = *ind.k;
    x += k * ind.ld;
    y += (k + 1) * ind.ld;
  }
  uint64_t const i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double part = 0.0;
  if (i < I.D) {
    uint64_t const r = I.reps[i];
    V acc = zero<V>();
    walk_row(r, T, [&](uint32_t, uint64_t st, uint32_t vid) {
      auto const c = canonicalize<W>((W)st, P, RT);
      int64_t const j = find_index((uint64_t)c.rep, I);
      if (j >= 0) {
        uint32_t const code = element_code(vid, c.phase, weights[j], C);
        mac(acc, load_table<V>(table, code, RealOp), Store<X>::load(x, (uint64_t)j));
      }
    });
    V dg;
    if constexpr (std::is_same<V, double>::value) {
      dg = row_diag<double>(r, T);
    } else {
      dg = RealOp ? cplx{row_diag<double>(r, T), 0.0} : row_diag<cplx>(r, T);
    }
    uint32_t const cls = divisor_class(weights[i], C);
    V const xi = Store<X>::load(x, i);
    V const yi = row_value<V>(mulv(dg, xi), inv_sqrt_s[cls], acc);
    Store<X>::store(y, i, yi);
    part = dot_re(xi, yi);
  }
  if (ind.partial) {
    double const tot = block_sum(part, red);
    if (threadIdx.x == 0) ind.partial[blockIdx.x] = tot;
  }
}

// ------------------------------------------------ fixed-point matvec ----
// (the mathematics is at FixView in operator_impl.cuh)

// Largest |x_j| of column blockIdx.y as a bit pattern (for finite
// non-negative doubles the integer order is the numeric order; NaN and
// infinity patterns are larger than every finite one). `max_bits` must be
// zero on entry.
__global__ void __launch_bounds__(kBlock) k_fix_max(double const* __restrict__ x, uint64_t ldx, uint64_t D,
                                                    unsigned long long* __restrict__ max_bits, Indirect ind) {
  __shared__ unsigned long long red[kBlock / 32];
  if (ind.stop && *ind.stop) return;
  if (ind.k) x += (uint64_t)*ind.k * ind.ld;
  x += (uint64_t)blockIdx.y * ldx;
  unsigned long long m = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (uint64_t)gridDim.x * blockDim.x)
    m = max(m, (unsigned long long)__double_as_longlong(x[i]) & 0x7FFFFFFFFFFFFFFFull);
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (unsigned w = 1; w < kBlock / 32; ++w) m = max(m, red[w]);
    atomicMax(max_bits + blockIdx.y, m);
  }
}

// u_j = round(sqrt(S_j) x_j 2^F) for column blockIdx.y; block 0 stores F.
// The class of row j comes from the stream form's row_class, or from the
// stabiliser orders when there is no stream form.
__global__ void __launch_bounds__(kBlock) k_fix_convert(double const* __restrict__ x, uint64_t ldx, uint64_t D,
                                                        uint8_t const* __restrict__ row_class,
                                                        uint32_t const* __restrict__ weights, CodeView C, FixView fv,
                                                        unsigned long long const* __restrict__ max_bits,
                                                        int64_t* __restrict__ F_out, int64_t* __restrict__ u,
                                                        uint64_t ldu, Indirect ind) {
  __shared__ double fac[kFixMaxClasses];
  if (ind.stop && *ind.stop) return;
  if (ind.k) x += (uint64_t)*ind.k * ind.ld;
  x += (uint64_t)blockIdx.y * ldx;
  u += (uint64_t)blockIdx.y * ldu;
  int64_t const F = fix_exponent(max_bits[blockIdx.y], fv.bound);
  if (blockIdx.x == 0 && threadIdx.x == 0) F_out[blockIdx.y] = F;
  // x 2^F sqrt(S) as (x 2^F1) (sqrt(S) 2^F2): F1 = 0 unless 2^F is not a
  // normal double (vectors whose largest entry is below about 1e-290 or
  // above about 1e290)
  int64_t const F1 = (F == kFixBad || (F >= -1000 && F <= 1000)) ? 0 : F / 2;
  double const p1 = fix_pow2(F1);
  double const p2 = F == kFixBad ? 0.0 : fix_pow2(F - F1);
  for (uint32_t c = threadIdx.x; c < fv.n_div; c += blockDim.x) fac[c] = fv.sqrt_s[c] * p2;
  __syncthreads();
  if (F1 == 0) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (uint64_t)gridDim.x * blockDim.x) {
      uint32_t const cls = row_class ? (uint32_t)row_class[i] : divisor_class(weights[i], C);
      u[i] = F == kFixBad ? 0 : fix_round(x[i] * fac[cls]);
    }
  } else {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (uint64_t)gridDim.x * blockDim.x) {
      uint32_t const cls = row_class ? (uint32_t)row_class[i] : divisor_class(weights[i], C);
      u[i] = fix_round((x[i] * p1) * fac[cls]);
    }
  }
}

// Adds +-g to the accumulator of value index t >> 1 (sign t & 1).
template <int NV>
__device__ __forceinline__ void fix_add(int64_t (&acc)[NV], uint32_t t, int64_t g) {
  int64_t const v = (t & 1u) ? -g : g;
  if constexpr (NV == 1) {
    acc[0] += v;
  } else {
    uint32_t const q = t >> 1;
#pragma unroll
    for (int k = 0; k < NV; ++k)
      if (q == (uint32_t)k) acc[k] += v;
  }
}

// The row factors g[cls NV + v] = (c_v / sqrt(S_cls)) 2^-min(F, 1000), one
// table per block in shared memory (one rounding of c_v / sqrt(S), then an
// exact power of two). F above 1000 only occurs for vectors whose largest
// entry is below about 1e-290; the rest of the scaling is then applied by
// fix_row after the sum, so that g stays a normal number. Every thread of
// the block calls it; the caller synchronises.
template <int NV>
__device__ __forceinline__ void fix_row_factors(FixView const& fv, double const* __restrict__ inv_sqrt_s, int64_t F,
                                                double* g) {
  int64_t const Fa = F > 1000 ? 1000 : F;
  for (uint32_t t = threadIdx.x; t < fv.n_div * NV; t += blockDim.x)
    g[t] = F == kFixBad ? 0.0 : fix_ldexp(__dmul_rn(inv_sqrt_s[t / NV], fv.c[t % NV]), -Fa);
}

// The row's epilogue, shared by every fixed-point kernel so that all of them
// round identically: y_i = d_i x_i + sum_v g[cls][v] acc_v (times
// 2^-(F - 1000) when F > 1000), with g from fix_row_factors (g points at the
// row's class).
template <int NV>
__device__ __forceinline__ double fix_row(int64_t const (&acc)[NV], double const* g, int64_t F, double dg, double xi) {
  if (F == kFixBad) return __longlong_as_double(0x7FF8000000000000ll);  // NaN in x gives NaN out
  if (F > 1000) {
    double o = 0.0;
#pragma unroll
    for (int k = 0; k < NV; ++k) o = __fma_rn(g[k], __ll2double_rn(acc[k]), o);
    return __fma_rn(o, fix_pow2(1000 - F), __dmul_rn(dg, xi));
  }
  double s = __dmul_rn(dg, xi);
#pragma unroll
  for (int k = 0; k < NV; ++k) s = __fma_rn(g[k], __ll2double_rn(acc[k]), s);
  return s;
}

// Sum of one double per thread over the block, in a fixed order, through
// shared memory (buf: blockDim.x doubles): the first warp adds eight values
// per lane, then across lanes. The total is valid in thread 0.
__device__ __forceinline__ double block_sum_fixed(double v, double* buf) {
  buf[threadIdx.x] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x < 32) {
    for (uint32_t q = threadIdx.x; q < blockDim.x; q += 32) s += buf[q];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  }
  return s;
}

// Streamed SpMV over SELL-32 slices in fixed point (real operators). Four
// entries per step: their loads, then their gathers, are issued back to back
// (a padding slot gathers nothing and adds zero). Indirect (Krylov) mode as
// in k_spmv.
template <bool Packed, int NV>
__global__ void __launch_bounds__(kBlock) k_spmv_fix(StreamView S, FixView fv, uint64_t D,
                                                     double const* __restrict__ x, int64_t const* __restrict__ u,
                                                     int64_t const* __restrict__ F_in, double* __restrict__ y,
                                                     Indirect ind) {
  extern __shared__ double fix_smem[];  // g[n_div NV], then code8[n_codes]
  __shared__ double red[kBlock];
  if (ind.stop && *ind.stop) return;  // uniform across the grid
  if (ind.k) {
    uint64_t const k = *ind.k;
    x += k * ind.ld;
    y += (k + 1) * ind.ld;
  }
  int64_t const F = F_in[0];
  double* g = fix_smem;
  uint8_t* code8 = reinterpret_cast<uint8_t*>(fix_smem + fv.n_div * NV);
  for (uint32_t c = threadIdx.x; c < fv.n_codes; c += blockDim.x) code8[c] = fv.code[c];
  fix_row_factors<NV>(fv, S.inv_sqrt_s, F, g);
  __syncthreads();
  uint64_t const i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t const s = i >> 5;
  double part = 0.0;
  if ((s << 5) < D) {
    uint32_t const lane = threadIdx.x & 31;
    uint64_t const base = S.slice_ptr[s];
    uint32_t const width = (uint32_t)((S.slice_ptr[s + 1] - base) >> 5);
    uint32_t const col_mask = Packed ? ((1u << S.col_bits) - 1u) : 0xFFFFFFFFu;
    int64_t acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0;
    uint32_t const* ent = S.entries + base + lane;
    constexpr uint32_t U = 8;
    uint32_t e = 0;
    for (; e + U <= width; e += U) {
      uint32_t v[U];
#pragma unroll
      for (uint32_t q = 0; q < U; ++q) v[q] = __ldcs(ent + (uint64_t)(e + q) * 32);
      int64_t g[U];
      uint32_t t[U];
#pragma unroll
      for (uint32_t q = 0; q < U; ++q) {
        g[q] = 0;
        t[q] = 0;
        if (v[q] != kNull) {
          uint32_t const code =
              Packed ? (v[q] >> S.col_bits) : (uint32_t)__ldcs(S.codes + base + lane + (uint64_t)(e + q) * 32);
          g[q] = u[v[q] & col_mask];
          t[q] = code8[code];
        }
      }
#pragma unroll
      for (uint32_t q = 0; q < U; ++q) fix_add<NV>(acc, t[q], g[q]);
    }
    for (; e < width; ++e) {
      uint32_t const v = __ldcs(ent + (uint64_t)e * 32);
      if (v != kNull) {
        uint32_t const code = Packed ? (v >> S.col_bits) : (uint32_t)__ldcs(S.codes + base + lane + (uint64_t)e * 32);
        fix_add<NV>(acc, code8[code], u[v & col_mask]);
      }
    }
    if (i < D) {
      double const xi = __ldcs(x + i);
      double const yi = fix_row<NV>(acc, g + (uint32_t)__ldcs(S.row_class + i) * NV, F,
                                    __ldcs(static_cast<double const*>(S.diag) + i), xi);
      __stcs(y + i, yi);
      part = xi * yi;
    }
  }
  if (ind.partial) {
    double const tot = block_sum_fixed(part, red);
    if (threadIdx.x == 0) ind.partial[blockIdx.x] = tot;
  }
}

// Block form in fixed point: K columns, u column c at u + c * D, F_in[c].
template <bool Packed, int NV, int K>
__global__ void __launch_bounds__(kBlock) k_spmv_block_fix(StreamView S, FixView fv, uint64_t D,
                                                           double const* __restrict__ x, uint64_t ldx,
                                                           int64_t const* __restrict__ u,
                                                           int64_t const* __restrict__ F_in, double* __restrict__ y,
                                                           uint64_t ldy) {
  extern __shared__ double fix_smem[];  // g[K][n_div NV], then code8[n_codes]
  uint8_t* code8 = reinterpret_cast<uint8_t*>(fix_smem + K * fv.n_div * NV);
  for (uint32_t c = threadIdx.x; c < fv.n_codes; c += blockDim.x) code8[c] = fv.code[c];
#pragma unroll
  for (int c = 0; c < K; ++c) fix_row_factors<NV>(fv, S.inv_sqrt_s, F_in[c], fix_smem + c * fv.n_div * NV);
  __syncthreads();
  uint64_t const i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t const s = i >> 5;
  if ((s << 5) >= D) return;
  uint32_t const lane = threadIdx.x & 31;
  uint64_t const base = S.slice_ptr[s];
  uint32_t const width = (uint32_t)((S.slice_ptr[s + 1] - base) >> 5);
  uint32_t const col_mask = Packed ? ((1u << S.col_bits) - 1u) : 0xFFFFFFFFu;
  int64_t acc[K][NV];
#pragma unroll
  for (int c = 0; c < K; ++c)
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[c][k] = 0;
  uint32_t const* ent = S.entries + base + lane;
  for (uint32_t e = 0; e < width; ++e) {
    uint32_t const v = __ldcs(ent + (uint64_t)e * 32);
    if (v != kNull) {
      uint32_t const col = v & col_mask;
      uint32_t const code = Packed ? (v >> S.col_bits) : (uint32_t)__ldcs(S.codes + base + lane + (uint64_t)e * 32);
      uint32_t const t = code8[code];
#pragma unroll
      for (int c = 0; c < K; ++c) fix_add<NV>(acc[c], t, u[(uint64_t)c * D + col]);
    }
  }
  if (i < D) {
    uint32_t const cls = S.row_class[i];
    double const dg = static_cast<double const*>(S.diag)[i];
#pragma unroll
    for (int c = 0; c < K; ++c)
      y[(uint64_t)c * ldy + i] =
          fix_row<NV>(acc[c], fix_smem + (c * fv.n_div + cls) * NV, F_in[c], dg, x[(uint64_t)c * ldx + i]);
  }
}

// On-the-fly matvec in fixed point: the same integer sums as k_spmv_fix
// (in another order, which integers do not notice) and the same epilogue.
template <class W, int NV>
__global__ void __launch_bounds__(kBlock)
    k_otf_fix(__grid_constant__ const PlanView P, IndexView I, TermsView T, CodeView C,
              uint32_t const* __restrict__ weights, FixView fv, double const* __restrict__ inv_sqrt_s,
              double const* __restrict__ x, int64_t const* __restrict__ u, int64_t const* __restrict__ F_in,
              double* __restrict__ y, Indirect ind) {
  __shared__ double red[kBlock];
  __shared__ double g[kFixMaxClasses * NV];
  __shared__ uint16_t srow[2048];
  if (ind.stop && *ind.stop) return;
  int64_t const F = F_in[0];
  fix_row_factors<NV>(fv, inv_sqrt_s, F, g);
  RowTab const RT = stage_rows(P, srow);
  __syncthreads();
  if (ind.k) {
    uint64_t const k = *ind.k;
    x += k * ind.ld;
    y += (k + 1) * ind.ld;
  }
  uint64_t const i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double part = 0.0;
  if (i < I.D) {
    uint64_t const r = I.reps[i];
    int64_t acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0;
    walk_row(r, T, [&](uint32_t, uint64_t st, uint32_t vid) {
      auto const c = canonicalize<W>((W)st, P, RT);
      int64_t const j = find_index((uint64_t)c.rep, I);
      if (j >= 0) fix_add<NV>(acc, vid << 1 | (c.phase != 0u ? 1u : 0u), u[(uint64_t)j]);
    });
    double const xi = x[i];
    double const yi = fix_row<NV>(acc, g + divisor_class(weights[i], C) * NV, F, row_diag<double>(r, T), xi);
    y[i] = yi;
    part = xi * yi;
  }
  if (ind.partial) {
    double const tot = block_sum_fixed(part, red);
    if (threadIdx.x == 0) ind.partial[blockIdx.x] = tot;
  }
}

template <class X>
__global__ void k_dot_conj(X const* __restrict__ x, X const* __restrict__ y, uint64_t n,
                           double2* __restrict__ partial) {
  using V = typename Store<X>::V;
  __shared__ double2 red[kBlock / 32];
  double re = 0.0, im = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    V const a = Store<X>::load(x, i), b = Store<X>::load(y, i);
    if constexpr (std::is_same<V, double>::value) {
      re = fma(a, b, re);
    } else {
      re = fma(a.re, b.re, fma(a.im, b.im, re));
      im = fma(a.re, b.im, fma(-a.im, b.re, im));
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_double2(re, im);
  __syncthreads();
  if (threadIdx.x == 0) {
    double2 s = make_double2(0.0, 0.0);
    for (unsigned w = 0; w < kBlock / 32; ++w) {
      s.x += red[w].x;
      s.y += red[w].y;
    }
    partial[blockIdx.x] = s;
  }
}

// ----------------------------------------------------------- host helpers --

std::vector<uint32_t> divisors_of(uint32_t n) {
  std::vector<uint32_t> d;
  for (uint32_t k = 1; k <= n; ++k)
    if (n % k == 0) d.push_back(k);
  return d;
}

void root_of_unity(uint32_t q, uint32_t L, double& re, double& im) {
  if (q == 0) {
    re = 1.0; im = 0.0;
  } else if (4 * q == L) {
    re = 0.0; im = -1.0;
  } else if (2 * q == L) {
    re = -1.0; im = 0.0;
  } else if (4 * q == 3 * L) {
    re = 0.0; im = 1.0;
  } else {
    double const ang = -2.0 * 3.14159265358979323846 * (double)q / (double)L;
    re = std::cos(ang);
    im = std::sin(ang);
  }
}

// ------------------------------------------------------------ orbit table --
// An alternative to canonicalising every generated element: a table over the
// whole weight class of the basis (C(n, w) words, or 2^n without a Hamming
// weight) that maps each word to the index of its orbit's representative and
// the sign of the character of the element taking it there (real characters
// only), filled by enumerating the orbit of every representative once. The
// stream form then costs one rank computation and one table load per element
// instead of a search over the group. Words of orbits outside the basis keep
// the fill value kNull.

constexpr uint32_t kTabSign = 0x80000000u;

// Colex rank of x among the words of weight hw (hw >= 0), or x itself.
__device__ __forceinline__ uint64_t word_rank(uint64_t x, int hw, uint64_t const* __restrict__ bin /* [64][33] */) {
  if (hw < 0) return x;
  uint64_t rk = 0;
  uint32_t i = 0;
  while (x) {
    uint32_t const p = (uint32_t)(__ffsll((long long)x) - 1);
    x &= x - 1;
    ++i;
    rk += bin[p * 33 + i];
  }
  return rk;
}

__device__ __forceinline__ void stage_binom(uint64_t const* __restrict__ binom, uint64_t* bin) {
  for (uint32_t q = threadIdx.x; q < 64 * 33; q += blockDim.x) {
    uint32_t const p = q / 33, i = q % 33;
    bin[q] = binom[p * 65 + i];
  }
}

// Colex rank by 6-bit chunks: R[(c * (w + 1) + m) * 64 + v] is the sum of
// C(6 c + q, m + i) over the set bits q of v (the i-th of them, from 1), for
// m set bits below chunk c; the rank is the sum over the chunks.
struct RankTab {
  uint64_t const* R;  // shared memory, or null for the bit-by-bit loop
  uint32_t n_chunks, wp1;
};

__device__ __forceinline__ uint64_t word_rank_tab(uint64_t x, int hw, RankTab const& T, uint64_t const* bin) {
  if (hw < 0) return x;
  if (!T.R) return word_rank(x, hw, bin);
  uint64_t rk = 0;
  uint32_t m = 0;
  for (uint32_t c = 0; c < T.n_chunks; ++c) {
    uint32_t const v = (uint32_t)(x >> (6 * c)) & 63u;
    rk += T.R[(c * T.wp1 + m) * 64 + v];
    m += __popc(v);
  }
  return rk;
}

// Stages the chunked rank table (rank_bytes > 0) or the binomial table into
// the dynamic shared memory `dyn`; returns the rank view.
__device__ __forceinline__ RankTab stage_rank(uint64_t const* __restrict__ binom, uint64_t const* __restrict__ rank_tab,
                                              uint32_t rank_words, uint32_t n_chunks, uint32_t wp1, uint64_t* dyn) {
  if (rank_words) {
    for (uint32_t q = threadIdx.x; q < rank_words; q += blockDim.x) dyn[q] = rank_tab[q];
    return RankTab{dyn, n_chunks, wp1};
  }
  stage_binom(binom, dyn);
  return RankTab{nullptr, 0, 0};
}

// Table index on a row-structured group: the stored words (rows_rot_min
// classes) have a smallest-rotation top row T, so the table is laid out as
// one segment per such T, of the ranks of the lower bits in their weight
// class: index = seg_off[T] + rank(low bits). seg_off[T] is ~0 for a top
// row that cannot occur.
struct RowIndex {
  uint64_t const* seg_off;  // [1 << row_bits], or null: plain colex rank of the whole word
  uint64_t low_mask;
  uint32_t top_shift;
};

__device__ __forceinline__ uint64_t table_index(uint64_t w, int hw, RankTab const& RK, uint64_t const* bin,
                                                RowIndex const& RI) {
  if (!RI.seg_off) return word_rank_tab(w, hw, RK, bin);
  uint64_t const off = __ldg(RI.seg_off + (w >> RI.top_shift));
  if (off == ~(uint64_t)0) return off;
  return off + word_rank_tab(w & RI.low_mask, hw, RK, bin);
}

// On a row-structured group (a torus: one generator rotates every row, the
// other shifts rows) the table stores, of each set {row rotations of z and of
// ~z}, only the smallest word: it has the smallest rotation of z's (or ~z's)
// top row on top, so only the rotations listed in the group's row tables are
// built. Returns the smallest word and the phase of the element (rotation,
// inversion) taking z to it.
template <class W>
__device__ __forceinline__ W rows_rot_min(W z, PlanView const& P, RowTab const& R, uint32_t* kphase) {
  W const mask = (W)P.mask;
  uint32_t const rm = (uint32_t)P.row_mask, top = P.n_rows - 1;
  uint32_t const tv = (uint32_t)(z >> (top * P.row_bits)) & rm;
  uint32_t M = R.min[tv];
  if (P.inv) {
    uint32_t const b = R.min[tv ^ rm];
    M = b < M ? b : M;
  }
  W best = mask;
  uint32_t br = 0, binv = 0;
  for (uint32_t inv = 0; inv <= (P.inv ? 1u : 0u); ++inv) {
    uint32_t const v = inv ? (tv ^ rm) : tv;
    if (R.min[v] != M) continue;
    uint32_t set = R.set[v];
    while (set) {
      uint32_t const r = (uint32_t)__builtin_ctz_sed(set);
      set &= set - 1;
      W const c = cand_image<W>(z, mask, P, top, r, inv);
      if (c < best) {
        best = c;
        br = r;
        binv = inv;
      }
    }
  }
  uint64_t ph = (uint64_t)P.rot_exp[br] * P.rot_phase;
  if (binv) ph += P.inv_phase;
  *kphase = (uint32_t)(ph % P.L);
  return best;
}

// One thread per (representative, coset): every image h(p_c(r)) (and its
// spin-inverted word) gets table entry j | sign(character of the element).
// With spin inversion in the group only words whose top bit (n - 1) is clear
// are stored (their colex ranks are the first C(n - 1, w)): of each pair
// {z, ~z} the one with the clear top bit is written, once, and a lookup of a
// word with the top bit set looks up its inverse and flips the sign by the
// inversion character.
template <class W>
__global__ void __launch_bounds__(256) k_orbit_scatter(__grid_constant__ const PlanView P, uint64_t const* __restrict__ reps,
                                                       uint64_t D, int hw, uint64_t const* __restrict__ binom,
                                                       uint32_t* __restrict__ table, uint64_t space,
                                                       int* __restrict__ error, uint64_t const* __restrict__ rank_tab,
                                                       uint32_t rank_words, uint32_t n_chunks, uint32_t wp1,
                                                       RowIndex RI) {
  extern __shared__ uint64_t dyn_rank[];
  __shared__ uint16_t rows_s[2048];
  uint64_t const* const bin = dyn_rank;
  RankTab const RK = stage_rank(binom, rank_tab, rank_words, n_chunks, wp1, dyn_rank);
  RowTab const RT = stage_rows(P, rows_s);  // synchronises the block
  __syncthreads();
  uint64_t const t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t const j = t / P.n_cosets;
  uint32_t const c = (uint32_t)(t % P.n_cosets);
  if (j >= D) return;
  W const mask = (W)P.mask;
  W const y = coset_apply<W>((W)reps[j], P, c);
  uint32_t const pc = P.coset_phase[c];
  if (P.rows == 1) {
    // The images with source row k at the top form one class under row
    // rotations and inversion; its smallest member has the smallest rotation
    // of row k (or of its inverse) on top, so only the rotations in the row
    // tables are built, and the class writes one entry.
    uint32_t const rm = (uint32_t)P.row_mask;
    for (uint32_t k = 0; k < P.n_rows; ++k) {
      uint32_t const rv = (uint32_t)(y >> (k * P.row_bits)) & rm;
      uint32_t M = RT.min[rv];
      if (P.inv) {
        uint32_t const b = RT.min[rv ^ rm];
        M = b < M ? b : M;
      }
      W best = mask;
      uint32_t br = 0, binv = 0;
      for (uint32_t inv = 0; inv <= (P.inv ? 1u : 0u); ++inv) {
        uint32_t const v = inv ? (rv ^ rm) : rv;
        if (RT.min[v] != M) continue;
        uint32_t set = RT.set[v];
        while (set) {
          uint32_t const r = (uint32_t)__builtin_ctz_sed(set);
          set &= set - 1;
          W const z = cand_image<W>(y, mask, P, k, r, inv);
          if (z < best) {
            best = z;
            br = r;
            binv = inv;
          }
        }
      }
      uint32_t const tt = k + 1 == P.n_rows ? 0u : k + 1;
      uint64_t ph = (uint64_t)pc + (uint64_t)P.rot_exp[br] * P.rot_phase + (uint64_t)P.sh_exp[tt] * P.shift_phase;
      if (binv) ph += P.inv_phase;
      uint64_t const k0 = table_index((uint64_t)best, hw, RK, bin, RI);
      if (k0 < space) table[k0] = (uint32_t)j | ((ph % P.L) ? kTabSign : 0u);
      else *error = 1;
    }
    return;
  }
  for (uint32_t h = 0; h < P.n_h; ++h) {
    W const z = shift_apply<W>(y, P.h_mask + (uint64_t)h * P.n_terms, P.h_rot + (uint64_t)h * P.n_terms, P.n_terms);
    uint32_t const ph = add_phase(pc, P.h_phase[h], P.L);
    W w = z;
    uint32_t pw = ph;
    if (P.inv && ((uint64_t)z >> (P.n_bits - 1)) & 1u) {
      w = (W)(~z & mask);
      pw = add_phase(ph, P.inv_phase, P.L);
    }
    uint64_t const k0 = table_index((uint64_t)w, hw, RK, bin, RI);
    if (k0 < space) table[k0] = (uint32_t)j | (pw ? kTabSign : 0u);
    else *error = 1;
  }
}

// The stream form from the orbit table: one warp per SELL-32 slice, one row
// per lane, elements in the canonical order of walk_row; same entries, codes,
// diagonal and row classes as k_record.
template <class W, bool Real>
__global__ void __launch_bounds__(256) k_record_table(__grid_constant__ const PlanView P, IndexView I, TermsView T, CodeView C, uint32_t const* __restrict__ weights,
                                                      uint64_t n_slices, uint64_t const* __restrict__ slice_ptr,
                                                      uint32_t col_bits, bool packed, uint32_t* __restrict__ entries,
                                                      uint16_t* __restrict__ codes, void* __restrict__ diag,
                                                      uint8_t* __restrict__ row_class, uint32_t const* __restrict__ table,
                                                      int hw, uint64_t const* __restrict__ binom, uint64_t space,
                                                      int* __restrict__ error, bool inv_half, bool inv_sign,
                                                      uint32_t n_bits, uint64_t word_mask,
                                                      uint64_t const* __restrict__ rank_tab, uint32_t rank_words,
                                                      uint32_t n_chunks, uint32_t wp1, RowIndex RI) {
  extern __shared__ uint64_t dyn_rank[];
  __shared__ uint16_t rows_s[2048];
  uint64_t const* const bin = dyn_rank;
  RankTab const RK = stage_rank(binom, rank_tab, rank_words, n_chunks, wp1, dyn_rank);
  RowTab const RT = stage_rows(P, rows_s);
  __syncthreads();
  uint32_t const lane = threadIdx.x & 31;
  uint64_t const s = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (s >= n_slices) return;  // warp-uniform
  uint64_t const i = s * 32 + lane;
  uint64_t const base = slice_ptr[s];
  uint32_t const width = (uint32_t)((slice_ptr[s + 1] - base) >> 5);
  uint32_t count = 0;
  if (i < I.D) {
    uint64_t const r = I.reps[i];
    walk_row(r, T, [&](uint32_t e, uint64_t st, uint32_t vid) {
      // terms that change the Hamming weight leave the sector: dropped, as
      // the canonicalising path drops them (their orbit is not in the basis)
      uint32_t v = kNull;
      if (hw < 0 || __popcll(st) == hw) {
        uint64_t w = st;
        bool flip = false;
        if (P.rows == 1) {
          uint32_t kp;
          w = (uint64_t)rows_rot_min<W>((W)st, P, RT, &kp);
          flip = kp != 0;
        } else if (inv_half && ((st >> (n_bits - 1)) & 1u)) {
          w = ~st & word_mask;
          flip = inv_sign;
        }
        uint64_t const k = table_index(w, hw, RK, bin, RI);
        if (k < space) v = __ldg(table + k);
        else *error = 1;
        if (flip && v != kNull) v ^= kTabSign;
      }
      uint32_t ent = kNull, code = 0;
      if (v != kNull) {
        uint32_t const jj = v & ~kTabSign;
        code = element_code(vid, (v & kTabSign) ? 1u : 0u, weights[jj], C);
        ent = packed ? (jj | (code << col_bits)) : jj;
      }
      entries[base + (uint64_t)e * 32 + lane] = ent;
      if (!packed) codes[base + (uint64_t)e * 32 + lane] = (uint16_t)code;
      count = e + 1;
    });
    if (Real) {
      static_cast<double*>(diag)[i] = row_diag<double>(r, T);
    } else {
      cplx const d = row_diag<cplx>(r, T);
      static_cast<double2*>(diag)[i] = make_double2(d.re, d.im);
    }
    row_class[i] = (uint8_t)divisor_class(weights[i], C);
  }
  for (uint32_t e = count; e < width; ++e) {
    entries[base + (uint64_t)e * 32 + lane] = kNull;
    if (!packed) codes[base + (uint64_t)e * 32 + lane] = 0;
  }
}

}  // namespace


namespace {

OperatorTables* tables_of(OperatorData const& op) { return op.tables.get(); }

int build_tables(OperatorData& op) {
  if (tables_of(op)) return LS_SUCCESS;
  BasisData const& b = *op.basis;
  auto t = std::make_unique<OperatorTables>();
  auto div = divisors_of(b.plan.group_order);
  uint32_t const n_div = (uint32_t)div.size();
  bool const real_phase = characters_real(b);
  uint32_t const n_ph = real_phase ? 2u : b.plan.L;
  uint32_t const n_val = (uint32_t)(op.off_values.size() / 2);
  uint64_t const n_codes = (uint64_t)std::max(1u, n_val) * n_ph * n_div;
  if (n_codes > kMaxCodes)
    return fail(LS_SYSTEM_ERROR, "too many distinct matrix-element codes (" + std::to_string(n_codes) + ")");
  std::vector<double> tr, tc;
  tc.resize(2 * n_codes, 0.0);
  for (uint32_t v = 0; v < std::max(1u, n_val); ++v)
    for (uint32_t p = 0; p < n_ph; ++p)
      for (uint32_t d = 0; d < n_div; ++d) {
        double cre = n_val ? op.off_values[2 * v] : 0.0, cim = n_val ? op.off_values[2 * v + 1] : 0.0;
        double xr, xi;
        root_of_unity(real_phase ? (p ? b.plan.L / 2 : 0) : p, b.plan.L, xr, xi);
        double const sq = std::sqrt((double)div[d]);
        uint64_t const code = ((uint64_t)v * n_ph + p) * n_div + d;
        tc[2 * code] = (cre * xr - cim * xi) * sq;
        tc[2 * code + 1] = (cre * xi + cim * xr) * sq;
      }
  std::vector<double> inv(n_div);
  for (uint32_t d = 0; d < n_div; ++d) inv[d] = 1.0 / std::sqrt((double)div[d]);
  if (int st = t->divisors.allocate(n_div * 4)) return st;
  if (int st = t->inv_sqrt_s.allocate(n_div * 8)) return st;
  SED_TRY_CUDA(cudaMemcpy(t->divisors.ptr, div.data(), n_div * 4, cudaMemcpyHostToDevice));
  SED_TRY_CUDA(cudaMemcpy(t->inv_sqrt_s.ptr, inv.data(), n_div * 8, cudaMemcpyHostToDevice));
  if (int st = t->table_c.allocate(n_codes * 16)) return st;
  SED_TRY_CUDA(cudaMemcpy(t->table_c.ptr, tc.data(), n_codes * 16, cudaMemcpyHostToDevice));
  if (op.is_real) {
    tr.resize(n_codes);
    for (uint64_t c = 0; c < n_codes; ++c) tr[c] = tc[2 * c];
    if (int st = t->table.allocate(n_codes * 8)) return st;
    SED_TRY_CUDA(cudaMemcpy(t->table.ptr, tr.data(), n_codes * 8, cudaMemcpyHostToDevice));
  }
  t->code.divisors = t->divisors.as<uint32_t>();
  t->code.n_div = n_div;
  t->code.n_ph = n_ph;
  t->code.real_phase = real_phase ? 1u : 0u;
  t->n_codes = (uint32_t)n_codes;
  // fixed-point form: real values and characters, few distinct values
  if (op.is_real && real_phase && n_val <= kFixMaxValues && n_div <= kFixMaxClasses && n_codes <= 16384 &&
      op.row_bound < (1ull << 40)) {
    std::vector<uint8_t> fc(n_codes);
    for (uint32_t v = 0; v < std::max(1u, n_val); ++v)
      for (uint32_t p = 0; p < n_ph; ++p)
        for (uint32_t d = 0; d < n_div; ++d) fc[((uint64_t)v * n_ph + p) * n_div + d] = (uint8_t)(v << 1 | p);
    std::vector<double> sq(n_div);
    for (uint32_t d = 0; d < n_div; ++d) sq[d] = std::sqrt((double)div[d]);
    if (int st = t->fix_code.allocate(n_codes)) return st;
    if (int st = t->fix_sqrt_s.allocate(n_div * 8)) return st;
    SED_TRY_CUDA(cudaMemcpy(t->fix_code.ptr, fc.data(), n_codes, cudaMemcpyHostToDevice));
    SED_TRY_CUDA(cudaMemcpy(t->fix_sqrt_s.ptr, sq.data(), n_div * 8, cudaMemcpyHostToDevice));
    t->fix.code = t->fix_code.as<uint8_t>();
    t->fix.sqrt_s = t->fix_sqrt_s.as<double>();
    t->fix.n_codes = (uint32_t)n_codes;
    t->fix.n_div = n_div;
    // (row count) x sqrt(S_max), rounded up by a margin far above the
    // rounding of this product
    t->fix.bound = (double)std::max<uint64_t>(1, op.row_bound) * sq[n_div - 1] * (1.0 + 1e-9);
    t->fix.sqrt_s_max = sq[n_div - 1] * (1.0 + 1e-9);
    for (uint32_t v = 0; v < kFixMaxValues; ++v) t->fix.c[v] = v < n_val ? op.off_values[2 * v] : 0.0;
    t->fix_nv = n_val <= 1 ? 1u : (n_val <= 2 ? 2u : 4u);
    t->fix_ok = true;
  }
  op.tables = std::move(t);
  return LS_SUCCESS;
}

int elem_size(int dtype) {
  switch (dtype) {
    case 0: return 4;
    case 1: return 8;
    case 2: return 8;
    case 3: return 16;
    default: return 0;
  }
}

bool is_device_pointer(void const* p) {
  cudaPointerAttributes a{};
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

int wait_for_caller(std::initializer_list<void const*> buffers) {
  for (void const* p : buffers)
    if (p && is_device_pointer(p)) {
      SED_TRY_CUDA(cudaDeviceSynchronize());
      return LS_SUCCESS;
    }
  return LS_SUCCESS;
}

OperatorData::~OperatorData() {
  tables.reset();
  if (fix_event) {
    ScopedDevice dev(basis ? basis->device : -1);
    cudaEventDestroy(fix_event);
  }
  if (cuda_stream) {
    ScopedDevice dev(basis ? basis->device : -1);
    cudaStreamDestroy(cuda_stream);
  }
}

int operator_upload_terms(OperatorData& op) {
  if (op.term_buf.ptr) return LS_SUCCESS;
  unsigned const n_terms = (unsigned)op.terms.size();
  // Distinct off-diagonal values (exact bitwise dedup).
  op.off_values.clear();
  std::vector<uint32_t> tuple_term, tuple_sites;
  std::vector<double> diag((size_t)std::max(1u, n_terms) * 16 * 2, 0.0);
  std::vector<uint8_t> n_off((size_t)std::max(1u, n_terms) * 16, 0), off_col((size_t)std::max(1u, n_terms) * 256, 0);
  std::vector<uint16_t> off_vid((size_t)std::max(1u, n_terms) * 256, 0);
  for (unsigned t = 0; t < n_terms; ++t) {
    InteractionData const& term = op.terms[t];
    unsigned const dim = 1u << term.k;
    for (unsigned a = 0; a < dim; ++a)
      for (unsigned a2 = 0; a2 < dim; ++a2) {
        double const re = term.matrix[2 * (a * dim + a2)], im = term.matrix[2 * (a * dim + a2) + 1];
        if (a2 == a) {
          diag[2 * (t * 16 + a)] = re;
          diag[2 * (t * 16 + a) + 1] = im;
          continue;
        }
        if (re == 0.0 && im == 0.0) continue;
        size_t vid = op.off_values.size() / 2;
        for (size_t q = 0; q < op.off_values.size() / 2; ++q)
          if (std::memcmp(&op.off_values[2 * q], &re, 8) == 0 &&
              std::memcmp(&op.off_values[2 * q + 1], &im, 8) == 0) {
            vid = q;
            break;
          }
        if (vid == op.off_values.size() / 2) {
          op.off_values.push_back(re);
          op.off_values.push_back(im);
        }
        unsigned const q = n_off[t * 16 + a]++;
        off_col[(t * 16 + a) * 16 + q] = (uint8_t)a2;
        off_vid[(t * 16 + a) * 16 + q] = (uint16_t)vid;
      }
    size_t const n_tuples = term.sites.size() / term.k;
    unsigned most = 0;
    for (unsigned a = 0; a < dim; ++a) most = std::max<unsigned>(most, n_off[t * 16 + a]);
    op.row_bound += (uint64_t)most * n_tuples;
    for (size_t u = 0; u < n_tuples; ++u) {
      uint32_t packed = 0;
      for (unsigned m = 0; m < term.k; ++m) packed |= (uint32_t)term.sites[u * term.k + m] << (8 * m);
      tuple_term.push_back(t | (term.k << 16));
      tuple_sites.push_back(packed);
    }
  }
  if (op.off_values.size() / 2 > 4096)
    return fail(LS_SYSTEM_ERROR, "too many distinct off-diagonal matrix values");
  size_t const nt = std::max<size_t>(1, tuple_term.size());
  auto align = [](size_t v) { return (v + 15) & ~(size_t)15; };
  size_t const sz_tt = align(nt * 4), sz_ts = align(nt * 4), sz_dg = align(diag.size() * 8),
               sz_no = align(n_off.size()), sz_oc = align(off_col.size()),
               sz_ov = align(off_vid.size() * 2),
               sz_val = align(std::max<size_t>(2, op.off_values.size()) * 8);
  size_t const total = sz_tt + sz_ts + sz_dg + sz_no + sz_oc + sz_ov + sz_val;
  std::vector<uint8_t> host(total, 0);
  size_t off = 0;
  auto put = [&](void const* src, size_t n, size_t sz) {
    if (n) std::memcpy(host.data() + off, src, n);
    size_t const at = off;
    off += sz;
    return at;
  };
  size_t const o_tt = put(tuple_term.data(), tuple_term.size() * 4, sz_tt);
  size_t const o_ts = put(tuple_sites.data(), tuple_sites.size() * 4, sz_ts);
  size_t const o_dg = put(diag.data(), diag.size() * 8, sz_dg);
  size_t const o_no = put(n_off.data(), n_off.size(), sz_no);
  size_t const o_oc = put(off_col.data(), off_col.size(), sz_oc);
  size_t const o_ov = put(off_vid.data(), off_vid.size() * 2, sz_ov);
  size_t const o_val = put(op.off_values.data(), op.off_values.size() * 8, sz_val);
  ScopedDevice dev(op.basis->device);
  if (int st = op.term_buf.allocate(total)) return st;
  SED_TRY_CUDA(cudaMemcpy(op.term_buf.ptr, host.data(), total, cudaMemcpyHostToDevice));
  uint8_t* base = op.term_buf.as<uint8_t>();
  op.terms_dev.n_tuples = (uint32_t)tuple_term.size();
  op.terms_dev.tuple_term = (uint32_t const*)(base + o_tt);
  op.terms_dev.tuple_sites = (uint32_t const*)(base + o_ts);
  op.terms_dev.diag = (double const*)(base + o_dg);
  op.terms_dev.n_off = base + o_no;
  op.terms_dev.off_col = base + o_oc;
  op.terms_dev.off_vid = (uint16_t const*)(base + o_ov);
  op.terms_dev.off_val = (double const*)(base + o_val);
  return LS_SUCCESS;
}

int operator_ensure_ready(OperatorData& op) {
  BasisData& b = *op.basis;
  if (!b.built) return fail(LS_CACHE_NOT_BUILT, "basis has not been built (call ls_build)");
  ScopedDevice dev(b.device);
  if (!op.cuda_stream) SED_TRY_CUDA(cudaStreamCreateWithFlags(&op.cuda_stream, cudaStreamNonBlocking));
  if (int st = basis_upload_plan(b, op.cuda_stream)) return st;
  if (int st = operator_upload_terms(op)) return st;
  if (int st = build_tables(op)) return st;
  if (int st = fix_reserve(op, 1)) return st;
  return LS_SUCCESS;
}

int g_record_mode = SED_RECORD_AUTO;

uint64_t host_binom(unsigned n, unsigned k) {
  if (k > n) return 0;
  uint64_t c = 1;
  for (unsigned i = 1; i <= k; ++i) c = c * (n - k + i) / i;  // exact: c * (n-k+i) is divisible by i
  return c;
}

StreamView stream_view(OperatorData const& op) {
  StreamForm const& sf = op.stream;
  OperatorTables const& tb = *op.tables;
  StreamView S{};
  S.slice_ptr = sf.slice_ptr.as<uint64_t>();
  S.entries = sf.entries.as<uint32_t>();
  S.codes = sf.values.as<uint16_t>();
  S.diag = sf.diag.ptr;
  S.row_class = sf.row_class.as<uint8_t>();
  S.table = op.is_real ? tb.table.ptr : tb.table_c.ptr;
  S.inv_sqrt_s = tb.inv_sqrt_s.as<double>();
  S.col_bits = sf.col_bits;
  S.n_codes = tb.n_codes;
  return S;
}

int operator_record_stream(OperatorData& op, cudaStream_t stream) {
  if (op.stream.ready) return LS_SUCCESS;
  if (int st = operator_ensure_ready(op)) return st;
  BasisData& b = *op.basis;
  OperatorTables const& tb = *tables_of(op);
  ScopedDevice dev(b.device);
  auto t0 = std::chrono::steady_clock::now();
  uint64_t const D = b.D;
  uint64_t const n_slices = (D + 31) / 32;
  unsigned col_bits = 1;
  while (col_bits < 32 && ((uint64_t)1 << col_bits) < std::max<uint64_t>(D, 2)) ++col_bits;
  if (D >= ((uint64_t)1 << 32) - 1)
    return fail(LS_OUT_OF_MEMORY, "stream form supports fewer than 2^32 - 1 representatives");
  unsigned code_bits = 0;
  while (((uint64_t)1 << code_bits) < tb.n_codes) ++code_bits;
  bool const packed = col_bits + code_bits <= 31;  // kNull stays unrepresentable
  StreamForm& sf = op.stream;
  sf = StreamForm{};
  DeviceBuffer elements, maxw;
  if (int st = sf.slice_ptr.allocate((n_slices + 1) * 8)) return st;
  if (int st = elements.allocate((n_slices + 1) * 8)) return st;
  if (int st = maxw.allocate(16)) return st;
  SED_TRY_CUDA(cudaMemsetAsync(maxw.ptr, 0, 4, stream));
  unsigned const grid = (unsigned)((n_slices * 32 + kBlock - 1) / kBlock);
  if (n_slices) {
    { k_count<<<grid, kBlock, 0, stream>>>(b.reps.as<uint64_t>(), D, op.terms_dev, n_slices,
                                         sf.slice_ptr.as<uint64_t>(), elements.as<uint64_t>(), maxw.as<unsigned>()); note_launches(1); }
    SED_TRY_CUDA(cudaGetLastError());
  }
  { k_scan_u64<<<1, 1024, 0, stream>>>(sf.slice_ptr.as<uint64_t>(), n_slices); note_launches(1); }
  { k_scan_u64<<<1, 1024, 0, stream>>>(elements.as<uint64_t>(), n_slices); note_launches(1); }
  SED_TRY_CUDA(cudaGetLastError());
  uint64_t n_entries = 0, n_elements = 0;
  unsigned max_width = 0;
  SED_TRY_CUDA(cudaMemcpyAsync(&n_entries, sf.slice_ptr.as<uint64_t>() + n_slices, 8, cudaMemcpyDeviceToHost, stream));
  SED_TRY_CUDA(cudaMemcpyAsync(&n_elements, elements.as<uint64_t>() + n_slices, 8, cudaMemcpyDeviceToHost, stream));
  SED_TRY_CUDA(cudaMemcpyAsync(&max_width, maxw.ptr, 4, cudaMemcpyDeviceToHost, stream));
  SED_TRY_CUDA(cudaStreamSynchronize(stream));
  size_t free_b = 0, total_b = 0;
  SED_TRY_CUDA(cudaMemGetInfo(&free_b, &total_b));
  uint64_t const need = n_entries * (packed ? 4 : 6) + D * (op.is_real ? 9 : 17);
  if (need > free_b)
    return fail(LS_OUT_OF_MEMORY, "stream form needs " + std::to_string(need) + " bytes, " +
                                      std::to_string(free_b) + " free");
  if (int st = sf.entries.allocate(std::max<uint64_t>(1, n_entries) * 4)) return st;
  if (!packed)
    if (int st = sf.values.allocate(std::max<uint64_t>(1, n_entries) * 2)) return st;
  if (int st = sf.diag.allocate(std::max<uint64_t>(1, D) * (op.is_real ? 8 : 16))) return st;
  if (int st = sf.row_class.allocate(std::max<uint64_t>(1, D))) return st;
  // orbit-table path: real characters, a weight class small enough to tabulate
  uint64_t space = 0;
  bool use_table = false;
  // row-structured plans: one segment per possible top row (see table_index)
  std::vector<uint64_t> seg_off;
  if (n_slices && g_record_mode != SED_RECORD_CANONICALISE && characters_real(b) && D < kTabSign) {
    bool const half = b.plan.inv != 0;
    if (b.hw >= 0 && b.hw <= 32 && b.n <= 64) space = host_binom(half ? b.n - 1 : b.n, (unsigned)b.hw);
    else if (b.hw < 0 && b.n <= 34) space = (uint64_t)1 << (half ? b.n - 1 : b.n);
    if (space && b.plan.rows == 1 && b.plan.row_bits <= 10 && b.n > b.plan.row_bits) {
      unsigned const B = b.plan.row_bits, L = b.n - B;
      uint32_t const rm = (1u << B) - 1u;
      uint64_t total = 0;
      seg_off.assign((size_t)1 << B, ~(uint64_t)0);
      for (uint32_t T = 0; T <= rm; ++T) {
        bool ok = b.plan.row_min[T] == T;
        if (b.plan.inv) ok = ok && b.plan.row_min[T ^ rm] >= T;
        int const need = b.hw - __builtin_popcount(T);
        uint64_t const cnt = b.hw < 0 ? ((uint64_t)1 << L)
                                      : (need < 0 || (unsigned)need > L ? 0 : host_binom(L, (unsigned)need));
        if (ok) {
          seg_off[T] = total;
          total += cnt;
        }
      }
      space = total;
    }
    size_t fr = 0, tt = 0;
    SED_TRY_CUDA(cudaMemGetInfo(&fr, &tt));
    use_table = space > 0 && space * 4 <= fr / 5 * 2;
  }
  if (use_table) {
    DeviceBuffer table;
    struct TableGuard {
      DeviceBuffer& b;
      ~TableGuard() { krylov_give(b); }
    } table_guard{table};
    DeviceBuffer err;
    if (int st = err.allocate(16)) return st;
    if (int st = krylov_take(space * 4, table)) return st;
    DeviceBuffer seg_buf;
    RowIndex RI{nullptr, 0, 0};
    if (!seg_off.empty()) {
      if (int st = seg_buf.allocate(seg_off.size() * 8)) return st;
      SED_TRY_CUDA(cudaMemcpyAsync(seg_buf.ptr, seg_off.data(), seg_off.size() * 8, cudaMemcpyHostToDevice, stream));
      unsigned const L = b.n - b.plan.row_bits;
      RI = RowIndex{seg_buf.as<uint64_t>(), ((uint64_t)1 << L) - 1, L};
    }
    SED_TRY_CUDA(cudaMemsetAsync(table.ptr, 0xFF, space * 4, stream));
    SED_TRY_CUDA(cudaMemsetAsync(err.ptr, 0, 16, stream));
    // chunked rank table (6-bit chunks) when it fits in 96 KB of shared memory
    uint32_t n_chunks = 0, wp1 = 0, rank_words = 0;
    DeviceBuffer rank_buf;
    if (b.hw >= 0) {
      n_chunks = (b.n + 5) / 6;
      wp1 = (uint32_t)b.hw + 1;
      uint64_t const words = (uint64_t)n_chunks * wp1 * 64;
      if (words * 8 <= 96 * 1024) {
        std::vector<uint64_t> R(words, 0);
        for (uint32_t c = 0; c < n_chunks; ++c)
          for (uint32_t m = 0; m < wp1; ++m)
            for (uint32_t v = 0; v < 64; ++v) {
              uint64_t acc = 0;
              uint32_t i = 0;
              for (uint32_t q = 0; q < 6; ++q)
                if ((v >> q) & 1u) {
                  ++i;
                  uint32_t const p = 6 * c + q;
                  if (p < 64) acc += host_binom(p, m + i);
                }
              R[((size_t)c * wp1 + m) * 64 + v] = acc;
            }
        if (int st = rank_buf.allocate(words * 8)) return st;
        SED_TRY_CUDA(cudaMemcpyAsync(rank_buf.ptr, R.data(), words * 8, cudaMemcpyHostToDevice, stream));
        SED_TRY_CUDA(cudaStreamSynchronize(stream));
        rank_words = (uint32_t)words;
      }
    }
    size_t const dsmem = rank_words ? (size_t)rank_words * 8 : (size_t)64 * 33 * 8;
    bool const wide = b.plan.n_bits > 32;
    uint64_t const threads = D * b.plan.n_cosets;
    unsigned const sgrid = (unsigned)((threads + 255) / 256);
    uint64_t const* rtab = rank_words ? rank_buf.as<uint64_t>() : nullptr;
    if (wide) {
      cudaFuncSetAttribute(k_orbit_scatter<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem);
      { k_orbit_scatter<uint64_t><<<sgrid, 256, dsmem, stream>>>(b.plan_dev, b.reps.as<uint64_t>(), D, b.hw, b.binom.as<uint64_t>(), table.as<uint32_t>(), space, err.as<int>(), rtab, rank_words, n_chunks, wp1, RI); note_launches(1); }
    } else {
      cudaFuncSetAttribute(k_orbit_scatter<uint32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem);
      { k_orbit_scatter<uint32_t><<<sgrid, 256, dsmem, stream>>>(b.plan_dev, b.reps.as<uint64_t>(), D, b.hw, b.binom.as<uint64_t>(), table.as<uint32_t>(), space, err.as<int>(), rtab, rank_words, n_chunks, wp1, RI); note_launches(1); }
    }
    SED_TRY_CUDA(cudaGetLastError());
    IndexView const I = b.index_view();
    unsigned const rgrid = (unsigned)((n_slices * 32 + 255) / 256);
    auto rec = [&](auto w_tag, auto real_tag) {
      using W = decltype(w_tag);
      constexpr bool R = decltype(real_tag)::value;
      cudaFuncSetAttribute(k_record_table<W, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem);
      { k_record_table<W, R><<<rgrid, 256, dsmem, stream>>>(b.plan_dev, I, op.terms_dev, tb.code, b.weights.as<uint32_t>(), n_slices, sf.slice_ptr.as<uint64_t>(), col_bits, packed, sf.entries.as<uint32_t>(), sf.values.as<uint16_t>(), sf.diag.ptr, sf.row_class.as<uint8_t>(), table.as<uint32_t>(), b.hw, b.binom.as<uint64_t>(), space, err.as<int>(), b.plan.inv != 0, b.plan.inv_phase != 0, b.plan.n_bits, b.plan.mask, rtab, rank_words, n_chunks, wp1, RI); note_launches(1); }
    };
    if (wide) {
      if (op.is_real) rec(uint64_t{}, std::true_type{});
      else rec(uint64_t{}, std::false_type{});
    } else {
      if (op.is_real) rec(uint32_t{}, std::true_type{});
      else rec(uint32_t{}, std::false_type{});
    }
    SED_TRY_CUDA(cudaGetLastError());
    int herr = 0;
    SED_TRY_CUDA(cudaMemcpyAsync(&herr, err.ptr, 4, cudaMemcpyDeviceToHost, stream));
    SED_TRY_CUDA(cudaStreamSynchronize(stream));
    if (herr) return fail(LS_SYSTEM_ERROR, "orbit table: a word outside the weight class (internal error)");
  } else if (n_slices) {
    bool const wide = b.plan.n_bits > 32;
    IndexView const I = b.index_view();
    auto launch = [&](auto w_tag, auto real_tag) {

      using W = decltype(w_tag);
      constexpr bool R = decltype(real_tag)::value;
      // descriptor slots for the widest slice (wider slices than kRecMaxElems
      // take the row-per-lane path), coset images for this plan's cosets
      unsigned const me = std::max(1u, std::min(max_width, kRecMaxElems));
      unsigned const nc = std::max(1u, std::min<unsigned>(b.plan.n_cosets, SED_PARAM_COSETS));
      size_t const smem = record_smem_bytes(me, nc);
      cudaFuncSetAttribute(k_record<W, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      { k_record<W, R><<<(unsigned)((n_slices + kRecWarps - 1) / kRecWarps), kRecWarps * 32, smem, stream>>>(
          b.plan_dev, I, op.terms_dev, tb.code, b.weights.as<uint32_t>(), n_slices,
          sf.slice_ptr.as<uint64_t>(), col_bits, packed, sf.entries.as<uint32_t>(),
          sf.values.as<uint16_t>(), sf.diag.ptr, sf.row_class.as<uint8_t>(), me, nc); note_launches(1); }
    };
    if (wide) {
      if (op.is_real) launch(uint64_t{}, std::true_type{});
      else launch(uint64_t{}, std::false_type{});
    } else {
      if (op.is_real) launch(uint32_t{}, std::true_type{});
      else launch(uint32_t{}, std::false_type{});
    }
    SED_TRY_CUDA(cudaGetLastError());
  }
  SED_TRY_CUDA(cudaStreamSynchronize(stream));
  sf.packed = packed;
  sf.col_bits = col_bits;
  sf.n_slices = n_slices;
  sf.n_entries = n_entries;
  sf.n_elements = n_elements;
  sf.n_codes = tb.n_codes;
  sf.ready = true;
  sf.orbit_table = use_table;
  sf.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (logging_enabled())
    log_line("stream form: %llu elements, %llu slots (%s), %.1f MB, %.3f s (%s)",
             (unsigned long long)n_elements, (unsigned long long)n_entries,
             packed ? "packed" : "split", sf.bytes() / 1e6, sf.seconds,
             use_table ? "orbit table" : "canonicalisation");
  return LS_SUCCESS;
}

int fix_reserve(OperatorData& op, uint32_t cols) {
  if (!op.tables || !op.tables->fix_ok || op.fix_cols >= cols) return LS_SUCCESS;
  uint64_t const D = std::max<uint64_t>(1, op.basis->D);
  if (int st = op.fix_u.allocate(D * cols * 8)) return st;
  if (int st = op.fix_slots.allocate((size_t)cols * 16)) return st;
  if (!op.fix_event) SED_TRY_CUDA(cudaEventCreateWithFlags(&op.fix_event, cudaEventDisableTiming));
  op.fix_cols = cols;
  return LS_SUCCESS;
}

int fix_wait(OperatorData& op) {
  if (op.fix_event && op.fix_event_recorded) SED_TRY_CUDA(cudaEventSynchronize(op.fix_event));
  return LS_SUCCESS;
}

namespace {

template <int NV>
void launch_spmv_fix(OperatorData& op, StreamView const& S, double const* x, int64_t const* u, int64_t const* F,
                     double* y, cudaStream_t stream, Indirect ind) {
  StreamForm const& sf = op.stream;
  OperatorTables const& tb = *op.tables;
  unsigned const grid = (unsigned)((sf.n_slices * 32 + kBlock - 1) / kBlock);
  size_t const smem = (size_t)tb.fix.n_div * NV * 8 + tb.fix.n_codes;
  if (sf.packed) k_spmv_fix<true, NV><<<grid, kBlock, smem, stream>>>(S, tb.fix, op.basis->D, x, u, F, y, ind);
  else k_spmv_fix<false, NV><<<grid, kBlock, smem, stream>>>(S, tb.fix, op.basis->D, x, u, F, y, ind);
  note_launches(1);
}

template <class W, int NV>
void launch_otf_fix(OperatorData& op, double const* x, int64_t const* u, int64_t const* F, double* y,
                    cudaStream_t stream, Indirect ind) {
  BasisData& b = *op.basis;
  OperatorTables const& tb = *op.tables;
  unsigned const grid = (unsigned)((b.D + kBlock - 1) / kBlock);
  k_otf_fix<W, NV><<<grid, kBlock, 0, stream>>>(b.plan_dev, b.index_view(), op.terms_dev, tb.code,
                                                b.weights.as<uint32_t>(), tb.fix, tb.inv_sqrt_s.as<double>(), x, u,
                                                F, y, ind);
  note_launches(1);
}

// y = H x in fixed point: max |x|, u = round(sqrt(S) x 2^F), then the SpMV.
// Outside a Krylov graph the shared workspace is ordered across the callers'
// streams by fix_event.
int launch_apply_fix(OperatorData& op, double const* x, double* y, cudaStream_t stream, bool use_stream,
                     Indirect ind) {
  BasisData& b = *op.basis;
  OperatorTables const& tb = *op.tables;
  uint64_t const D = b.D;
  auto* mx = op.fix_slots.as<unsigned long long>();
  auto* F = reinterpret_cast<int64_t*>(mx + op.fix_cols);
  int64_t* u = op.fix_u.as<int64_t>();
  bool const ordered = ind.k == nullptr;
  if (ordered && op.fix_event_recorded) SED_TRY_CUDA(cudaStreamWaitEvent(stream, op.fix_event, 0));
  if (!ind.prescaled) {
    SED_TRY_CUDA(cudaMemsetAsync(mx, 0, 8, stream));
    unsigned const vg = grid_size(D, b.device, 8);
    k_fix_max<<<vg, kBlock, 0, stream>>>(x, 0, D, mx, ind);
    k_fix_convert<<<vg, kBlock, 0, stream>>>(x, 0, D, use_stream ? op.stream.row_class.as<uint8_t>() : nullptr,
                                             b.weights.as<uint32_t>(), tb.code, tb.fix, mx, F, u, D, ind);
    note_launches(2);
  }
  if (use_stream) {
    StreamView const S = stream_view(op);
    switch (tb.fix_nv) {
      case 1: launch_spmv_fix<1>(op, S, x, u, F, y, stream, ind); break;
      case 2: launch_spmv_fix<2>(op, S, x, u, F, y, stream, ind); break;
      default: launch_spmv_fix<4>(op, S, x, u, F, y, stream, ind); break;
    }
  } else if (b.plan.n_bits > 32) {
    switch (tb.fix_nv) {
      case 1: launch_otf_fix<uint64_t, 1>(op, x, u, F, y, stream, ind); break;
      case 2: launch_otf_fix<uint64_t, 2>(op, x, u, F, y, stream, ind); break;
      default: launch_otf_fix<uint64_t, 4>(op, x, u, F, y, stream, ind); break;
    }
  } else {
    switch (tb.fix_nv) {
      case 1: launch_otf_fix<uint32_t, 1>(op, x, u, F, y, stream, ind); break;
      case 2: launch_otf_fix<uint32_t, 2>(op, x, u, F, y, stream, ind); break;
      default: launch_otf_fix<uint32_t, 4>(op, x, u, F, y, stream, ind); break;
    }
  }
  SED_TRY_CUDA(cudaGetLastError());
  if (ordered) {
    SED_TRY_CUDA(cudaEventRecord(op.fix_event, stream));
    op.fix_event_recorded = true;
  }
  return LS_SUCCESS;
}

}  // namespace

bool fix_slots(OperatorData& op, FixSlots* out) {
  if (!op.tables || !op.tables->fix_ok || op.fix_cols < 1 || !op.stream.ready || op.form == SED_FORM_ON_THE_FLY)
    return false;
  auto* mx = op.fix_slots.as<unsigned long long>();
  out->max_bits = mx;
  out->F = reinterpret_cast<int64_t*>(mx + op.fix_cols);
  out->u = op.fix_u.as<int64_t>();
  out->row_class = op.stream.row_class.as<uint8_t>();
  out->view = op.tables->fix;
  return true;
}

int fix_prescale(OperatorData& op, double const* base, Indirect ind, cudaStream_t stream) {
  FixSlots fs;
  if (!fix_slots(op, &fs)) return fail(LS_SYSTEM_ERROR, "fix_prescale: the operator has no fixed-point form");
  BasisData& b = *op.basis;
  SED_TRY_CUDA(cudaMemsetAsync(fs.max_bits, 0, 8, stream));
  unsigned const vg = grid_size(b.D, b.device, 8);
  k_fix_max<<<vg, kBlock, 0, stream>>>(base, 0, b.D, fs.max_bits, ind);
  k_fix_convert<<<vg, kBlock, 0, stream>>>(base, 0, b.D, fs.row_class, b.weights.as<uint32_t>(), op.tables->code,
                                           fs.view, fs.max_bits, fs.F, fs.u, b.D, ind);
  note_launches(2);
  SED_TRY_CUDA(cudaGetLastError());
  return LS_SUCCESS;
}

namespace {

template <class X>
int launch_apply(OperatorData& op, X const* x, X* y, cudaStream_t stream, bool use_stream,
                 Indirect ind) {
  BasisData& b = *op.basis;
  OperatorTables const& tb = *tables_of(op);
  if constexpr (std::is_same<X, double>::value)
    if (tb.fix_ok && op.fix_cols >= 1) return launch_apply_fix(op, x, y, stream, use_stream, ind);
  using V = typename Store<X>::V;
  constexpr bool complex_storage = std::is_same<V, cplx>::value;
  uint64_t const D = b.D;
  if (D == 0) return LS_SUCCESS;
  bool const real_tab = op.is_real;  // real table exists
  if (use_stream) {
    StreamForm const& sf = op.stream;
    StreamView const S = stream_view(op);
    unsigned const grid = (unsigned)((sf.n_slices * 32 + kBlock - 1) / kBlock);
    size_t const smem = std::min<size_t>(32768, (size_t)tb.n_codes * (real_tab ? 8 : 16));
    if (real_tab) {
      if (sf.packed) { k_spmv<X, true, true><<<grid, kBlock, smem, stream>>>(S, D, x, y, ind); note_launches(1); }
      else { k_spmv<X, true, false><<<grid, kBlock, smem, stream>>>(S, D, x, y, ind); note_launches(1); }
    } else {
      if constexpr (complex_storage) {
        if (sf.packed) { k_spmv<X, false, true><<<grid, kBlock, smem, stream>>>(S, D, x, y, ind); note_launches(1); }
        else { k_spmv<X, false, false><<<grid, kBlock, smem, stream>>>(S, D, x, y, ind); note_launches(1); }
      } else {
        return fail(LS_OPERATOR_IS_COMPLEX, "complex operator applied to real vectors");
      }
    }
  } else {
    IndexView const I = b.index_view();
    unsigned const grid = (unsigned)((D + kBlock - 1) / kBlock);
    void const* table = real_tab ? tb.table.ptr : tb.table_c.ptr;
    bool const wide = b.plan.n_bits > 32;
    if (real_tab) {
      if (wide)
        { k_otf<uint64_t, X, true><<<grid, kBlock, 0, stream>>>(b.plan_dev, I, op.terms_dev, tb.code,
                                                              b.weights.as<uint32_t>(), table,
                                                              tb.inv_sqrt_s.as<double>(), x, y, ind); note_launches(1); }
      else
        { k_otf<uint32_t, X, true><<<grid, kBlock, 0, stream>>>(b.plan_dev, I, op.terms_dev, tb.code,
                                                              b.weights.as<uint32_t>(), table,
                                                              tb.inv_sqrt_s.as<double>(), x, y, ind); note_launches(1); }
    } else {
      if constexpr (complex_storage) {
        if (wide)
          { k_otf<uint64_t, X, false><<<grid, kBlock, 0, stream>>>(b.plan_dev, I, op.terms_dev, tb.code,
                                                                 b.weights.as<uint32_t>(), table,
                                                                 tb.inv_sqrt_s.as<double>(), x, y, ind); note_launches(1); }
        else
          { k_otf<uint32_t, X, false><<<grid, kBlock, 0, stream>>>(b.plan_dev, I, op.terms_dev, tb.code,
                                                                 b.weights.as<uint32_t>(), table,
                                                                 tb.inv_sqrt_s.as<double>(), x, y, ind); note_launches(1); }
      } else {
        return fail(LS_OPERATOR_IS_COMPLEX, "complex operator applied to real vectors");
      }
    }
  }
  SED_TRY_CUDA(cudaGetLastError());
  return LS_SUCCESS;
}

}  // namespace

namespace {

template <class X, bool R, bool Pk>
void launch_block_k(unsigned K, StreamView const& S, uint64_t D, X const* x, uint64_t ldx, X* y, uint64_t ldy,
                    unsigned grid, size_t smem, cudaStream_t stream) {
  switch (K) {
    case 16: { k_spmv_block<X, R, Pk, 16><<<grid, kBlock, smem, stream>>>(S, D, x, ldx, y, ldy); note_launches(1); } break;
    case 8: { k_spmv_block<X, R, Pk, 8><<<grid, kBlock, smem, stream>>>(S, D, x, ldx, y, ldy); note_launches(1); } break;
    case 4: { k_spmv_block<X, R, Pk, 4><<<grid, kBlock, smem, stream>>>(S, D, x, ldx, y, ldy); note_launches(1); } break;
    default: { k_spmv_block<X, R, Pk, 2><<<grid, kBlock, smem, stream>>>(S, D, x, ldx, y, ldy); note_launches(1); } break;
  }
}

template <int NV, bool Pk>
void launch_block_fix_k(unsigned K, StreamView const& S, FixView const& fv, uint64_t D, double const* x, uint64_t ldx,
                        int64_t const* u, int64_t const* F, double* y, uint64_t ldy, unsigned grid, size_t smem,
                        cudaStream_t stream) {
  switch (K) {
    case 16: k_spmv_block_fix<Pk, NV, 16><<<grid, kBlock, smem, stream>>>(S, fv, D, x, ldx, u, F, y, ldy); break;
    case 8: k_spmv_block_fix<Pk, NV, 8><<<grid, kBlock, smem, stream>>>(S, fv, D, x, ldx, u, F, y, ldy); break;
    case 4: k_spmv_block_fix<Pk, NV, 4><<<grid, kBlock, smem, stream>>>(S, fv, D, x, ldx, u, F, y, ldy); break;
    default: k_spmv_block_fix<Pk, NV, 2><<<grid, kBlock, smem, stream>>>(S, fv, D, x, ldx, u, F, y, ldy); break;
  }
  note_launches(1);
}

// K columns in fixed point (the same per-column sums as launch_apply_fix).
int launch_block_fix(OperatorData& op, unsigned K, double const* x, uint64_t ldx, double* y, uint64_t ldy,
                     cudaStream_t stream) {
  if (int st = fix_reserve(op, K)) return st;
  BasisData& b = *op.basis;
  OperatorTables const& tb = *op.tables;
  StreamForm const& sf = op.stream;
  uint64_t const D = b.D;
  auto* mx = op.fix_slots.as<unsigned long long>();
  auto* F = reinterpret_cast<int64_t*>(mx + op.fix_cols);
  int64_t* u = op.fix_u.as<int64_t>();
  if (op.fix_event_recorded) SED_TRY_CUDA(cudaStreamWaitEvent(stream, op.fix_event, 0));
  SED_TRY_CUDA(cudaMemsetAsync(mx, 0, (size_t)K * 8, stream));
  dim3 const vg(grid_size(D, b.device, 8), K);
  k_fix_max<<<vg, kBlock, 0, stream>>>(x, ldx, D, mx, Indirect{});
  k_fix_convert<<<vg, kBlock, 0, stream>>>(x, ldx, D, sf.row_class.as<uint8_t>(), b.weights.as<uint32_t>(), tb.code,
                                           tb.fix, mx, F, u, D, Indirect{});
  note_launches(2);
  StreamView const S = stream_view(op);
  unsigned const grid = (unsigned)((sf.n_slices * 32 + kBlock - 1) / kBlock);
  size_t const smem = (size_t)K * tb.fix.n_div * tb.fix_nv * 8 + tb.fix.n_codes;
  if (smem > 48 * 1024) return fail(LS_SYSTEM_ERROR, "fixed-point block matvec: tables exceed shared memory");
  switch (tb.fix_nv * 2 + (sf.packed ? 1 : 0)) {
    case 3: launch_block_fix_k<1, true>(K, S, tb.fix, D, x, ldx, u, F, y, ldy, grid, smem, stream); break;
    case 2: launch_block_fix_k<1, false>(K, S, tb.fix, D, x, ldx, u, F, y, ldy, grid, smem, stream); break;
    case 5: launch_block_fix_k<2, true>(K, S, tb.fix, D, x, ldx, u, F, y, ldy, grid, smem, stream); break;
    case 4: launch_block_fix_k<2, false>(K, S, tb.fix, D, x, ldx, u, F, y, ldy, grid, smem, stream); break;
    case 9: launch_block_fix_k<4, true>(K, S, tb.fix, D, x, ldx, u, F, y, ldy, grid, smem, stream); break;
    default: launch_block_fix_k<4, false>(K, S, tb.fix, D, x, ldx, u, F, y, ldy, grid, smem, stream); break;
  }
  SED_TRY_CUDA(cudaGetLastError());
  SED_TRY_CUDA(cudaEventRecord(op.fix_event, stream));
  op.fix_event_recorded = true;
  return LS_SUCCESS;
}

template <class X>
int launch_block(OperatorData& op, unsigned K, X const* x, uint64_t ldx, X* y, uint64_t ldy, cudaStream_t stream) {
  if constexpr (std::is_same<X, double>::value)
    if (op.tables->fix_ok) return launch_block_fix(op, K, x, ldx, y, ldy, stream);
  using V = typename Store<X>::V;
  constexpr bool complex_storage = std::is_same<V, cplx>::value;
  StreamForm const& sf = op.stream;
  StreamView const S = stream_view(op);
  OperatorTables const& tb = *op.tables;
  bool const real_tab = op.is_real;
  unsigned const grid = (unsigned)((sf.n_slices * 32 + kBlock - 1) / kBlock);
  size_t const smem = std::min<size_t>(32768, (size_t)tb.n_codes * (real_tab ? 8 : 16));
  uint64_t const D = op.basis->D;
  if (real_tab) {
    if (sf.packed) launch_block_k<X, true, true>(K, S, D, x, ldx, y, ldy, grid, smem, stream);
    else launch_block_k<X, true, false>(K, S, D, x, ldx, y, ldy, grid, smem, stream);
  } else {
    if constexpr (complex_storage) {
      if (sf.packed) launch_block_k<X, false, true>(K, S, D, x, ldx, y, ldy, grid, smem, stream);
      else launch_block_k<X, false, false>(K, S, D, x, ldx, y, ldy, grid, smem, stream);
    } else {
      return fail(LS_OPERATOR_IS_COMPLEX, "complex operator applied to real vectors");
    }
  }
  SED_TRY_CUDA(cudaGetLastError());
  return LS_SUCCESS;
}

}  // namespace

int operator_apply_device(OperatorData& op, int dtype, uint64_t block, void const* x,
                          uint64_t ldx, void* y, uint64_t ldy, cudaStream_t stream, int form) {
  if (int st = operator_ensure_ready(op)) return st;
  if (dtype < 0 || dtype > 3) return fail(LS_INVALID_DATATYPE, "dtype must be 0..3");
  if (!op.is_real && dtype < 2) return fail(LS_OPERATOR_IS_COMPLEX, "operator is complex; use dtype 2 or 3");
  if (form == SED_FORM_AUTO) form = op.form;
  bool use_stream = op.stream.ready && form != SED_FORM_ON_THE_FLY;
  if (!use_stream && form != SED_FORM_ON_THE_FLY) {
    int st = operator_record_stream(op, stream);
    if (st == LS_SUCCESS) use_stream = true;
    else if (form == SED_FORM_STREAM) return st;  // AUTO falls back to on-the-fly
  }
  size_t const es = (size_t)elem_size(dtype);
  uint64_t c0 = 0;
  // the fixed-point block kernel keeps K tables of row factors in shared
  // memory: at most kmax columns per pass fit in 48 KB
  unsigned kmax = 16;
  if (dtype == 1 && op.tables->fix_ok) {
    size_t const per = (size_t)op.tables->fix.n_div * op.tables->fix_nv * 8;
    size_t const room = 48 * 1024 - op.tables->fix.n_codes;
    kmax = (unsigned)std::min<size_t>(16, room / per);
  }
  if (use_stream && block > 1 && kmax >= 2) {
    // K-column passes over the stream form (K = 16, 8, 4, 2)
    while (block - c0 >= 2) {
      uint64_t const left = std::min<uint64_t>(block - c0, kmax);
      unsigned const K = left >= 16 ? 16 : left >= 8 ? 8 : left >= 4 ? 4 : 2;
      void const* xc = static_cast<char const*>(x) + c0 * ldx * es;
      void* yc = static_cast<char*>(y) + c0 * ldy * es;
      int st;
      switch (dtype) {
        case 0: st = launch_block<float>(op, K, (float const*)xc, ldx, (float*)yc, ldy, stream); break;
        case 1: st = launch_block<double>(op, K, (double const*)xc, ldx, (double*)yc, ldy, stream); break;
        case 2: st = launch_block<float2>(op, K, (float2 const*)xc, ldx, (float2*)yc, ldy, stream); break;
        default: st = launch_block<double2>(op, K, (double2 const*)xc, ldx, (double2*)yc, ldy, stream); break;
      }
      if (st) return st;
      c0 += K;
    }
  }
  for (uint64_t c = c0; c < block; ++c) {
    void const* xc = static_cast<char const*>(x) + c * ldx * es;
    void* yc = static_cast<char*>(y) + c * ldy * es;
    int st;
    switch (dtype) {
      case 0: st = launch_apply<float>(op, (float const*)xc, (float*)yc, stream, use_stream, Indirect{}); break;
      case 1: st = launch_apply<double>(op, (double const*)xc, (double*)yc, stream, use_stream, Indirect{}); break;
      case 2: st = launch_apply<float2>(op, (float2 const*)xc, (float2*)yc, stream, use_stream, Indirect{}); break;
      default: st = launch_apply<double2>(op, (double2 const*)xc, (double2*)yc, stream, use_stream, Indirect{}); break;
    }
    if (st) return st;
  }
  return LS_SUCCESS;
}

namespace {

__global__ void k_to_float(double const* __restrict__ a, uint64_t n, float* __restrict__ b) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// FP32 streamed SpMV (real operators): FP32 entries of the value table and
// diagonal, FP32 accumulation per row; the partial sums of x_i y_i are
// reduced per warp in FP32 and per block in FP64.
template <bool Packed>
__global__ void __launch_bounds__(kBlock)
    k_spmv32(StreamView S, float const* __restrict__ table_f, float const* __restrict__ diag_f,
             float const* __restrict__ invs_f, uint64_t D, float const* __restrict__ x,
             float* __restrict__ y, Indirect ind) {
  extern __shared__ float tab[];  // value table, n_codes entries when it fits (dynamic size)
  __shared__ double red[kBlock / 32];
  if (ind.stop && *ind.stop) return;
  if (ind.k) {
    uint64_t const k = *ind.k;
    x += k * ind.ld;
    y += (k + 1) * ind.ld;
  }
  bool const in_smem = S.n_codes <= 8192u;
  if (in_smem) {
    for (uint32_t c = threadIdx.x; c < S.n_codes; c += blockDim.x) tab[c] = table_f[c];
    __syncthreads();
  }
  float const* tb = in_smem ? tab : table_f;
  uint64_t const i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t const s = i >> 5;
  float part = 0.0f;
  if ((s << 5) < D) {
    uint32_t const lane = threadIdx.x & 31;
    uint64_t const base = S.slice_ptr[s];
    uint32_t const width = (uint32_t)((S.slice_ptr[s + 1] - base) >> 5);
    uint32_t const col_mask = Packed ? ((1u << S.col_bits) - 1u) : 0xFFFFFFFFu;
    float acc = 0.0f;
    uint32_t const* ent = S.entries + base + lane;
    // Four entries per step: their loads, then their gathers, are issued
    // back to back (padding reads x[0] with a zero value); the sum keeps
    // entry order.
    constexpr uint32_t U = 4;
    uint32_t e = 0;
    for (; e + U <= width; e += U) {
      uint32_t v[U];
#pragma unroll
      for (uint32_t q = 0; q < U; ++q) v[q] = __ldcs(ent + (uint64_t)(e + q) * 32);
      float xv[U], tv[U];
#pragma unroll
      for (uint32_t q = 0; q < U; ++q) {
        bool const ok = v[q] != kNull;
        uint32_t const col = ok ? (v[q] & col_mask) : 0u;
        uint32_t code = 0;
        if (ok)
          code = Packed ? (v[q] >> S.col_bits) : (uint32_t)__ldcs(S.codes + base + lane + (uint64_t)(e + q) * 32);
        xv[q] = x[col];
        tv[q] = ok ? tb[code] : 0.0f;
      }
#pragma unroll
      for (uint32_t q = 0; q < U; ++q) acc = fmaf(tv[q], xv[q], acc);
    }
    for (; e < width; ++e) {
      uint32_t const v = __ldcs(ent + (uint64_t)e * 32);
      if (v != kNull) {
        uint32_t const col = v & col_mask;
        uint32_t const code =
            Packed ? (v >> S.col_bits) : (uint32_t)__ldcs(S.codes + base + lane + (uint64_t)e * 32);
        acc = fmaf(tb[code], x[col], acc);
      }
    }
    if (i < D) {
      float const xi = x[i];
      float const yi = fmaf(diag_f[i], xi, invs_f[S.row_class[i]] * acc);
      y[i] = yi;
      part = xi * yi;
    }
  }
  if (ind.partial) {
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    double const tot = block_sum((threadIdx.x & 31) == 0 ? (double)part : 0.0, red);
    if (threadIdx.x == 0) ind.partial[blockIdx.x] = tot;
  }
}

// FP32-stored form in fixed point. The stored vector x is FP32; its gather
// copy u_j = round(sqrt(S_j) x_j 2^F) is int32 (4 bytes streamed per
// element, like FP32), the row sums are exact in int64 and the matrix
// values, the diagonal and the row epilogue are FP64; y is stored in FP32.
__global__ void __launch_bounds__(kBlock) k_fix_max32(float const* __restrict__ x, uint64_t D,
                                                      unsigned long long* __restrict__ max_bits, Indirect ind) {
  __shared__ unsigned long long red[kBlock / 32];
  if (ind.stop && *ind.stop) return;
  if (ind.k) x += (uint64_t)*ind.k * ind.ld;
  uint32_t m = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (uint64_t)gridDim.x * blockDim.x)
    m = max(m, (uint32_t)__float_as_uint(x[i]) & 0x7FFFFFFFu);
  m = __reduce_max_sync(0xffffffffu, m);
  // as the double of the same value (finite floats keep their order; a float
  // NaN or infinity maps to the double infinity pattern or above)
  unsigned long long d;
  if (m >= 0x7F800000u) d = 0x7FF0000000000000ull | (m & 0x7FFFFFu);
  else d = (unsigned long long)__double_as_longlong((double)__uint_as_float(m));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = d;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (unsigned w = 1; w < kBlock / 32; ++w) d = max(d, red[w]);
    atomicMax(max_bits, d);
  }
}

__global__ void __launch_bounds__(kBlock) k_fix_convert32(float const* __restrict__ x, uint64_t D,
                                                          uint8_t const* __restrict__ row_class, FixView fv,
                                                          unsigned long long const* __restrict__ max_bits,
                                                          int64_t* __restrict__ F_out, int32_t* __restrict__ u,
                                                          Indirect ind) {
  __shared__ double fac[kFixMaxClasses];
  if (ind.stop && *ind.stop) return;
  if (ind.k) x += (uint64_t)*ind.k * ind.ld;
  int64_t const F = fix_exponent32(max_bits[0], fv.sqrt_s_max);
  if (blockIdx.x == 0 && threadIdx.x == 0) F_out[0] = F;
  double const p2 = F == kFixBad ? 0.0 : fix_pow2(F);
  for (uint32_t c = threadIdx.x; c < fv.n_div; c += blockDim.x) fac[c] = fv.sqrt_s[c] * p2;
  __syncthreads();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (uint64_t)gridDim.x * blockDim.x)
    u[i] = F == kFixBad ? 0 : (int32_t)fix_round((double)x[i] * fac[row_class[i]]);
}

template <bool Packed, int NV>
__global__ void __launch_bounds__(kBlock) k_spmv32_fix(StreamView S, FixView fv, uint64_t D,
                                                       float const* __restrict__ x, int32_t const* __restrict__ u,
                                                       int64_t const* __restrict__ F_in, float* __restrict__ y,
                                                       Indirect ind) {
  extern __shared__ double fix_smem[];  // g[n_div NV], then code8[n_codes]
  __shared__ double red[kBlock / 32];
  if (ind.stop && *ind.stop) return;
  if (ind.k) {
    uint64_t const k = *ind.k;
    x += k * ind.ld;
    y += (k + 1) * ind.ld;
  }
  int64_t const F = F_in[0];
  double* g = fix_smem;
  uint8_t* code8 = reinterpret_cast<uint8_t*>(fix_smem + fv.n_div * NV);
  for (uint32_t c = threadIdx.x; c < fv.n_codes; c += blockDim.x) code8[c] = fv.code[c];
  fix_row_factors<NV>(fv, S.inv_sqrt_s, F, g);
  __syncthreads();
  uint64_t const i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t const s = i >> 5;
  float part = 0.0f;
  if ((s << 5) < D) {
    uint32_t const lane = threadIdx.x & 31;
    uint64_t const base = S.slice_ptr[s];
    uint32_t const width = (uint32_t)((S.slice_ptr[s + 1] - base) >> 5);
    uint32_t const col_mask = Packed ? ((1u << S.col_bits) - 1u) : 0xFFFFFFFFu;
    int64_t acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0;
    uint32_t const* ent = S.entries + base + lane;
    constexpr uint32_t U = 8;
    uint32_t e = 0;
    for (; e + U <= width; e += U) {
      uint32_t v[U];
#pragma unroll
      for (uint32_t q = 0; q < U; ++q) v[q] = __ldcs(ent + (uint64_t)(e + q) * 32);
      int32_t gv[U];
      uint32_t t[U];
#pragma unroll
      for (uint32_t q = 0; q < U; ++q) {
        gv[q] = 0;
        t[q] = 0;
        if (v[q] != kNull) {
          uint32_t const code =
              Packed ? (v[q] >> S.col_bits) : (uint32_t)__ldcs(S.codes + base + lane + (uint64_t)(e + q) * 32);
          gv[q] = u[v[q] & col_mask];
          t[q] = code8[code];
        }
      }
#pragma unroll
      for (uint32_t q = 0; q < U; ++q) fix_add<NV>(acc, t[q], (int64_t)gv[q]);
    }
    for (; e < width; ++e) {
      uint32_t const v = __ldcs(ent + (uint64_t)e * 32);
      if (v != kNull) {
        uint32_t const code = Packed ? (v >> S.col_bits) : (uint32_t)__ldcs(S.codes + base + lane + (uint64_t)e * 32);
        fix_add<NV>(acc, code8[code], (int64_t)u[v & col_mask]);
      }
    }
    if (i < D) {
      float const xf = __ldcs(x + i);
      double const yi = fix_row<NV>(acc, g + (uint32_t)__ldcs(S.row_class + i) * NV, F,
                                    __ldcs(static_cast<double const*>(S.diag) + i), (double)xf);
      float const yf = (float)yi;
      __stcs(y + i, yf);
      part = xf * yf;
    }
  }
  if (ind.partial) {
    // the product of the stored FP32 values summed per warp in FP32, then
    // per block in FP64 (fixed order)
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = (double)part;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0.0;
      for (unsigned w = 0; w < kBlock / 32; ++w) tot += red[w];
      ind.partial[blockIdx.x] = tot;
    }
  }
}

}  // namespace

int operator_prepare_fp32(OperatorData& op, cudaStream_t stream) {
  StreamForm& sf = op.stream;
  if (!sf.ready) return fail(LS_CACHE_NOT_BUILT, "the FP32 SpMV needs the stream form");
  if (!op.is_real) return fail(LS_OPERATOR_IS_COMPLEX, "the FP32 Krylov phase supports real operators");
  if (sf.diag_f.ptr) return LS_SUCCESS;
  OperatorTables const& tb = *op.tables;
  uint64_t const D = op.basis->D;
  if (tb.fix_ok) {
    if (int st = op.fix_u32.allocate(std::max<uint64_t>(1, D) * 4)) return st;
    if (int st = op.fix_slots32.allocate(16)) return st;
  }
  if (int st = sf.diag_f.allocate(std::max<uint64_t>(1, D) * 4)) return st;
  if (int st = sf.table_f.allocate((size_t)tb.n_codes * 4)) return st;
  if (int st = sf.invs_f.allocate((size_t)tb.code.n_div * 4)) return st;
  { k_to_float<<<grid_size(D, op.basis->device, 8), kBlock, 0, stream>>>(sf.diag.as<double>(), D, sf.diag_f.as<float>()); note_launches(1); }
  { k_to_float<<<1, kBlock, 0, stream>>>(tb.table.as<double>(), tb.n_codes, sf.table_f.as<float>()); note_launches(1); }
  { k_to_float<<<1, kBlock, 0, stream>>>(tb.inv_sqrt_s.as<double>(), tb.code.n_div, sf.invs_f.as<float>()); note_launches(1); }
  SED_TRY_CUDA(cudaGetLastError());
  SED_TRY_CUDA(cudaStreamSynchronize(stream));
  return LS_SUCCESS;
}

namespace {
template <int NV>
void launch_spmv32_fix(OperatorData& op, StreamView const& S, float const* x, float* y, Indirect ind,
                       cudaStream_t stream, unsigned grid) {
  OperatorTables const& tb = *op.tables;
  auto* slots = op.fix_slots32.as<unsigned long long>();
  auto* F = reinterpret_cast<int64_t*>(slots + 1);
  int32_t* u = op.fix_u32.as<int32_t>();
  uint64_t const D = op.basis->D;
  size_t const smem = (size_t)tb.fix.n_div * NV * 8 + tb.fix.n_codes;
  if (op.stream.packed)
    k_spmv32_fix<true, NV><<<grid, kBlock, smem, stream>>>(S, tb.fix, D, x, u, F, y, ind);
  else
    k_spmv32_fix<false, NV><<<grid, kBlock, smem, stream>>>(S, tb.fix, D, x, u, F, y, ind);
  note_launches(1);
}

int launch32(OperatorData& op, float const* x, float* y, Indirect ind, cudaStream_t stream, unsigned* blocks) {
  StreamForm const& sf = op.stream;
  if (!sf.diag_f.ptr) return fail(LS_CACHE_NOT_BUILT, "FP32 companions are not prepared");
  StreamView const S = stream_view(op);
  unsigned const grid = (unsigned)((sf.n_slices * 32 + kBlock - 1) / kBlock);
  if (blocks) *blocks = grid;
  OperatorTables const& tb = *op.tables;
  if (tb.fix_ok && op.fix_u32.ptr) {
    uint64_t const D = op.basis->D;
    auto* slots = op.fix_slots32.as<unsigned long long>();
    SED_TRY_CUDA(cudaMemsetAsync(slots, 0, 8, stream));
    unsigned const vg = grid_size(D, op.basis->device, 8);
    k_fix_max32<<<vg, kBlock, 0, stream>>>(x, D, slots, ind);
    k_fix_convert32<<<vg, kBlock, 0, stream>>>(x, D, sf.row_class.as<uint8_t>(), tb.fix, slots,
                                               reinterpret_cast<int64_t*>(slots + 1), op.fix_u32.as<int32_t>(), ind);
    note_launches(2);
    switch (tb.fix_nv) {
      case 1: launch_spmv32_fix<1>(op, S, x, y, ind, stream, grid); break;
      case 2: launch_spmv32_fix<2>(op, S, x, y, ind, stream, grid); break;
      default: launch_spmv32_fix<4>(op, S, x, y, ind, stream, grid); break;
    }
    SED_TRY_CUDA(cudaGetLastError());
    return LS_SUCCESS;
  }
  // size the table to the codes: a large carve-out would shrink L1 for the gathers
  size_t const smem = S.n_codes <= 8192u ? (size_t)S.n_codes * 4 : 0;
  if (sf.packed)
    { k_spmv32<true><<<grid, kBlock, smem, stream>>>(S, sf.table_f.as<float>(), sf.diag_f.as<float>(), sf.invs_f.as<float>(), op.basis->D, x, y, ind); note_launches(1); }
  else
    { k_spmv32<false><<<grid, kBlock, smem, stream>>>(S, sf.table_f.as<float>(), sf.diag_f.as<float>(), sf.invs_f.as<float>(), op.basis->D, x, y, ind); note_launches(1); }
  SED_TRY_CUDA(cudaGetLastError());
  return LS_SUCCESS;
}
}  // namespace

int operator_apply_krylov32(OperatorData& op, float* base, Indirect ind, cudaStream_t stream, unsigned* blocks) {
  return launch32(op, base, base, ind, stream, blocks);
}

int operator_apply32(OperatorData& op, float const* x, float* y, cudaStream_t stream) {
  return launch32(op, x, y, Indirect{}, stream, nullptr);
}

int operator_apply_krylov(OperatorData& op, int dtype, void* base, Indirect ind, cudaStream_t stream,
                          unsigned* blocks) {
  bool const use_stream = op.stream.ready && op.form != SED_FORM_ON_THE_FLY;
  uint64_t const D = op.basis->D;
  *blocks = use_stream ? (unsigned)((op.stream.n_slices * 32 + kBlock - 1) / kBlock)
                       : (unsigned)((D + kBlock - 1) / kBlock);
  switch (dtype) {
    case 1: return launch_apply<double>(op, (double const*)base, (double*)base, stream, use_stream, ind);
    case 3: return launch_apply<double2>(op, (double2 const*)base, (double2*)base, stream, use_stream, ind);
    case 0: return launch_apply<float>(op, (float const*)base, (float*)base, stream, use_stream, ind);
    default: return launch_apply<float2>(op, (float2 const*)base, (float2*)base, stream, use_stream, ind);
  }
}

}  // namespace sed

using namespace sed;

namespace {

int create_interaction(ls_interaction** ptr, unsigned k, void const* matrix, unsigned number_nodes,
                       uint16_t const* nodes) {
  if (!ptr || !matrix || (number_nodes && !nodes))
    return fail(LS_INVALID_ARGUMENT, "ls_create_interaction: NULL argument");
  unsigned const dim = 1u << k;
  auto* it = new (std::nothrow) ls_interaction;
  if (!it) return fail(LS_OUT_OF_MEMORY, "ls_create_interaction");
  it->d.k = k;
  double const* m = static_cast<double const*>(matrix);
  it->d.matrix.assign(m, m + 2 * dim * dim);
  it->d.sites.assign(nodes, nodes + (size_t)number_nodes * k);
  for (unsigned u = 0; u < number_nodes; ++u)
    for (unsigned a = 0; a < k; ++a)
      for (unsigned c = 0; c < a; ++c)
        if (nodes[u * k + a] == nodes[u * k + c]) {
          delete it;
          return fail(LS_INVALID_ARGUMENT, "a site tuple repeats a site");
        }
  it->d.is_real = true;
  for (unsigned q = 0; q < dim * dim; ++q)
    if (m[2 * q + 1] != 0.0) it->d.is_real = false;
  *ptr = it;
  return LS_SUCCESS;
}

int host_blocks(OperatorData& op, int dtype, uint64_t size, uint64_t block, void const* x,
                uint64_t ldx, void* y, uint64_t ldy) {
  BasisData& b = *op.basis;
  size_t const es = (size_t)elem_size(dtype);
  bool const x_dev = is_device_pointer(x), y_dev = is_device_pointer(y);
  if (x_dev || y_dev) SED_TRY_CUDA(cudaDeviceSynchronize());  // the caller's writes of x, reads of y
  cudaStream_t s = op.cuda_stream;
  DeviceBuffer xb, yb;
  void const* xd = x;
  void* yd = y;
  uint64_t lx = ldx, ly = ldy;
  if (!x_dev) {
    if (int st = xb.allocate(size * block * es)) return st;
    SED_TRY_CUDA(cudaMemcpy2DAsync(xb.ptr, size * es, x, ldx * es, size * es, block, cudaMemcpyHostToDevice, s));
    xd = xb.ptr;
    lx = size;
  }
  if (!y_dev) {
    if (int st = yb.allocate(size * block * es)) return st;
    yd = yb.ptr;
    ly = size;
  }
  if (int st = operator_apply_device(op, dtype, block, xd, lx, yd, ly, s, SED_FORM_AUTO)) return st;
  if (!y_dev)
    SED_TRY_CUDA(cudaMemcpy2DAsync(y, ldy * es, yd, size * es, size * es, block, cudaMemcpyDeviceToHost, s));
  SED_TRY_CUDA(cudaStreamSynchronize(s));
  (void)b;
  return LS_SUCCESS;
}

int check_block(OperatorData const& op, int dtype, uint64_t size, uint64_t block, uint64_t ldx) {
  if (!op.basis->built) return fail(LS_CACHE_NOT_BUILT, "basis has not been built (call ls_build)");
  if (dtype < 0 || dtype > 3) return fail(LS_INVALID_DATATYPE, "dtype must be 0..3");
  if (size != op.basis->D)
    return fail(LS_DIMENSION_MISMATCH, "vector length " + std::to_string(size) +
                                           " != basis dimension " + std::to_string(op.basis->D));
  if (block > 0 && ldx < size) return fail(LS_INVALID_ARGUMENT, "column stride is smaller than the size");
  return LS_SUCCESS;
}

}  // namespace

extern "C" {

int ls_create_interaction1(ls_interaction** p, void const* m, unsigned n, uint16_t const* s) {
  return create_interaction(p, 1, m, n, s);
}
int ls_create_interaction2(ls_interaction** p, void const* m, unsigned n, uint16_t const* s) {
  return create_interaction(p, 2, m, n, s);
}
int ls_create_interaction3(ls_interaction** p, void const* m, unsigned n, uint16_t const* s) {
  return create_interaction(p, 3, m, n, s);
}
int ls_create_interaction4(ls_interaction** p, void const* m, unsigned n, uint16_t const* s) {
  return create_interaction(p, 4, m, n, s);
}
bool ls_interaction_is_real(ls_interaction const* i) { return i && i->d.is_real; }
void ls_destroy_interaction(ls_interaction* i) { delete i; }

int ls_create_operator(ls_operator** ptr, ls_spin_basis const* basis, unsigned number_terms,
                       ls_interaction const* const terms[]) {
  if (!ptr || !basis || (number_terms && !terms))
    return fail(LS_INVALID_ARGUMENT, "ls_create_operator: NULL argument");
  try {
    auto d = std::make_shared<OperatorData>();
    d->basis = basis->d;
    d->is_real = true;
    for (unsigned t = 0; t < number_terms; ++t) {
      if (!terms[t]) return fail(LS_INVALID_ARGUMENT, "ls_create_operator: NULL term");
      for (uint16_t s : terms[t]->d.sites)
        if (s >= basis->d->n)
          return fail(LS_INVALID_ARGUMENT, "site index " + std::to_string(s) +
                                               " is not below number_spins " + std::to_string(basis->d->n));
      d->terms.push_back(terms[t]->d);
      d->is_real = d->is_real && terms[t]->d.is_real;
    }
    d->is_real = d->is_real && characters_real(*basis->d);
    auto* op = new ls_operator;
    op->d = std::move(d);
    *ptr = op;
    return LS_SUCCESS;
  } catch (std::bad_alloc const&) {
    return fail(LS_OUT_OF_MEMORY, "ls_create_operator");
  }
}

void ls_destroy_operator(ls_operator* op) { delete op; }
bool ls_operator_is_real(ls_operator const* op) { return op && op->d->is_real; }

int ls_operator_matmat(ls_operator const* op, int dtype, uint64_t size, uint64_t block_size,
                       void const* x, uint64_t x_stride, void* y, uint64_t y_stride) {
  if (!op || (block_size && (!x || !y))) return fail(LS_INVALID_ARGUMENT, "ls_operator_matmat: NULL argument");
  OperatorData& d = *op->d;
  std::lock_guard<std::mutex> lock(d.mu);
  if (int st = check_block(d, dtype, size, block_size, x_stride)) return st;
  if (block_size && y_stride < size) return fail(LS_INVALID_ARGUMENT, "column stride is smaller than the size");
  if (!d.is_real && dtype < 2) return fail(LS_OPERATOR_IS_COMPLEX, "operator is complex; use dtype 2 or 3");
  if (block_size == 0 || size == 0) return LS_SUCCESS;
  try {
    ScopedDevice dev(d.basis->device);
    if (int st = operator_ensure_ready(d)) return st;
    return host_blocks(d, dtype, size, block_size, x, x_stride, y, y_stride);
  } catch (std::exception const& e) {
    return fail(LS_SYSTEM_ERROR, e.what());
  }
}

int sed_operator_matmat_device(ls_operator const* op, int dtype, uint64_t size, uint64_t block_size,
                               void const* x, uint64_t x_stride, void* y, uint64_t y_stride,
                               void* stream) {
  if (!op || (block_size && (!x || !y))) return fail(LS_INVALID_ARGUMENT, "sed_operator_matmat_device: NULL argument");
  OperatorData& d = *op->d;
  std::lock_guard<std::mutex> lock(d.mu);
  if (int st = check_block(d, dtype, size, block_size, x_stride)) return st;
  if (block_size == 0 || size == 0) return LS_SUCCESS;
  ScopedDevice dev(d.basis->device);
  if (int st = operator_ensure_ready(d)) return st;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : d.cuda_stream;
  return operator_apply_device(d, dtype, block_size, x, x_stride, y, y_stride, s, SED_FORM_AUTO);
}

int ls_operator_expectation(ls_operator const* op, int dtype, uint64_t size, uint64_t block_size,
                            void const* x, uint64_t x_stride, void* out) {
  if (!op || !out || (block_size && !x)) return fail(LS_INVALID_ARGUMENT, "ls_operator_expectation: NULL argument");
  OperatorData& d = *op->d;
  std::lock_guard<std::mutex> lock(d.mu);
  if (int st = check_block(d, dtype, size, block_size, x_stride)) return st;
  if (!d.is_real && dtype < 2) return fail(LS_OPERATOR_IS_COMPLEX, "operator is complex; use dtype 2 or 3");
  double* res = static_cast<double*>(out);
  if (block_size == 0) return LS_SUCCESS;
  if (size == 0) {
    for (uint64_t c = 0; c < block_size; ++c) res[2 * c] = res[2 * c + 1] = 0.0;
    return LS_SUCCESS;
  }
  try {
    ScopedDevice dev(d.basis->device);
    if (int st = operator_ensure_ready(d)) return st;
    size_t const es = (size_t)elem_size(dtype);
    cudaStream_t s = d.cuda_stream;
    if (int st = wait_for_caller({x})) return st;
    DeviceBuffer xb, yb, part;
    if (int st = xb.allocate(size * block_size * es)) return st;
    if (int st = yb.allocate(size * block_size * es)) return st;
    SED_TRY_CUDA(cudaMemcpy2DAsync(xb.ptr, size * es, x, x_stride * es, size * es, block_size, cudaMemcpyDefault, s));
    if (int st = operator_apply_device(d, dtype, block_size, xb.ptr, size, yb.ptr, size, s, SED_FORM_AUTO)) return st;
    unsigned const grid = grid_size(size, d.basis->device, 4);
    if (int st = part.allocate((size_t)grid * 16 * block_size)) return st;
    for (uint64_t c = 0; c < block_size; ++c) {
      char const* xc = xb.as<char>() + c * size * es;
      char const* yc = yb.as<char>() + c * size * es;
      double2* pc = part.as<double2>() + c * grid;
      switch (dtype) {
        case 0: { k_dot_conj<float><<<grid, kBlock, 0, s>>>((float const*)xc, (float const*)yc, size, pc); note_launches(1); } break;
        case 1: { k_dot_conj<double><<<grid, kBlock, 0, s>>>((double const*)xc, (double const*)yc, size, pc); note_launches(1); } break;
        case 2: { k_dot_conj<float2><<<grid, kBlock, 0, s>>>((float2 const*)xc, (float2 const*)yc, size, pc); note_launches(1); } break;
        default: { k_dot_conj<double2><<<grid, kBlock, 0, s>>>((double2 const*)xc, (double2 const*)yc, size, pc); note_launches(1); } break;
      }
    }
    SED_TRY_CUDA(cudaGetLastError());
    std::vector<double2> h((size_t)grid * block_size);
    SED_TRY_CUDA(cudaMemcpyAsync(h.data(), part.ptr, h.size() * 16, cudaMemcpyDeviceToHost, s));
    SED_TRY_CUDA(cudaStreamSynchronize(s));
    for (uint64_t c = 0; c < block_size; ++c) {
      double re = 0.0, im = 0.0;
      for (unsigned g = 0; g < grid; ++g) {
        re += h[c * grid + g].x;
        im += h[c * grid + g].y;
      }
      res[2 * c] = re;
      res[2 * c + 1] = im;
    }
    return LS_SUCCESS;
  } catch (std::exception const& e) {
    return fail(LS_SYSTEM_ERROR, e.what());
  }
}

void sed_set_record_mode(int mode) {
  g_record_mode = mode == SED_RECORD_CANONICALISE ? SED_RECORD_CANONICALISE : SED_RECORD_AUTO;
}

int sed_operator_recorded_with_table(ls_operator const* op) {
  return op && op->d->stream.ready && op->d->stream.orbit_table ? 1 : 0;
}

int sed_operator_time_matvec(ls_operator const* op, void const* x, void* y, unsigned repetitions,
                             double* ms_matvec, double* ms_kernel) {
  if (!op || !x || !y || !ms_matvec || !ms_kernel || repetitions == 0)
    return fail(LS_INVALID_ARGUMENT, "sed_operator_time_matvec: bad argument");
  OperatorData& d = *op->d;
  std::lock_guard<std::mutex> lock(d.mu);
  if (!d.is_real) return fail(LS_OPERATOR_IS_COMPLEX, "sed_operator_time_matvec: real operators only");
  try {
    ScopedDevice dev(d.basis->device);
    if (int st = operator_ensure_ready(d)) return st;
    if (!is_device_pointer(x) || !is_device_pointer(y))
      return fail(LS_INVALID_ARGUMENT, "sed_operator_time_matvec: x and y must be device memory");
    if (int st = wait_for_caller({x, y})) return st;
    if (int st = fix_wait(d)) return st;
    cudaStream_t s = d.cuda_stream;
    double const* xd = static_cast<double const*>(x);
    double* yd = static_cast<double*>(y);
    bool const use_stream = d.stream.ready && d.form != SED_FORM_ON_THE_FLY;
    cudaEvent_t e0, e1;
    SED_TRY_CUDA(cudaEventCreate(&e0));
    SED_TRY_CUDA(cudaEventCreate(&e1));
    struct EvGuard {
      cudaEvent_t a, b;
      ~EvGuard() { cudaEventDestroy(a); cudaEventDestroy(b); }
    } eg{e0, e1};
    auto timed = [&](bool kernel_only, double* out) -> int {
      for (unsigned r = 0; r < repetitions + 2; ++r) {
        if (r == 2) SED_TRY_CUDA(cudaEventRecord(e0, s));
        Indirect ind;
        ind.prescaled = kernel_only;
        if (int st = launch_apply<double>(d, xd, yd, s, use_stream, ind)) return st;
      }
      SED_TRY_CUDA(cudaEventRecord(e1, s));
      SED_TRY_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      SED_TRY_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      *out = ms / repetitions;
      return LS_SUCCESS;
    };
    if (int st = timed(false, ms_matvec)) return st;  // leaves u and F of x in the workspace
    FixSlots fs;
    if (fix_slots(d, &fs)) {
      if (int st = timed(true, ms_kernel)) return st;
    } else {
      *ms_kernel = *ms_matvec;
    }
    SED_TRY_CUDA(cudaStreamSynchronize(s));
    return LS_SUCCESS;
  } catch (std::exception const& e) {
    return fail(LS_SYSTEM_ERROR, e.what());
  }
}

int sed_operator_prepare(ls_operator* op, int form) {
  if (!op) return fail(LS_INVALID_ARGUMENT, "sed_operator_prepare: NULL operator");
  OperatorData& d = *op->d;
  std::lock_guard<std::mutex> lock(d.mu);
  ScopedDevice dev(d.basis ? d.basis->device : -1);
  if (int st = operator_ensure_ready(d)) return st;
  if (form < SED_FORM_AUTO || form > SED_FORM_ON_THE_FLY) return fail(LS_INVALID_ARGUMENT, "unknown form");
  d.form = form;
  if (form == SED_FORM_ON_THE_FLY) return LS_SUCCESS;
  int st = operator_record_stream(d, d.cuda_stream);
  return (form == SED_FORM_AUTO && st == LS_OUT_OF_MEMORY) ? LS_SUCCESS : st;
}

uint64_t sed_operator_stream_bytes(ls_operator const* op) {
  return (op && op->d->stream.ready) ? op->d->stream.bytes() : 0;
}
uint64_t sed_operator_stream_elements(ls_operator const* op) {
  return (op && op->d->stream.ready) ? op->d->stream.n_elements : 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// sed_operator_expectation_noalloc: ls_operator_expectation without any device
// allocation.
//
// Some callers cannot let a library call cudaMalloc: a process whose device
// memory is already handed out to its own pool allocator (the allocation would
// fail or fragment the pool), or a latency-critical loop for which cudaMalloc's
// and cudaFree's implicit device synchronisation is unacceptable. For them this
// entry point computes Y = H X into the caller's device buffer and
// out[c] = <x_c|y_c> with the per-block partial sums kept in the file-scope
// array below, so the call itself allocates nothing (the operator must already
// be prepared, see sed.h).
namespace sed {
namespace {

constexpr unsigned kNoAllocCols = 64;        // columns per call
constexpr unsigned kNoAllocPartials = 4096;  // partial sums shared by all columns
// Scratch shared by every call in this process: partial sums, then the
// per-column results. 4096 x 16 B + 64 x 16 B = 66 KiB on every GPU that
// loads the library, held until exit.
static __device__ __align__(256) double2 g_noalloc_scratch[kNoAllocPartials + kNoAllocCols];

std::mutex g_noalloc_mu;
// Device address of the scratch, per device, looked up on the first call on
// that device. A device reset (cudaDeviceReset) invalidates it together with
// every libsed handle's device memory, so handles and this cache go stale at
// the same moment: after a reset, no libsed object may be used again.
void* g_noalloc_addr[64] = {nullptr};

// Set-up, once per device and with that device current: the host-side name of
// g_noalloc_scratch is not a device address, so look the address up.
int noalloc_scratch(int device, double2** out) {
  if (device < 0 || device >= 64) return fail(LS_CUDA_ERROR, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return fail(LS_CUDA_ERROR, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
    g_noalloc_addr[device] = p;
  }
  *out = static_cast<double2*>(g_noalloc_addr[device]);
  return LS_SUCCESS;
}

// Per-block partial sums of conj(x_i) y_i into partial[blockIdx.x].
template <class X>
__global__ void k_dot_conj_noalloc(X const* __restrict__ x, X const* __restrict__ y, uint64_t n,
                                   double2* __restrict__ partial) {
  using V = typename Store<X>::V;
  __shared__ double red_re[kBlock / 32], red_im[kBlock / 32];
  double re = 0.0, im = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    V const a = Store<X>::load(x, i), b = Store<X>::load(y, i);
    if constexpr (std::is_same<V, double>::value) {
      re = fma(a, b, re);
    } else {
      re = fma(a.re, b.re, fma(a.im, b.im, re));
      im = fma(a.re, b.im, fma(-a.im, b.re, im));
    }
  }
  double const sre = block_sum(re, red_re);
  double const sim = block_sum(im, red_im);
  if (threadIdx.x == 0) partial[blockIdx.x] = make_double2(sre, sim);
}

// results[c] = sum of the `per_col` partials of column c.
__global__ void k_sum_partials_noalloc(double2 const* __restrict__ partial, unsigned per_col,
                                       unsigned cols, double2* __restrict__ results) {
  __shared__ double red_re[kBlock / 32], red_im[kBlock / 32];
  for (unsigned c = 0; c < cols; ++c) {
    double re = 0.0, im = 0.0;
    for (unsigned i = threadIdx.x; i < per_col; i += blockDim.x) {
      re += partial[(uint64_t)c * per_col + i].x;
      im += partial[(uint64_t)c * per_col + i].y;
    }
    double const sre = block_sum(re, red_re);
    double const sim = block_sum(im, red_im);
    if (threadIdx.x == 0) results[c] = make_double2(sre, sim);
  }
}

}  // namespace
}  // namespace sed

extern "C" int sed_operator_expectation_noalloc(ls_operator const* op, int dtype, uint64_t size,
                                                uint64_t block_size, void const* x, uint64_t x_stride,
                                                void* y, uint64_t y_stride, void* out, void* stream) {
  using namespace sed;
  if (!op || !out || (block_size && (!x || !y)))
    return fail(LS_INVALID_ARGUMENT, "sed_operator_expectation_noalloc: NULL argument");
  OperatorData& d = *op->d;
  std::lock_guard<std::mutex> lock(d.mu);
  if (int st = check_block(d, dtype, size, block_size, x_stride)) return st;
  if (block_size && y_stride < size) return fail(LS_INVALID_ARGUMENT, "column stride is smaller than the size");
  if (block_size > kNoAllocCols)
    return fail(LS_INVALID_ARGUMENT, "sed_operator_expectation_noalloc: at most " + std::to_string(kNoAllocCols) +
                                         " columns per call (got " + std::to_string(block_size) + ")");
  if (!d.is_real && dtype < 2) return fail(LS_OPERATOR_IS_COMPLEX, "operator is complex; use dtype 2 or 3");
  if (!d.tables || !d.term_buf.ptr || !d.cuda_stream || !d.basis->plan_buf.ptr)
    return fail(LS_CACHE_NOT_BUILT,
                "sed_operator_expectation_noalloc: prepare the operator first (sed_operator_prepare)");
  if (block_size == 0) return LS_SUCCESS;
  if (!is_device_pointer(x) || !is_device_pointer(y))
    return fail(LS_INVALID_ARGUMENT, "sed_operator_expectation_noalloc: x and y must be device memory");
  ScopedDevice dev(d.basis->device);
  double2* scratch = nullptr;
  if (int st = noalloc_scratch(d.basis->device, &scratch)) return st;
  // The caller's stream orders this work after the caller's writes of x (and
  // of y); NULL means the operator's own stream, which is ordered with
  // nothing the caller enqueued.
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : d.cuda_stream;
  bool const use_stream = d.stream.ready && d.form != SED_FORM_ON_THE_FLY;
  size_t const es = (size_t)elem_size(dtype);
  unsigned const per_col = std::max(1u, std::min(grid_size(size, d.basis->device, 4),
                                                 kNoAllocPartials / (unsigned)block_size));
  for (uint64_t c = 0; c < block_size; ++c) {
    char const* xc = static_cast<char const*>(x) + c * x_stride * es;
    char* yc = static_cast<char*>(y) + c * y_stride * es;
    double2* pc = scratch + c * per_col;
    int st;
    switch (dtype) {
      case 0:
        st = launch_apply<float>(d, (float const*)xc, (float*)yc, s, use_stream, Indirect{});
        if (!st) { k_dot_conj_noalloc<float><<<per_col, kBlock, 0, s>>>((float const*)xc, (float const*)yc, size, pc); note_launches(1); }
        break;
      case 1:
        st = launch_apply<double>(d, (double const*)xc, (double*)yc, s, use_stream, Indirect{});
        if (!st) { k_dot_conj_noalloc<double><<<per_col, kBlock, 0, s>>>((double const*)xc, (double const*)yc, size, pc); note_launches(1); }
        break;
      case 2:
        st = launch_apply<float2>(d, (float2 const*)xc, (float2*)yc, s, use_stream, Indirect{});
        if (!st) { k_dot_conj_noalloc<float2><<<per_col, kBlock, 0, s>>>((float2 const*)xc, (float2 const*)yc, size, pc); note_launches(1); }
        break;
      default:
        st = launch_apply<double2>(d, (double2 const*)xc, (double2*)yc, s, use_stream, Indirect{});
        if (!st) { k_dot_conj_noalloc<double2><<<per_col, kBlock, 0, s>>>((double2 const*)xc, (double2 const*)yc, size, pc); note_launches(1); }
        break;
    }
    if (st) return st;
  }
  double2* results = scratch + kNoAllocPartials;
  { k_sum_partials_noalloc<<<1, kBlock, 0, s>>>(scratch, per_col, (unsigned)block_size, results); note_launches(1); }
  SED_TRY_CUDA(cudaGetLastError());
  SED_TRY_CUDA(cudaMemcpyAsync(out, results, block_size * sizeof(double2), cudaMemcpyDefault, s));
  SED_TRY_CUDA(cudaStreamSynchronize(s));
  return LS_SUCCESS;
}
