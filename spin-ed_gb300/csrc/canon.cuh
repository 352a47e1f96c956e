// canon.cuh — orbit canonicalisation of spin configurations, shared by the
// host (single-state queries, plan checks) and the sm_103a kernels.
//
// A symmetry group G (closure of the user's generators, src/SpinED/Internal.hs:120-150)
// is split into right cosets of a subgroup H of "cheap" permutations:
//     G = H p_0  u  H p_1  u ... ,   p_0 = identity.
// Elements of H (lattice translations in practice) move each bit by one of
// at most SED_MAX_TERMS displacements, so h(y) = OR_t rotl(y & m_t, r_t): a
// handful of integer ops. Each coset representative p is applied once per
// state through a Benes network of delta swaps
//     t = ((x >> s) ^ x) & m;  x ^= t ^ (t << s).
// Spin inversion (x -> ~x within n bits) commutes with every permutation and
// is applied to each image for free.
//
// Orbit minima are the representatives (what lattice-symmetries' ls_build
// returns, Internal.hs:178-179); a representative belongs to the sector iff
// the character is trivial on its stabiliser, and its stabiliser order S
// fixes the norm sqrt(S / |G|).
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define SED_HD __host__ __device__ __forceinline__
#else
#define SED_HD inline
#endif

namespace sed {

constexpr unsigned SED_MAX_TERMS = 4;    // displacements per element of H
constexpr unsigned SED_MAX_STAGES = 11;  // Benes stages for 64 bits
constexpr unsigned SED_PARAM_COSETS = 16;  // cosets whose networks travel in kernel parameters
constexpr unsigned SED_MAX_ROWS = 8;       // rows handled in registers by the row path

struct PlanView {
  // Benes masks of every coset for the full, unpruned network of the word
  // width (stage shifts 32,16,...,1,...,16,32 for 64 bits; 16,...,1,...,16 for
  // 32), carried in kernel-parameter space when n_cosets <= SED_PARAM_COSETS
  // (fixed_nets = 1) so that each stage is a handful of immediate-shift ops.
  uint32_t fixed_nets;
  uint64_t nets[SED_PARAM_COSETS][SED_MAX_STAGES];
  // pos[c * 64 + i]: bit position where bit i of x lands under coset
  // representative c (so P_c(x ^ d) = P_c(x) ^ P_c(d) is cheap for sparse d)
  uint8_t const* pos;
  // When cyc > 0, H = <g1> x <g2> (cyc = number of generators) is walked by
  // nested loops that apply the generators' two-term shift decompositions
  // held right here (kernel-parameter space): no memory traffic per image.
  uint32_t cyc;
  uint32_t cyc_ord[2];
  uint32_t cyc_phase[2];
  uint32_t cyc_rot[2][2];
  uint64_t cyc_mask[2][2];
  uint64_t mask;
  uint32_t n_bits;
  int32_t inv;  // 0 none, +1 / -1
  uint32_t L;
  uint32_t inv_phase;
  uint32_t n_cosets, n_h, n_stages, n_terms;
  uint64_t const* benes_mask;  // [n_cosets][n_stages]
  uint32_t const* benes_shift; // [n_stages]
  uint64_t const* h_mask;      // [n_h][n_terms]
  uint32_t const* h_rot;       // [n_h][n_terms]
  uint32_t const* coset_phase; // [n_cosets]
  uint32_t const* h_phase;     // [n_h]
  // Row structure of H (rows != 0): the word is n_rows blocks ("rows") of
  // row_bits bits, one generator rotates every row by the same amount, the
  // other (if n_rows > 1) shifts rows cyclically. rows == 1: row_bits <= 10,
  // smallest rotation of each row from a table; rows == 2: a single row
  // (chains), smallest rotation from the longest circular run of zeros.
  uint32_t rows;
  uint32_t row_bits, n_rows;
  uint32_t rot_phase, shift_phase;  // characters of the rotation / shift generators
  uint64_t row_mask;
  uint16_t const* row_min;     // [1 << row_bits] smallest rotation of a row
  uint16_t const* row_set;     // [1 << row_bits] rotations r reaching it (bit r)
  uint64_t const* rot_mask;    // [row_bits][2] two-term shift: rotate every row left by r
  uint32_t const* rot_rot;     // [row_bits][2]
  uint32_t const* rot_exp;     // [row_bits] exponent of the rotation generator
  uint64_t const* sh_mask;     // [n_rows][2] shift: image row j <- source row (j + t) mod n_rows
  uint32_t const* sh_rot;      // [n_rows][2]
  uint32_t const* sh_exp;      // [n_rows] exponent of the shift generator
  // Line tables (rows == 1, line_fast = 1): every row of every coset image
  // of x is a row or (on a square torus, line_cols = 1) a column of x, read
  // forwards or backwards from some start. The smallest rotation of an image
  // row is then a table lookup on that line of x: line_row[v] / line_col[v]
  // is the smallest of row_min over the orientations (and inversions) in
  // which the cosets present a row / column with bits v. Column j of x, as
  // a row value (bit r = bit r * row_bits + j of x), is
  // (((x >> j) & col_m) * col_k) >> col_s, masked to n_rows bits.
  uint32_t line_fast, line_cols, col_s;
  uint64_t col_m, col_k;
  uint16_t const* line_row;  // [1 << row_bits]
  uint16_t const* line_col;  // [1 << row_bits]
};

struct IndexView {
  uint64_t const* reps;
  uint64_t const* prefix;  // [(1 << bits) + 1]
  uint64_t D;
  uint32_t bits, shift;
};

template <class W>
SED_HD W rotl(W v, unsigned s) {
  constexpr unsigned B = sizeof(W) * 8;
#ifdef __CUDA_ARCH__
  if constexpr (B == 32) {
    return __funnelshift_l(v, v, s);
  } else {
    uint32_t lo = (uint32_t)v, hi = (uint32_t)(v >> 32);
    if (s & 32u) {
      uint32_t t = lo;
      lo = hi;
      hi = t;
    }
    uint32_t nhi = __funnelshift_l(lo, hi, s);
    uint32_t nlo = __funnelshift_l(hi, lo, s);
    return ((uint64_t)nhi << 32) | nlo;
  }
#else
  s &= B - 1;
  return s ? (W)((v << s) | (v >> (B - s))) : v;
#endif
}

template <class W>
SED_HD W benes_apply(W x, uint64_t const* masks, uint32_t const* shifts, unsigned n) {
  for (unsigned i = 0; i < n; ++i) {
    W const m = (W)masks[i];
    unsigned const s = shifts[i];
    W const t = ((x >> s) ^ x) & m;
    x ^= t ^ (t << s);
  }
  return x;
}

template <class W>
SED_HD W benes_fixed(W x, uint64_t const* m) {
  constexpr unsigned B = sizeof(W) * 8;
  constexpr unsigned L = B == 64 ? 6 : 5;
#pragma unroll
  for (unsigned i = 0; i < 2 * L - 1; ++i) {
    unsigned const s = i < L ? (B >> (i + 1)) : (B >> (2 * L - 1 - i));
    W const t = ((x >> s) ^ x) & (W)m[i];
    x ^= t ^ (t << s);
  }
  return x;
}

// Image of x under coset representative c.
template <class W>
SED_HD W coset_apply(W x, PlanView const& P, uint32_t c) {
  if (c == 0) return x;
  if (P.fixed_nets) return benes_fixed<W>(x, P.nets[c]);
  return benes_apply<W>(x, P.benes_mask + (uint64_t)c * P.n_stages, P.benes_shift, P.n_stages);
}

template <class W>
SED_HD W shift_apply(W y, uint64_t const* masks, uint32_t const* rots, unsigned n_terms) {
  W z = 0;
  for (unsigned t = 0; t < n_terms; ++t) z |= rotl<W>(y & (W)masks[t], rots[t]);
  return z;
}

SED_HD int __builtin_ctz_sed(uint32_t v) {
#ifdef __CUDA_ARCH__
  return __ffs((int)v) - 1;
#else
  return __builtin_ctz(v);
#endif
}
SED_HD int __builtin_ctzll_sed(uint64_t v) {
#ifdef __CUDA_ARCH__
  return __ffsll((long long)v) - 1;
#else
  return __builtin_ctzll(v);
#endif
}

SED_HD uint32_t add_phase(uint32_t a, uint32_t b, uint32_t L) {
  uint32_t s = a + b;
  return s >= L ? s - L : s;
}

template <class W>
struct Canon {
  W rep;
  uint32_t phase;  // character of the element mapping x to rep: exp(-2 pi i phase / L)
};

template <class W>
SED_HD W apply2(W y, uint64_t m0, uint64_t m1, unsigned r0, unsigned r1) {
  return rotl<W>(y & (W)m0, r0) | rotl<W>(y & (W)m1, r1);
}

// --- row-structured subgroup ------------------------------------------------
struct RowTab {
  uint16_t const* min;  // smallest rotation of a row
  uint16_t const* set;  // rotations reaching it
  uint16_t const* lrow = nullptr;  // line tables (PlanView::line_row / line_col), when staged
  uint16_t const* lcol = nullptr;
};
// Both routines enumerate the H-images (of y, and of ~y with inversion) that
// can be the smallest one: the smallest image has the smallest top row (most
// significant row_bits bits), so only (row, rotation) pairs reaching that top
// row can produce it. f(image, r, t, inverted) returns false to stop early.

template <class W>
SED_HD W rotl_n(W v, unsigned r, unsigned n, W mask) {
  return r ? (W)(((v << r) | (v >> (n - r))) & mask) : v;
}

template <class W>
SED_HD W rotr_n(W v, unsigned r, unsigned n, W mask) {
  return r ? (W)(((v >> r) | (v << (n - r))) & mask) : v;
}

// Row j (0 = top) of the candidate image that takes source row k of y to the
// top with rotation r; rows come from y (and ~y when inv).
template <class W>
SED_HD uint32_t cand_row(W y, PlanView const& P, uint32_t k, uint32_t j, uint32_t r, uint32_t invm) {
  uint32_t const src = k >= j ? k - j : k + P.n_rows - j;
  uint32_t const B = P.row_bits, rm = (uint32_t)P.row_mask;
  uint32_t const v = ((uint32_t)(y >> (src * B)) & rm) ^ invm;
  return r ? (((v << r) | (v >> (B - r))) & rm) : v;
}

// Lexicographic comparison, from the top row down, of the candidate image
// (source row k of y at the top, rotation r) with the word ref; rows 0..j0-1
// are known to be equal. Returns -1, 0 or +1.
template <class W>
SED_HD int cand_compare(W y, PlanView const& P, uint32_t k, uint32_t r, uint32_t invm, W ref, uint32_t j0) {
  uint32_t const B = P.row_bits, rm = (uint32_t)P.row_mask, R = P.n_rows;
  for (uint32_t j = j0; j < R; ++j) {
    uint32_t const a = cand_row<W>(y, P, k, j, r, invm);
    uint32_t const b = (uint32_t)(ref >> ((R - 1 - j) * B)) & rm;
    if (a != b) return a < b ? -1 : 1;
  }
  return 0;
}

// Full image for candidate (source row k to the top, rotation r, orientation).
template <class W>
SED_HD W cand_image(W y, W mask, PlanView const& P, uint32_t k, uint32_t r, uint32_t inv) {
  uint32_t const t = k + 1 == P.n_rows ? 0u : k + 1;
  W const yy = inv ? (W)(~y & mask) : y;
  W z = apply2<W>(yy, P.rot_mask[2 * r], P.rot_mask[2 * r + 1], P.rot_rot[2 * r], P.rot_rot[2 * r + 1]);
  return apply2<W>(z, P.sh_mask[2 * t], P.sh_mask[2 * t + 1], P.sh_rot[2 * t], P.sh_rot[2 * t + 1]);
}

// Smallest top row over the rows (and inverted rows) of y.
template <class W>
SED_HD uint32_t rows_min_top(W y, PlanView const& P, RowTab const& T) {
  uint32_t best = 0xFFFFFFFFu;
  uint32_t const rm = (uint32_t)P.row_mask;
  W v = y;
#pragma unroll
  for (uint32_t k = 0; k < SED_MAX_ROWS; ++k) {
    if (k < P.n_rows) {
      uint32_t const row = (uint32_t)v & rm;
      v >>= P.row_bits;
      uint32_t const a = T.min[row];
      best = a < best ? a : best;
      if (P.inv) {
        uint32_t const b = T.min[row ^ rm];
        best = b < best ? b : best;
      }
    }
  }
  return best;
}

// Single row of n bits (chains): rotations of v that bring a longest circular
// run of zeros to the top. Returns the run length and writes the run starts.
template <class W>
SED_HD uint32_t zero_runs(W v, unsigned n, W mask, W* starts) {
  W const Z = (W)(~v & mask);
  if (Z == 0) {  // no zeros: every rotation is the same word
    *starts = mask;
    return 0;
  }
  // pw[i]: starts of circular zero runs of length >= 2^i (fully unrolled, so
  // every index is a compile-time constant and pw stays in registers)
  W pw[7];
  pw[0] = Z;
  int top = 0;
#pragma unroll
  for (int i = 1; i < 7; ++i) {
    unsigned const len = 1u << (i - 1);
    pw[i] = 0;
    if (2 * len <= n && top == i - 1) {
      W const nxt = pw[i - 1] & rotr_n<W>(pw[i - 1], len, n, mask);
      if (nxt) {
        pw[i] = nxt;
        top = i;
      }
    }
  }
  W cur = pw[0];
#pragma unroll
  for (int i = 1; i < 7; ++i)
    if (top == i) cur = pw[i];
  uint32_t len = 1u << top;
#pragma unroll
  for (int j = 5; j >= 0; --j) {
    if (j < top) {
      uint32_t const s = 1u << j;
      if (len + s <= n) {
        W const t = cur & rotr_n<W>(pw[j], len, n, mask);
        if (t) {
          cur = t;
          len += s;
        }
      }
    }
  }
  *starts = cur;
  return len;
}

template <class W, class F>
SED_HD bool chain_each(W y, W mask, PlanView const& P, F&& f) {
  unsigned const n = P.row_bits;
  W s0, s1 = 0;
  uint32_t const k0 = zero_runs<W>(y, n, mask, &s0);
  uint32_t k1 = 0;
  if (P.inv) k1 = zero_runs<W>((W)(~y & mask), n, mask, &s1);
  for (uint32_t inv = 0; inv <= (P.inv ? 1u : 0u); ++inv) {
    uint32_t const k = inv ? k1 : k0;
    if (k < (inv ? k0 : k1)) continue;  // a longer leading run of zeros always wins
    W set = inv ? s1 : s0;
    W const yy = inv ? (W)(~y & mask) : y;
    while (set) {
      uint32_t const p = (uint32_t)__builtin_ctzll_sed((uint64_t)set);
      set &= set - 1;
      uint32_t const r = (n - k - p + 2 * n) % n;
      if (!f(rotl_n<W>(yy, r, n, mask), r, 0u, inv)) return false;
    }
  }
  return true;
}

#ifdef __CUDACC__
// Copies the row tables into shared memory (2048 uint16 slots) and returns
// them. Every thread of the block must call it.
// Line tables into sm[0 .. 2048) (rows == 1, line_fast); call before
// stage_rows, whose barrier publishes them, then attach with attach_lines.
__device__ __forceinline__ void stage_lines(PlanView const& P, uint16_t* sm) {
  if (P.rows == 1 && P.line_fast) {
    unsigned const n = 1u << P.row_bits;
    for (unsigned i = threadIdx.x; i < n; i += blockDim.x) {
      sm[i] = P.line_row[i];
      sm[1024 + i] = P.line_cols ? P.line_col[i] : (uint16_t)0;
    }
  }
}
__device__ __forceinline__ void attach_lines(PlanView const& P, uint16_t const* sm, RowTab& T) {
  if (P.rows == 1 && P.line_fast) {
    T.lrow = sm;
    T.lcol = sm + 1024;
  }
}

__device__ __forceinline__ RowTab stage_rows(PlanView const& P, uint16_t* sm) {
  if (P.rows == 1) {
    unsigned const n = 1u << P.row_bits;
    for (unsigned i = threadIdx.x; i < n; i += blockDim.x) {
      sm[i] = P.row_min[i];
      sm[1024 + i] = P.row_set[i];
    }
    __syncthreads();
    return {sm, sm + 1024};
  }
  return {P.row_min, P.row_set};
}
#endif

// Orbit minimum of x and the phase of an element mapping x onto it.
// img(c) returns the image of x under coset representative c.
template <class W, class Img>
SED_HD Canon<W> canonicalize_img(W x, PlanView const& P, RowTab const& T, Img&& img) {
  W best = x;
  W const mask = (W)P.mask;
  if (P.rows == 1) {
    // Per coset: the smallest top row any rotation/shift can reach (from the
    // row tables); cosets that cannot beat the best image's top row are
    // skipped, the others build every image with that top row in full.
    uint32_t const rm = (uint32_t)P.row_mask;
    uint32_t const top_shift = (P.n_rows - 1) * P.row_bits;
    uint32_t bc = 0, br = 0, bt = 0, binv = 0;
    for (uint32_t c = 0; c < P.n_cosets; ++c) {
      W const y = img(c);
      uint32_t rv[SED_MAX_ROWS];
      uint32_t top = 0xFFFFFFFFu;
      {
        W v = y;
#pragma unroll
        for (uint32_t k = 0; k < SED_MAX_ROWS; ++k) {
          if (k < P.n_rows) {
            rv[k] = (uint32_t)v & rm;
            v >>= P.row_bits;
            uint32_t const a = T.min[rv[k]];
            top = a < top ? a : top;
            if (P.inv) {
              uint32_t const b = T.min[rv[k] ^ rm];
              top = b < top ? b : top;
            }
          }
        }
      }
      if (top > (uint32_t)(best >> top_shift)) continue;
#pragma unroll
      for (uint32_t k = 0; k < SED_MAX_ROWS; ++k) {
        if (k >= P.n_rows) break;
        for (uint32_t inv = 0; inv <= (P.inv ? 1u : 0u); ++inv) {
          uint32_t const v = inv ? (rv[k] ^ rm) : rv[k];
          if (T.min[v] != top) continue;
          uint32_t set = T.set[v];
          while (set) {
            uint32_t const r = (uint32_t)__builtin_ctz_sed(set);
            set &= set - 1;
            W const z = cand_image<W>(y, mask, P, k, r, inv);
            if (z < best) {
              best = z;
              bc = c;
              br = r;
              bt = k + 1 == P.n_rows ? 0u : k + 1;
              binv = inv;
            }
          }
        }
      }
    }
    uint64_t ph = (uint64_t)P.coset_phase[bc] + (uint64_t)P.rot_exp[br] * P.rot_phase +
                  (uint64_t)P.sh_exp[bt] * P.shift_phase;
    if (binv) ph += P.inv_phase;
    return {best, (uint32_t)(ph % P.L)};
  }
  if (P.rows == 2) {
    uint32_t bc = 0, br = 0, binv = 0;
    for (uint32_t c = 0; c < P.n_cosets; ++c) {
      auto take = [&](W z, uint32_t r, uint32_t, uint32_t inv) {
        if (z < best) {
          best = z;
          bc = c;
          br = r;
          binv = inv;
        }
        return true;
      };
      chain_each<W>(img(c), mask, P, take);
    }
    uint64_t ph = (uint64_t)P.coset_phase[bc] + (uint64_t)P.rot_exp[br] * P.rot_phase;
    if (binv) ph += P.inv_phase;
    return {best, (uint32_t)(ph % P.L)};
  }
  if (P.cyc) {
    // candidate index: ((c * o1) + a) * o2 + b, bit 31 = inversion
    uint32_t const o1 = P.cyc_ord[0], o2 = P.cyc_ord[1];
    uint32_t bc = 0, cand = 0;
    for (uint32_t c = 0; c < P.n_cosets; ++c) {
      W y = img(c);
      for (uint32_t a = 0; a < o1; ++a) {
        W z = y;
        for (uint32_t b = 0; b < o2; ++b, ++cand) {
          if (z < best) {
            best = z;
            bc = cand;
          }
          if (P.inv) {
            W const zi = ~z & mask;
            if (zi < best) {
              best = zi;
              bc = cand | 0x80000000u;
            }
          }
          z = apply2<W>(z, P.cyc_mask[1][0], P.cyc_mask[1][1], P.cyc_rot[1][0], P.cyc_rot[1][1]);
        }
        y = apply2<W>(y, P.cyc_mask[0][0], P.cyc_mask[0][1], P.cyc_rot[0][0], P.cyc_rot[0][1]);
      }
    }
    uint32_t const k = bc & 0x7FFFFFFFu;
    uint32_t const c = k / (o1 * o2), rem = k % (o1 * o2);
    uint32_t const a = rem / o2, b = rem % o2;
    uint64_t ph = (uint64_t)P.coset_phase[c] + (uint64_t)a * P.cyc_phase[0] + (uint64_t)b * P.cyc_phase[1];
    if (bc >> 31) ph += P.inv_phase;
    return {best, (uint32_t)(ph % P.L)};
  }
  uint32_t bc = 0, bh = 0, binv = 0;
  for (uint32_t c = 0; c < P.n_cosets; ++c) {
    W const y = img(c);
    for (uint32_t h = 0; h < P.n_h; ++h) {
      W const z = shift_apply<W>(y, P.h_mask + (uint64_t)h * P.n_terms,
                                 P.h_rot + (uint64_t)h * P.n_terms, P.n_terms);
      if (z < best) {
        best = z;
        bc = c;
        bh = h;
        binv = 0;
      }
      if (P.inv) {
        W const zi = ~z & mask;
        if (zi < best) {
          best = zi;
          bc = c;
          bh = h;
          binv = 1;
        }
      }
    }
  }
  uint32_t ph = add_phase(P.coset_phase[bc], P.h_phase[bh], P.L);
  if (binv) ph = add_phase(ph, P.inv_phase, P.L);
  return {best, ph};
}

// Stabiliser order of x if x is a representative of the sector, else 0.
template <class W>
SED_HD uint32_t representative_weight(W x, PlanView const& P, RowTab const& T) {
  uint32_t S = 0;
  W const mask = (W)P.mask;
  if (P.rows == 1) {
    uint32_t const rm = (uint32_t)P.row_mask;
    uint32_t const xt = (uint32_t)(x >> ((P.n_rows - 1) * P.row_bits));
    if (T.lrow) {  // pass A from the lines of x: the image rows of all cosets at once
      W v = x;
#pragma unroll
      for (uint32_t k = 0; k < SED_MAX_ROWS; ++k) {
        if (k < P.n_rows) {
          if (T.lrow[(uint32_t)v & rm] < xt) return 0;
          v >>= P.row_bits;
        }
      }
      if (P.line_cols) {
#pragma unroll
        for (uint32_t j = 0; j < SED_MAX_ROWS; ++j) {
          if (j < P.row_bits) {
            uint64_t const col = ((((uint64_t)x >> j) & P.col_m) * P.col_k) >> P.col_s;
            if (T.lcol[(uint32_t)col & rm] < xt) return 0;
          }
        }
      }
    } else {
      for (uint32_t c = 0; c < P.n_cosets; ++c)  // pass A with early rejection
        if (rows_min_top<W>(coset_apply<W>(x, P, c), P, T) < xt) return 0;
    }
    for (uint32_t c = 0; c < P.n_cosets; ++c) {  // pass B: images whose top row equals x's
      W const y = coset_apply<W>(x, P, c);
      for (uint32_t k = 0; k < P.n_rows; ++k) {
        uint32_t const row = (uint32_t)(y >> (k * P.row_bits)) & rm;
        for (uint32_t inv = 0; inv <= (P.inv ? 1u : 0u); ++inv) {
          uint32_t const v = inv ? (row ^ rm) : row;
          if (T.min[v] != xt) continue;
          uint32_t set = T.set[v];
          while (set) {
            uint32_t const r = (uint32_t)__builtin_ctz_sed(set);
            set &= set - 1;
            int const cmp = cand_compare<W>(y, P, k, r, inv ? rm : 0u, x, 1);
            if (cmp < 0) return 0;
            if (cmp == 0) {
              uint32_t const t = k + 1 == P.n_rows ? 0u : k + 1;
              uint64_t ph = (uint64_t)P.coset_phase[c] + (uint64_t)P.rot_exp[r] * P.rot_phase +
                            (uint64_t)P.sh_exp[t] * P.shift_phase + (inv ? P.inv_phase : 0u);
              if (ph % P.L != 0) return 0;
              ++S;
            }
          }
        }
      }
    }
    return S;
  }
  if (P.rows == 2) {
    bool reject = false;
    for (uint32_t c = 0; c < P.n_cosets && !reject; ++c) {
      auto visit = [&](W z, uint32_t r, uint32_t, uint32_t inv) {
        if (z < x) {
          reject = true;
          return false;
        }
        if (z == x) {
          uint64_t ph = (uint64_t)P.coset_phase[c] + (uint64_t)P.rot_exp[r] * P.rot_phase +
                        (inv ? P.inv_phase : 0u);
          if (ph % P.L != 0) {
            reject = true;
            return false;
          }
          ++S;
        }
        return true;
      };
      chain_each<W>(coset_apply<W>(x, P, c), mask, P, visit);
    }
    return reject ? 0 : S;
  }
  if (P.cyc) {
    uint32_t const o1 = P.cyc_ord[0], o2 = P.cyc_ord[1];
    for (uint32_t c = 0; c < P.n_cosets; ++c) {
      W y = coset_apply<W>(x, P, c);
      uint32_t pa = P.coset_phase[c];
      for (uint32_t a = 0; a < o1; ++a) {
        W z = y;
        uint32_t pb = pa;
        for (uint32_t b = 0; b < o2; ++b) {
          if (z < x) return 0;
          if (z == x) {
            if (pb != 0) return 0;
            ++S;
          }
          if (P.inv) {
            W const zi = ~z & mask;
            if (zi < x) return 0;
            if (zi == x) {
              if (add_phase(pb, P.inv_phase, P.L) != 0) return 0;
              ++S;
            }
          }
          z = apply2<W>(z, P.cyc_mask[1][0], P.cyc_mask[1][1], P.cyc_rot[1][0], P.cyc_rot[1][1]);
          pb = add_phase(pb, P.cyc_phase[1], P.L);
        }
        y = apply2<W>(y, P.cyc_mask[0][0], P.cyc_mask[0][1], P.cyc_rot[0][0], P.cyc_rot[0][1]);
        pa = add_phase(pa, P.cyc_phase[0], P.L);
      }
    }
    return S;
  }
  for (uint32_t c = 0; c < P.n_cosets; ++c) {
    W const y = coset_apply<W>(x, P, c);
    for (uint32_t h = 0; h < P.n_h; ++h) {
      W const z = shift_apply<W>(y, P.h_mask + (uint64_t)h * P.n_terms,
                                 P.h_rot + (uint64_t)h * P.n_terms, P.n_terms);
      if (z < x) return 0;
      if (z == x) {
        if (add_phase(P.coset_phase[c], P.h_phase[h], P.L) != 0) return 0;
        ++S;
      }
      if (P.inv) {
        W const zi = ~z & mask;
        if (zi < x) return 0;
        if (zi == x) {
          if (add_phase(add_phase(P.coset_phase[c], P.h_phase[h], P.L), P.inv_phase, P.L) != 0)
            return 0;
          ++S;
        }
      }
    }
  }
  return S;
}

template <class W>
SED_HD Canon<W> canonicalize(W x, PlanView const& P, RowTab const& T) {
  return canonicalize_img<W>(x, P, T, [&](uint32_t c) { return coset_apply<W>(x, P, c); });
}
template <class W>
SED_HD Canon<W> canonicalize(W x, PlanView const& P) {
  return canonicalize<W>(x, P, RowTab{P.row_min, P.row_set});
}
template <class W>
SED_HD uint32_t representative_weight(W x, PlanView const& P) {
  return representative_weight<W>(x, P, RowTab{P.row_min, P.row_set});
}

// ------------------------------------------------ fixed-weight word order ---
// Words of n bits with popcount w, in increasing numeric order (colex order
// of the set-bit positions). binom is a [65][65] table of C(i, j).
SED_HD uint64_t unrank_word(uint64_t k, unsigned n, int w, uint64_t const* binom) {
  if (w < 0) return k;
  uint64_t x = 0;
  unsigned m = (unsigned)w;
  int c = (int)n - 1;
  while (m > 0) {
    while (binom[c * 65 + m] > k) --c;
    k -= binom[c * 65 + m];
    x |= (uint64_t)1 << c;
    --m;
    --c;
  }
  return x;
}

SED_HD uint64_t next_same_weight(uint64_t x) {
  uint64_t const t = x | (x - 1);
#ifdef __CUDA_ARCH__
  unsigned const tz = (unsigned)__ffsll((long long)x) - 1u;
#else
  unsigned const tz = (unsigned)__builtin_ctzll(x);
#endif
  uint64_t const nt = ~t;
  uint64_t const low_nt = nt & (0 - nt);
  uint64_t const tail = tz + 1 >= 64 ? 0 : ((low_nt - 1) >> (tz + 1));
  return (t + 1) | tail;
}

// Index of representative rho in the sorted list, or -1.
SED_HD int64_t find_index(uint64_t rho, IndexView const& I) {
  uint64_t const key = rho >> I.shift;
  if (key >= ((uint64_t)1 << I.bits)) return -1;
  uint64_t lo = I.prefix[key];
  uint64_t const end = I.prefix[key + 1];
  uint64_t hi = end;
  while (lo < hi) {
    uint64_t const mid = (lo + hi) >> 1;
    if (I.reps[mid] < rho)
      lo = mid + 1;
    else
      hi = mid;
  }
  return (lo < end && I.reps[lo] == rho) ? (int64_t)lo : -1;
}

// --------------------------------------------------------------- terms ---
// Flattened interaction terms. For every k-site tuple the local index of a
// configuration r is a = sum_m bit(site_m) << (k-1-m); row a of the term's
// matrix gives the diagonal value and the off-diagonal columns a' with
// values <r|H|s> (src/SpinED/Internal.hs:258-270).
struct TermsView {
  uint32_t n_tuples;
  uint32_t const* tuple_term;   // [n_tuples] term index | k << 16
  uint32_t const* tuple_sites;  // [n_tuples] 4 x 8-bit site indices
  double const* diag;           // [n_terms][16][2]
  uint8_t const* n_off;         // [n_terms][16]
  uint8_t const* off_col;       // [n_terms][16][16]
  uint16_t const* off_vid;      // [n_terms][16][16] index into off_val
  double const* off_val;        // [n_values][2]
};

SED_HD unsigned local_index(uint64_t r, uint32_t sites, unsigned k) {
  unsigned a = 0;
  for (unsigned m = 0; m < k; ++m) a = (a << 1) | (unsigned)((r >> ((sites >> (8 * m)) & 0xFFu)) & 1u);
  return a;
}

SED_HD uint64_t replace_local(uint64_t r, uint32_t sites, unsigned k, unsigned a) {
  for (unsigned m = 0; m < k; ++m) {
    unsigned const s = (sites >> (8 * m)) & 0xFFu;
    uint64_t const bit = (uint64_t)((a >> (k - 1 - m)) & 1u);
    r = (r & ~((uint64_t)1 << s)) | (bit << s);
  }
  return r;
}

}  // namespace sed
