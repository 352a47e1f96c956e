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

struct PlanView {
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
SED_HD W shift_apply(W y, uint64_t const* masks, uint32_t const* rots, unsigned n_terms) {
  W z = 0;
  for (unsigned t = 0; t < n_terms; ++t) z |= rotl<W>(y & (W)masks[t], rots[t]);
  return z;
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

// Orbit minimum of x and the phase of an element mapping x onto it.
template <class W>
SED_HD Canon<W> canonicalize(W x, PlanView const& P) {
  W best = x;
  W const mask = (W)P.mask;
  if (P.cyc) {
    // candidate index: ((c * o1) + a) * o2 + b, bit 31 = inversion
    uint32_t const o1 = P.cyc_ord[0], o2 = P.cyc_ord[1];
    uint32_t bc = 0, cand = 0;
    for (uint32_t c = 0; c < P.n_cosets; ++c) {
      W y = benes_apply<W>(x, P.benes_mask + (uint64_t)c * P.n_stages, P.benes_shift,
                           c == 0 ? 0u : P.n_stages);
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
    W const y = benes_apply<W>(x, P.benes_mask + (uint64_t)c * P.n_stages, P.benes_shift,
                               c == 0 ? 0u : P.n_stages);
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
SED_HD uint32_t representative_weight(W x, PlanView const& P) {
  uint32_t S = 0;
  W const mask = (W)P.mask;
  if (P.cyc) {
    uint32_t const o1 = P.cyc_ord[0], o2 = P.cyc_ord[1];
    for (uint32_t c = 0; c < P.n_cosets; ++c) {
      W y = benes_apply<W>(x, P.benes_mask + (uint64_t)c * P.n_stages, P.benes_shift,
                           c == 0 ? 0u : P.n_stages);
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
    W const y = benes_apply<W>(x, P.benes_mask + (uint64_t)c * P.n_stages, P.benes_shift,
                               c == 0 ? 0u : P.n_stages);
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
