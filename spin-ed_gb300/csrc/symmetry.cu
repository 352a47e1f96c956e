// symmetry.cu — symmetries, groups and the per-basis symmetry plan (host).
//
// ls_create_symmetry / ls_create_group replace the lattice-symmetries calls
// bound at src/SpinED/Internal.hs:69-79,120-127. The plan (canon.cuh) splits
// the closed group into cosets of a subgroup of cheap, shift-like elements and
// routes every coset representative through a Benes network.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <unordered_map>

#include "sed_internal.hpp"

namespace sed {
namespace {

constexpr unsigned kMaxGroup = 65536;

bool is_permutation(unsigned n, unsigned const* p) {
  if (n == 0 || n > 64) return false;
  bool seen[64] = {false};
  for (unsigned i = 0; i < n; ++i) {
    if (p[i] >= n || seen[p[i]]) return false;
    seen[p[i]] = true;
  }
  return true;
}

unsigned periodicity_of(std::vector<uint8_t> const& p) {
  unsigned const n = (unsigned)p.size();
  std::vector<bool> seen(n, false);
  unsigned per = 1;
  for (unsigned i = 0; i < n; ++i) {
    if (seen[i]) continue;
    unsigned len = 0;
    for (unsigned j = i; !seen[j]; j = p[j]) {
      seen[j] = true;
      ++len;
    }
    per = per / std::gcd(per, len) * len;
  }
  return per;
}

std::string key_of(uint8_t const* p, unsigned n) { return std::string((char const*)p, n); }

// Applies y_i = x_{p[i]} bit by bit (the defining convention).
uint64_t apply_naive(std::vector<uint8_t> const& p, uint64_t x) {
  uint64_t y = 0;
  for (unsigned i = 0; i < p.size(); ++i) y |= ((x >> p[i]) & 1u) << i;
  return y;
}

// --- Benes routing (looping algorithm) -------------------------------------
// dst[i] is the output position of the bit at input position i, over a
// block of `size` positions starting at `base`. Stage `level` (distance
// size/2) and its mirror stage receive this block's swap masks.
void route(std::vector<int> const& dst, unsigned base, unsigned size, unsigned level,
           unsigned n_levels, std::vector<uint64_t>& masks) {
  if (size == 2) {
    if (dst[0] == 1) masks[level] |= (uint64_t)1 << base;
    return;
  }
  unsigned const h = size / 2;
  std::vector<int> inv(size), color(size, -1);
  for (unsigned i = 0; i < size; ++i) inv[dst[i]] = (int)i;
  for (unsigned start = 0; start < size; ++start) {
    if (color[start] != -1) continue;
    unsigned i = start;
    int c = 0;
    while (color[i] == -1) {
      color[i] = c;
      unsigned const ip = i ^ h;  // input-pair partner
      color[ip] = 1 - c;
      i = (unsigned)inv[(unsigned)dst[ip] ^ h];  // output-pair partner of ip
    }
  }
  std::vector<int> lower(h), upper(h);
  unsigned const last = 2 * n_levels - 2 - level;
  for (unsigned j = 0; j < h; ++j) {
    unsigned const e0 = color[j] == 0 ? j : j + h;
    unsigned const e1 = e0 ^ h;
    if (color[j] == 1) masks[level] |= (uint64_t)1 << (base + j);
    lower[j] = dst[e0] & (int)(h - 1);
    upper[j] = dst[e1] & (int)(h - 1);
  }
  for (unsigned d = 0; d < h; ++d) {
    // The colour-0 element of output pair d leaves the lower sub-network at d.
    unsigned const e_lo = (unsigned)inv[d];
    unsigned const e_hi = (unsigned)inv[d + h];
    unsigned const zero_el = color[e_lo] == 0 ? e_lo : e_hi;
    if ((unsigned)dst[zero_el] == d + h) masks[last] |= (uint64_t)1 << (base + d);
  }
  route(lower, base, h, level + 1, n_levels, masks);
  route(upper, base + h, h, level + 1, n_levels, masks);
}

// Benes masks (in application order) for permutation p on `width` bits.
std::vector<uint64_t> benes_masks(std::vector<uint8_t> const& p, unsigned width) {
  unsigned n_levels = 0;
  while ((1u << n_levels) < width) ++n_levels;
  std::vector<int> dst(width);
  for (unsigned i = 0; i < width; ++i) dst[i] = (int)i;
  for (unsigned i = 0; i < p.size(); ++i) dst[p[i]] = (int)i;  // bit p[i] lands on i
  std::vector<uint64_t> masks(2 * n_levels - 1, 0);
  route(dst, 0, width, 0, n_levels, masks);
  return masks;
}

std::vector<uint32_t> benes_shifts(unsigned width) {
  unsigned n_levels = 0;
  while ((1u << n_levels) < width) ++n_levels;
  std::vector<uint32_t> s(2 * n_levels - 1);
  for (unsigned l = 0; l < n_levels; ++l) {
    s[l] = width >> (l + 1);
    s[2 * n_levels - 2 - l] = width >> (l + 1);
  }
  return s;
}

// Shift decomposition: groups bits by displacement; returns false if more
// than max_terms displacements are needed.
bool shift_terms(std::vector<uint8_t> const& p, unsigned width, unsigned max_terms,
                 std::vector<uint64_t>& masks, std::vector<uint32_t>& rots) {
  masks.clear();
  rots.clear();
  for (unsigned i = 0; i < p.size(); ++i) {
    int const d = (int)i - (int)p[i];
    uint32_t const r = (uint32_t)((d % (int)width + (int)width) % (int)width);
    auto it = std::find(rots.begin(), rots.end(), r);
    size_t idx = (size_t)(it - rots.begin());
    if (it == rots.end()) {
      if (rots.size() == max_terms) return false;
      rots.push_back(r);
      masks.push_back(0);
    }
    masks[idx] |= (uint64_t)1 << p[i];
  }
  return true;
}

}  // namespace

// Self-check of the structured plan (cyclic-product walk, row and line
// tables) against the plan's explicit element list on 256 random words and
// their representatives (about 3 ms on the host).
int check_plan(SymPlanHost const& out) {
  unsigned const width = out.n_bits <= 32 ? 32u : 64u;
  if (out.cyc) {
    PlanView vx = out.view();
    PlanView ve = vx;
    ve.cyc = 0;
    ve.rows = 0;
    uint64_t rng = 0x9E3779B97F4A7C15ull;
    for (int t = 0; t < 256; ++t) {  // 256 random words and their representatives (about 3 ms)
      rng ^= rng << 13;
      rng ^= rng >> 7;
      rng ^= rng << 17;
      uint64_t const x = rng & out.mask;
      bool same;
      if (width == 32) {
        auto c1 = canonicalize<uint32_t>((uint32_t)x, vx), c2 = canonicalize<uint32_t>((uint32_t)x, ve);
        uint32_t const w1 = representative_weight<uint32_t>((uint32_t)x, vx);
        uint32_t const w2 = representative_weight<uint32_t>((uint32_t)x, ve);
        same = c1.rep == c2.rep && w1 == w2 &&
               (representative_weight<uint32_t>(c2.rep, ve) == 0 || c1.phase == c2.phase);
        uint32_t const r = c2.rep;  // the representative itself: weights must agree too
        same = same && representative_weight<uint32_t>(r, vx) == representative_weight<uint32_t>(r, ve);
      } else {
        auto c1 = canonicalize<uint64_t>(x, vx), c2 = canonicalize<uint64_t>(x, ve);
        uint32_t const w1 = representative_weight<uint64_t>(x, vx);
        uint32_t const w2 = representative_weight<uint64_t>(x, ve);
        same = c1.rep == c2.rep && w1 == w2 &&
               (representative_weight<uint64_t>(c2.rep, ve) == 0 || c1.phase == c2.phase);
        uint64_t const r = c2.rep;
        same = same && representative_weight<uint64_t>(r, vx) == representative_weight<uint64_t>(r, ve);
      }
      if (!same) return fail(LS_SYSTEM_ERROR, "structured subgroup walk disagrees with the explicit list");
      if (out.line_fast) {  // the line-table test of the row path against the explicit list
        RowTab const TL{out.row_min.data(), out.row_set.data(), out.line_row.data(),
                        out.line_cols ? out.line_col.data() : nullptr};
        uint64_t const r = canonicalize<uint64_t>(x, ve).rep;
        bool const lines_same =
            width == 32
                ? representative_weight<uint32_t>((uint32_t)x, vx, TL) == representative_weight<uint32_t>((uint32_t)x, ve) &&
                      representative_weight<uint32_t>((uint32_t)r, vx, TL) ==
                          representative_weight<uint32_t>((uint32_t)r, ve)
                : representative_weight<uint64_t>(x, vx, TL) == representative_weight<uint64_t>(x, ve) &&
                      representative_weight<uint64_t>(r, vx, TL) == representative_weight<uint64_t>(r, ve);
        if (!lines_same) return fail(LS_SYSTEM_ERROR, "line tables disagree with the explicit list");
      }
    }
  }
  return LS_SUCCESS;
}

int build_plan(GroupData const& group, unsigned n_bits, int spin_inversion, SymPlanHost& out, bool self_check) {
  unsigned const width = n_bits <= 32 ? 32u : 64u;
  out = SymPlanHost{};
  out.n_bits = n_bits;
  out.mask = n_bits == 64 ? ~(uint64_t)0 : (((uint64_t)1 << n_bits) - 1);
  out.inv = spin_inversion;
  unsigned const scale = (spin_inversion == -1 && (group.L % 2)) ? 2u : 1u;
  out.L = group.L * scale;
  out.inv_phase = spin_inversion == -1 ? out.L / 2 : 0;

  // Elements of the group as permutations on n_bits sites.
  unsigned const G = group.n ? group.size() : 1u;
  std::vector<std::vector<uint8_t>> elems(G);
  std::vector<uint32_t> phase(G, 0);
  std::unordered_map<std::string, unsigned> index;
  for (unsigned g = 0; g < G; ++g) {
    elems[g].resize(n_bits);
    if (group.n)
      std::memcpy(elems[g].data(), group.perms.data() + (size_t)g * n_bits, n_bits);
    else
      for (unsigned i = 0; i < n_bits; ++i) elems[g][i] = (uint8_t)i;
    phase[g] = group.n ? (group.phase[g] * scale) % out.L : 0;
    index.emplace(key_of(elems[g].data(), n_bits), g);
  }
  out.group_order = G * (spin_inversion ? 2u : 1u);

  auto compose = [&](std::vector<uint8_t> const& first, std::vector<uint8_t> const& then) {
    // apply `first`, then `then`: z_i = x_{first[then[i]]}
    std::vector<uint8_t> c(n_bits);
    for (unsigned i = 0; i < n_bits; ++i) c[i] = first[then[i]];
    return c;
  };
  auto closure_of = [&](std::vector<unsigned> const& gens) {
    std::vector<unsigned> H{0};
    std::vector<bool> in(G, false);
    in[0] = true;
    for (size_t head = 0; head < H.size(); ++head)
      for (unsigned g : gens) {
        auto c = compose(elems[H[head]], elems[g]);
        unsigned k = index.at(key_of(c.data(), n_bits));
        if (!in[k]) {
          in[k] = true;
          H.push_back(k);
        }
      }
    return H;
  };

  // Candidate subgroup H: closure of the cheap generators (two displacements).
  std::vector<unsigned> cheap;
  for (auto const& s : group.generators) {
    std::vector<uint64_t> m;
    std::vector<uint32_t> r;
    if (s.perm.size() == n_bits && shift_terms(s.perm, width, 2, m, r))
      cheap.push_back(index.at(key_of(s.perm.data(), n_bits)));
  }
  auto all_cheap = [&](std::vector<unsigned> const& H) {
    std::vector<uint64_t> m;
    std::vector<uint32_t> r;
    for (unsigned h : H)
      if (!shift_terms(elems[h], width, SED_MAX_TERMS, m, r)) return false;
    return true;
  };
  std::vector<unsigned> H{0};
  if (!cheap.empty()) {
    auto Hc = closure_of(cheap);
    if (all_cheap(Hc)) {
      H = Hc;
    } else {
      for (unsigned g : cheap) {
        auto Hg = closure_of({g});
        if (Hg.size() > H.size() && all_cheap(Hg)) H = Hg;
      }
    }
  }
  // Right cosets H p.
  std::vector<bool> covered(G, false);
  std::vector<unsigned> cosets;
  for (unsigned g = 0; g < G; ++g) {
    if (covered[g]) continue;
    cosets.push_back(g);
    for (unsigned h : H) {
      auto c = compose(elems[g], elems[h]);
      unsigned k = index.at(key_of(c.data(), n_bits));
      if (add_phase(phase[h], phase[g], out.L) != phase[k])
        return fail(LS_INCOMPATIBLE_SYMMETRIES, "character is not a homomorphism on the group");
      covered[k] = true;
    }
  }
  if (cosets.size() * H.size() != G)
    return fail(LS_SYSTEM_ERROR, "coset decomposition of the symmetry group failed");

  // If H does not pay for itself, treat every element as a coset.
  unsigned const stage_cost = width == 32 ? 4 : 8;
  unsigned const term_cost = width == 32 ? 3 : 6;
  {
    unsigned terms = 1;
    std::vector<uint64_t> m;
    std::vector<uint32_t> r;
    for (unsigned h : H) {
      shift_terms(elems[h], width, SED_MAX_TERMS, m, r);
      terms = std::max<unsigned>(terms, (unsigned)r.size());
    }
    unsigned const stages = 2 * (width == 32 ? 5u : 6u) - 1;
    double const with_h = (double)cosets.size() * stages * stage_cost + (double)G * terms * term_cost;
    double const without = (double)G * stages * stage_cost + (double)G * term_cost;
    if (without < with_h && H.size() > 1) {
      H = {0};
      cosets.resize(G);
      std::iota(cosets.begin(), cosets.end(), 0u);
    }
  }

  // H as a product of at most two cyclic groups of two-term generators.
  unsigned cyc_g[2] = {0, 0};
  if (H.size() > 1) {
    auto order_of = [&](unsigned g) { return (unsigned)closure_of({g}).size(); };
    auto two_terms = [&](unsigned g, std::vector<uint64_t>& m, std::vector<uint32_t>& r) {
      return shift_terms(elems[g], width, 2, m, r);
    };
    std::vector<unsigned> cand;
    for (unsigned g : cheap)
      if (std::find(H.begin(), H.end(), g) != H.end()) cand.push_back(g);
    unsigned g1 = 0, g2 = 0;
    bool found = false;
    for (unsigned a : cand)
      if (!found && order_of(a) == H.size()) {
        g1 = a;
        g2 = 0;
        found = true;
      }
    for (size_t i = 0; i < cand.size() && !found; ++i)
      for (size_t j = i + 1; j < cand.size() && !found; ++j) {
        unsigned const a = cand[i], b = cand[j];
        if (compose(elems[a], elems[b]) != compose(elems[b], elems[a])) continue;
        if ((size_t)order_of(a) * order_of(b) == H.size() && closure_of({a, b}).size() == H.size()) {
          g1 = a;
          g2 = b;
          found = true;
        }
      }
    if (found) {
      cyc_g[0] = g1;
      cyc_g[1] = g2;
      unsigned const gens[2] = {g1, g2};
      for (int q = 0; q < 2; ++q) {
        std::vector<uint64_t> m;
        std::vector<uint32_t> r;
        two_terms(gens[q], m, r);
        out.cyc_ord[q] = gens[q] ? order_of(gens[q]) : 1u;
        out.cyc_phase[q] = phase[gens[q]];
        for (size_t t = 0; t < 2; ++t) {
          out.cyc_mask[q][t] = t < m.size() ? m[t] : 0;
          out.cyc_rot[q][t] = t < r.size() ? r[t] : 0;
        }
        if (!gens[q]) {  // identity: keep every bit in place
          out.cyc_mask[q][0] = out.mask;
          out.cyc_mask[q][1] = 0;
          out.cyc_rot[q][0] = out.cyc_rot[q][1] = 0;
        }
      }
      // Check: g1^a g2^b runs over H exactly once with the closure's phases.
      std::vector<bool> seen(G, false);
      std::vector<uint8_t> pa = elems[0];
      bool ok = true;
      for (unsigned a = 0; a < out.cyc_ord[0] && ok; ++a) {
        std::vector<uint8_t> pb = pa;
        for (unsigned b = 0; b < out.cyc_ord[1] && ok; ++b) {
          unsigned const k = index.at(key_of(pb.data(), n_bits));
          uint64_t const want = ((uint64_t)a * out.cyc_phase[0] + (uint64_t)b * out.cyc_phase[1]) % out.L;
          if (seen[k] || phase[k] != want || std::find(H.begin(), H.end(), k) == H.end()) ok = false;
          seen[k] = true;
          pb = compose(pb, elems[g2]);
        }
        pa = compose(pa, elems[g1]);
      }
      out.cyc = ok ? (g2 ? 2u : 1u) : 0u;
    }
  }

  // H as shift decompositions.
  out.n_h = (unsigned)H.size();
  out.n_terms = 1;
  std::vector<std::vector<uint64_t>> hm(H.size());
  std::vector<std::vector<uint32_t>> hr(H.size());
  for (size_t i = 0; i < H.size(); ++i) {
    shift_terms(elems[H[i]], width, SED_MAX_TERMS, hm[i], hr[i]);
    out.n_terms = std::max<unsigned>(out.n_terms, (unsigned)hr[i].size());
  }
  out.h_mask.assign((size_t)out.n_h * out.n_terms, 0);
  out.h_rot.assign((size_t)out.n_h * out.n_terms, 0);
  out.h_phase.resize(out.n_h);
  for (size_t i = 0; i < H.size(); ++i) {
    for (size_t t = 0; t < hr[i].size(); ++t) {
      out.h_mask[i * out.n_terms + t] = hm[i][t];
      out.h_rot[i * out.n_terms + t] = hr[i][t];
    }
    out.h_phase[i] = phase[H[i]];
  }
  // Cosets as Benes networks; drop stages that are empty for every coset.
  out.n_cosets = (unsigned)cosets.size();
  auto shifts = benes_shifts(width);
  std::vector<std::vector<uint64_t>> nets(cosets.size());
  std::vector<bool> used(shifts.size(), false);
  for (size_t c = 0; c < cosets.size(); ++c) {
    nets[c] = benes_masks(elems[cosets[c]], width);
    for (size_t s = 0; s < shifts.size(); ++s)
      if (nets[c][s]) used[s] = true;
  }
  out.pos.assign(cosets.size() * 64, 0);
  for (size_t c = 0; c < cosets.size(); ++c)
    for (unsigned j = 0; j < n_bits; ++j) out.pos[c * 64 + elems[cosets[c]][j]] = (uint8_t)j;  // bit p[j] -> j
  out.full_nets.assign(cosets.size() * SED_MAX_STAGES, 0);
  for (size_t c = 0; c < cosets.size(); ++c)
    for (size_t st = 0; st < shifts.size(); ++st) out.full_nets[c * SED_MAX_STAGES + st] = nets[c][st];
  out.benes_shift.clear();
  for (size_t s = 0; s < shifts.size(); ++s)
    if (used[s]) out.benes_shift.push_back(shifts[s]);
  out.n_stages = (unsigned)out.benes_shift.size();
  out.benes_mask.assign((size_t)out.n_cosets * out.n_stages, 0);
  out.coset_phase.resize(out.n_cosets);
  for (size_t c = 0; c < cosets.size(); ++c) {
    unsigned q = 0;
    for (size_t s = 0; s < shifts.size(); ++s)
      if (used[s]) out.benes_mask[c * out.n_stages + q++] = nets[c][s];
    out.coset_phase[c] = phase[cosets[c]];
  }
  // Verify every network and decomposition against the defining action.
  PlanView const v = out.view();
  for (size_t c = 0; c < cosets.size(); ++c)
    for (unsigned bit = 0; bit < n_bits; ++bit) {
      uint64_t const x = (uint64_t)1 << bit;
      uint64_t const want = apply_naive(elems[cosets[c]], x);
      uint64_t const got =
          width == 32
              ? (uint64_t)benes_apply<uint32_t>((uint32_t)x, v.benes_mask + c * v.n_stages,
                                                v.benes_shift, c == 0 ? 0 : v.n_stages)
              : benes_apply<uint64_t>(x, v.benes_mask + c * v.n_stages, v.benes_shift,
                                      c == 0 ? 0 : v.n_stages);
      if (want != got) return fail(LS_SYSTEM_ERROR, "Benes network routing failed");
    }
  for (size_t i = 0; i < H.size(); ++i)
    for (unsigned bit = 0; bit < n_bits; ++bit) {
      uint64_t const x = (uint64_t)1 << bit;
      uint64_t const want = apply_naive(elems[H[i]], x);
      uint64_t const got =
          width == 32 ? (uint64_t)shift_apply<uint32_t>((uint32_t)x, v.h_mask + i * v.n_terms,
                                                        v.h_rot + i * v.n_terms, v.n_terms)
                      : shift_apply<uint64_t>(x, v.h_mask + i * v.n_terms, v.h_rot + i * v.n_terms,
                                              v.n_terms);
      if (want != got) return fail(LS_SYSTEM_ERROR, "shift decomposition failed");
    }
  // Row structure: a rotation within rows of B bits (and a cyclic shift of rows).
  if (out.cyc) {
    unsigned const gens[2] = {cyc_g[0], cyc_g[1]};
    auto rotation_rows = [&](unsigned g, unsigned& B) -> bool {  // +-1 rotation inside rows
      B = closure_of({g}).size();
      if (B < 2 || n_bits % B) return false;
      int d = -1;
      for (unsigned i = 0; i < n_bits; ++i) {
        unsigned const q = elems[g][i];
        if (q / B != i / B) return false;
        int const di = (int)((q % B + B - i % B) % B);
        if (d < 0) d = di;
        if (di != d) return false;
      }
      return d == 1 || d == (int)B - 1;
    };
    auto shift_rows = [&](unsigned g, unsigned B) -> bool {  // +-B shift of the whole word
      unsigned const R = n_bits / B;
      if (closure_of({g}).size() != R) return false;
      for (int sgn : {1, -1}) {
        bool ok = true;
        for (unsigned i = 0; i < n_bits && ok; ++i)
          ok = elems[g][i] == (unsigned)(((int)i + sgn * (int)B + 2 * (int)n_bits) % (int)n_bits);
        if (ok) return true;
      }
      return false;
    };
    unsigned rot_g = 0, sh_g = 0, B = 0;
    bool found = false;
    if (out.cyc == 1 && rotation_rows(gens[0], B) && B == n_bits) {
      rot_g = gens[0];
      found = true;
      out.rows = 2;
    } else if (out.cyc == 2) {
      for (int q = 0; q < 2 && !found; ++q) {
        unsigned Bq = 0;
        if (rotation_rows(gens[q], Bq) && Bq <= 10 && Bq < n_bits && shift_rows(gens[1 - q], Bq)) {
          rot_g = gens[q];
          sh_g = gens[1 - q];
          B = Bq;
          found = true;
          out.rows = 1;
        }
      }
    }
    if (found && n_bits / B > SED_MAX_ROWS) found = false, out.rows = 0;
    if (found) {
      out.row_bits = B;
      out.n_rows = n_bits / B;
      out.row_mask = B == 64 ? ~(uint64_t)0 : (((uint64_t)1 << B) - 1);
      out.rot_phase = phase[rot_g];
      out.shift_phase = sh_g ? phase[sh_g] : 0u;
      out.rot_mask.assign(2 * B, 0);
      out.rot_rot.assign(2 * B, 0);
      out.rot_exp.assign(B, 0);
      out.sh_mask.assign(2 * out.n_rows, 0);
      out.sh_rot.assign(2 * out.n_rows, 0);
      out.sh_exp.assign(out.n_rows, 0);
      bool ok = true;
      std::vector<uint8_t> pw = elems[0];
      for (unsigned a = 0; a < B && ok; ++a) {  // powers of the rotation generator
        unsigned q = 0;
        while (pw[q] != 0) ++q;  // where bit 0 of the source lands
        unsigned const r = q % B;
        std::vector<uint64_t> m;
        std::vector<uint32_t> rr;
        ok = q < B && shift_terms(pw, width, 2, m, rr);
        if (ok) {
          out.rot_exp[r] = a;
          for (size_t t = 0; t < m.size(); ++t) {
            out.rot_mask[2 * r + t] = m[t];
            out.rot_rot[2 * r + t] = rr[t];
          }
        }
        pw = compose(pw, elems[rot_g]);
      }
      pw = elems[0];
      for (unsigned b = 0; b < out.n_rows && ok; ++b) {  // powers of the shift generator
        unsigned q = 0;
        while (pw[q] != 0) ++q;
        unsigned const t = (out.n_rows - q / B) % out.n_rows;
        std::vector<uint64_t> m;
        std::vector<uint32_t> rr;
        ok = shift_terms(pw, width, 2, m, rr);
        if (ok) {
          out.sh_exp[t] = b;
          for (size_t k = 0; k < m.size(); ++k) {
            out.sh_mask[2 * t + k] = m[k];
            out.sh_rot[2 * t + k] = rr[k];
          }
        }
        if (sh_g) pw = compose(pw, elems[sh_g]);
      }
      if (out.rows == 2) {  // no shift generator: the single "shift" is the identity
        out.sh_mask[0] = out.mask;
        out.sh_mask[1] = 0;
        out.sh_rot[0] = out.sh_rot[1] = 0;
        out.sh_exp[0] = 0;
      }
      if (out.rows == 1) {
        unsigned const nv = 1u << B;
        out.row_min.assign(nv, 0);
        out.row_set.assign(nv, 0);
        for (unsigned v = 0; v < nv; ++v) {
          unsigned best = ~0u, set = 0;
          for (unsigned r = 0; r < B; ++r) {
            unsigned const w = r ? (((v << r) | (v >> (B - r))) & (nv - 1)) : v;
            if (w < best) {
              best = w;
              set = 0;
            }
            if (w == best) set |= 1u << r;
          }
          out.row_min[v] = (uint16_t)best;
          out.row_set[v] = (uint16_t)set;
        }
        // Line tables: image row k of coset representative c takes source
        // bits p[k B + t], t < B (image bit j <- source bit p[j]). Each must be
        // a row (same source row, within-row positions stepping by +1 or -1
        // cyclically) or, when there are as many rows as bits per row, a
        // column (same source column, rows stepping by +1 or -1); and each
        // (kind, direction) that occurs must occur for every line of its
        // kind. Then the image rows of all cosets are exactly those lines.
        unsigned const R = out.n_rows;
        uint32_t used[2][2] = {{0, 0}, {0, 0}};  // [row, column][forward, backward]: lines seen
        bool lines_ok = true;
        for (size_t c = 0; c < cosets.size() && lines_ok; ++c) {
          auto const& p = elems[cosets[c]];
          for (unsigned k = 0; k < R && lines_ok; ++k) {
            unsigned sp[64];  // source bit of image bit t of row k
            for (unsigned t = 0; t < B; ++t) sp[t] = p[k * B + t];
            int kind = -1, dir = -1;
            unsigned line = 0;
            bool same_row = true, same_col = true;
            for (unsigned t = 0; t < B; ++t) {
              same_row = same_row && sp[t] / B == sp[0] / B;
              same_col = same_col && sp[t] % B == sp[0] % B;
            }
            if (same_row) {
              unsigned const a = sp[0] % B;
              bool f = true, b = true;
              for (unsigned t = 0; t < B; ++t) {
                f = f && sp[t] % B == (a + t) % B;
                b = b && sp[t] % B == (a + B - t) % B;
              }
              if (f || b) kind = 0, dir = f ? 0 : 1, line = sp[0] / B;
            } else if (same_col && R == B) {
              unsigned const a = sp[0] / B;
              bool f = true, b = true;
              for (unsigned t = 0; t < B; ++t) {
                f = f && sp[t] / B == (a + t) % R;
                b = b && sp[t] / B == (a + R - t) % R;
              }
              if (f || b) kind = 1, dir = f ? 0 : 1, line = sp[0] % B;
            }
            if (kind < 0) lines_ok = false;
            else used[kind][dir] |= 1u << line;
          }
        }
        uint32_t const all_rows = (1u << R) - 1u, all_cols = (1u << B) - 1u;
        for (int d = 0; d < 2 && lines_ok; ++d)
          lines_ok = (used[0][d] == 0 || used[0][d] == all_rows) && (used[1][d] == 0 || used[1][d] == all_cols);
        if (lines_ok) {
          auto rev = [&](unsigned v) {
            unsigned r = 0;
            for (unsigned t = 0; t < B; ++t) r |= ((v >> t) & 1u) << (B - 1 - t);
            return r;
          };
          auto table = [&](uint32_t const (&u)[2], std::vector<uint16_t>& out_tab) {
            out_tab.assign(nv, 0xFFFF);
            for (unsigned v = 0; v < nv; ++v)
              for (int d = 0; d < 2; ++d) {
                if (!u[d]) continue;
                unsigned const w = d ? rev(v) : v;
                out_tab[v] = std::min(out_tab[v], out.row_min[w]);
                if (spin_inversion) out_tab[v] = std::min(out_tab[v], out.row_min[w ^ (nv - 1)]);
              }
          };
          table(used[0], out.line_row);
          out.line_cols = (used[1][0] | used[1][1]) ? 1u : 0u;
          if (out.line_cols) {
            table(used[1], out.line_col);
            out.col_s = (R - 1) * (B - 1);
            out.col_m = 0;
            out.col_k = 0;
            for (unsigned r = 0; r < R; ++r) {
              out.col_m |= (uint64_t)1 << (r * B);
              out.col_k |= (uint64_t)1 << (out.col_s - r * (B - 1));
            }
          }
          out.line_fast = 1;
        }
      }
      if (!ok) out.rows = 0;
    }
  }
  if (self_check)
    if (int st = check_plan(out)) return st;
  if (logging_enabled())
    log_line("symmetry plan: |G| = %u (x%u inversion), |H| = %u (cyclic product: %u, rows: %u of %u bits, "
             "mode %u), cosets = %u, stages = %u, terms = %u, line tables: %u (columns: %u)",
             G, spin_inversion ? 2u : 1u, out.n_h, out.cyc, out.n_rows, out.row_bits, out.rows, out.n_cosets,
             out.n_stages, out.n_terms, out.line_fast, out.line_cols);
  return LS_SUCCESS;
}

PlanView SymPlanHost::view() const {
  PlanView v{};
  v.mask = mask;
  v.n_bits = n_bits;
  v.inv = inv;
  v.L = L;
  v.inv_phase = inv_phase;
  v.n_cosets = n_cosets;
  v.n_h = n_h;
  v.n_stages = n_stages;
  v.n_terms = n_terms;
  v.benes_mask = benes_mask.data();
  v.benes_shift = benes_shift.data();
  v.h_mask = h_mask.data();
  v.h_rot = h_rot.data();
  v.coset_phase = coset_phase.data();
  v.h_phase = h_phase.data();
  v.pos = pos.data();
  v.fixed_nets = n_cosets <= SED_PARAM_COSETS ? 1u : 0u;
  for (unsigned c = 0; c < SED_PARAM_COSETS; ++c)
    for (unsigned st = 0; st < SED_MAX_STAGES; ++st)
      v.nets[c][st] = (v.fixed_nets && c < n_cosets) ? full_nets[c * SED_MAX_STAGES + st] : 0;
  v.rows = rows;
  v.row_bits = row_bits;
  v.n_rows = n_rows;
  v.rot_phase = rot_phase;
  v.shift_phase = shift_phase;
  v.row_mask = row_mask;
  v.line_fast = line_fast;
  v.line_cols = line_cols;
  v.col_s = col_s;
  v.col_m = col_m;
  v.col_k = col_k;
  v.line_row = line_row.data();
  v.line_col = line_col.data();
  v.row_min = row_min.data();
  v.row_set = row_set.data();
  v.rot_mask = rot_mask.data();
  v.rot_rot = rot_rot.data();
  v.rot_exp = rot_exp.data();
  v.sh_mask = sh_mask.data();
  v.sh_rot = sh_rot.data();
  v.sh_exp = sh_exp.data();
  v.cyc = cyc;
  for (int q = 0; q < 2; ++q) {
    v.cyc_ord[q] = cyc_ord[q];
    v.cyc_phase[q] = cyc_phase[q];
    for (int t = 0; t < 2; ++t) {
      v.cyc_rot[q][t] = cyc_rot[q][t];
      v.cyc_mask[q][t] = cyc_mask[q][t];
    }
  }
  return v;
}

}  // namespace sed

using namespace sed;

extern "C" {

int ls_create_symmetry(ls_symmetry** ptr, unsigned length, unsigned const permutation[],
                       unsigned sector) {
  if (!ptr) return fail(LS_INVALID_ARGUMENT, "ls_create_symmetry: ptr is NULL");
  if (length > 64)
    return fail(LS_PERMUTATION_TOO_LONG, "permutation longer than 64 sites: " + std::to_string(length));
  if (!permutation || !is_permutation(length, permutation))
    return fail(LS_INVALID_PERMUTATION, "not a permutation of 0.." + std::to_string(length) + "-1");
  auto* s = new (std::nothrow) ls_symmetry;
  if (!s) return fail(LS_OUT_OF_MEMORY, "ls_create_symmetry");
  s->d.perm.assign(permutation, permutation + length);
  s->d.periodicity = periodicity_of(s->d.perm);
  if (sector >= s->d.periodicity) {
    unsigned const per = s->d.periodicity;
    delete s;
    return fail(LS_INVALID_SECTOR, "sector " + std::to_string(sector) +
                                       " is not below the periodicity " + std::to_string(per));
  }
  s->d.sector = sector;
  *ptr = s;
  return LS_SUCCESS;
}

void ls_destroy_symmetry(ls_symmetry* symmetry) { delete symmetry; }
unsigned ls_get_sector(ls_symmetry const* s) { return s ? s->d.sector : 0; }
unsigned ls_get_periodicity(ls_symmetry const* s) { return s ? s->d.periodicity : 0; }
double ls_get_phase(ls_symmetry const* s) {
  return s ? (double)s->d.sector / (double)s->d.periodicity : 0.0;
}

int ls_create_group(ls_group** ptr, unsigned size, ls_symmetry const* generators[]) {
  if (!ptr) return fail(LS_INVALID_ARGUMENT, "ls_create_group: ptr is NULL");
  if (size > 0 && !generators) return fail(LS_INVALID_ARGUMENT, "ls_create_group: generators is NULL");
  auto* g = new (std::nothrow) ls_group;
  if (!g) return fail(LS_OUT_OF_MEMORY, "ls_create_group");
  GroupData& d = g->d;
  if (size == 0) {
    *ptr = g;  // trivial group; its size follows the basis
    return LS_SUCCESS;
  }
  unsigned const n = (unsigned)generators[0]->d.perm.size();
  unsigned L = 1;
  for (unsigned i = 0; i < size; ++i) {
    if (!generators[i] || generators[i]->d.perm.size() != n) {
      delete g;
      return fail(LS_INVALID_ARGUMENT, "generators act on different numbers of sites");
    }
    L = L / std::gcd(L, generators[i]->d.periodicity) * generators[i]->d.periodicity;
    d.generators.push_back(generators[i]->d);
  }
  d.n = n;
  d.L = L;
  d.perms.resize(n);
  for (unsigned i = 0; i < n; ++i) d.perms[i] = (uint8_t)i;
  d.phase.push_back(0);
  std::unordered_map<std::string, unsigned> index;
  index.emplace(key_of(d.perms.data(), n), 0u);
  std::vector<uint8_t> c(n);
  for (size_t head = 0; head < d.phase.size(); ++head) {
    for (auto const& s : d.generators) {
      uint8_t const* e = d.perms.data() + head * n;
      for (unsigned i = 0; i < n; ++i) c[i] = e[s.perm[i]];  // s after e
      uint32_t const ph = (d.phase[head] + s.sector * (L / s.periodicity)) % L;
      auto it = index.find(key_of(c.data(), n));
      if (it != index.end()) {
        if (d.phase[it->second] != ph) {
          delete g;
          return fail(LS_INCOMPATIBLE_SYMMETRIES,
                      "symmetry sectors are incompatible: a group element has two characters");
        }
        continue;
      }
      if (d.phase.size() == kMaxGroup) {
        delete g;
        return fail(LS_GROUP_TOO_BIG, "symmetry group has more than 65536 elements");
      }
      index.emplace(key_of(c.data(), n), (unsigned)d.phase.size());
      d.perms.insert(d.perms.end(), c.begin(), c.end());
      d.phase.push_back(ph);
    }
  }
  *ptr = g;
  return LS_SUCCESS;
}

void ls_destroy_group(ls_group* group) { delete group; }
unsigned ls_get_group_size(ls_group const* group) { return group ? group->d.size() : 0; }

}  // extern "C"
