/*
 * oracle.c — CPU restatement of the SpinED exact-diagonalisation hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h). Plain C11 + OpenMP so that it
 * builds with gcc on both x86_64 and aarch64; no intrinsics.
 *
 * Every routine follows a call site of the reference; the arithmetic it
 * restates lives in lattice-symmetries (unpinned `master`, configure:26),
 * whose published semantics are: closure of symmetry generators with
 * one-dimensional characters, orbit-minimum representatives, and the
 * symmetry-adapted matrix elements
 *     <r_i~|H|r_j~> = sum_{s : rho(s) = r_j} <r_i|H|s> chi(h_s) n_j / n_i,
 * with h_s(s) = rho(s) the orbit minimum and n = ||P r||.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_MAX_GROUP 65536u
#define OR_TWO_PI 6.283185307179586476925286766559

/* ------------------------------------------------------------------------ */
/* Symmetries (src/SpinED/Internal.hs:99-116; test/Spec.hs:38-43)            */
/* ------------------------------------------------------------------------ */

static int is_permutation(unsigned n, const unsigned* perm) {
  if (n == 0 || n > 64) return 0;
  unsigned char seen[64] = {0};
  for (unsigned i = 0; i < n; ++i) {
    if (perm[i] >= n || seen[perm[i]]) return 0;
    seen[perm[i]] = 1;
  }
  return 1;
}

static unsigned gcd_u(unsigned a, unsigned b) {
  while (b) {
    unsigned t = a % b;
    a = b;
    b = t;
  }
  return a;
}

int or_symmetry_info(unsigned n, const unsigned* perm, unsigned sector, unsigned* periodicity) {
  if (!is_permutation(n, perm)) return OR_INVALID_PERMUTATION;
  /* Periodicity = lcm of cycle lengths. */
  unsigned char seen[64] = {0};
  unsigned per = 1;
  for (unsigned i = 0; i < n; ++i) {
    if (seen[i]) continue;
    unsigned len = 0, j = i;
    while (!seen[j]) {
      seen[j] = 1;
      j = perm[j];
      ++len;
    }
    per = per / gcd_u(per, len) * len;
  }
  if (sector >= per) return OR_INVALID_SECTOR;
  if (periodicity) *periodicity = per;
  return OR_OK;
}

/* ------------------------------------------------------------------------ */
/* Group closure (src/SpinED/Internal.hs:141-150; test/Spec.hs:72-79)        */
/* ------------------------------------------------------------------------ */

/* Element "g after e": (g.(e.x))_i = x_{p_e[p_g[i]]}. */
static void compose(unsigned n, const unsigned* e, const unsigned* g, unsigned* out) {
  for (unsigned i = 0; i < n; ++i) out[i] = e[g[i]];
}

static long find_perm(unsigned n, const unsigned* elems, unsigned count, const unsigned* p) {
  for (unsigned k = 0; k < count; ++k)
    if (memcmp(elems + (size_t)k * n, p, n * sizeof(unsigned)) == 0) return (long)k;
  return -1;
}

int or_group_closure(unsigned n_gens, unsigned n, const unsigned* perms, const unsigned* sectors,
                     unsigned max_size, unsigned* out_perms, unsigned* out_phase, unsigned* out_L,
                     unsigned* out_size) {
  if (n == 0 || n > 64 || max_size == 0) return OR_INVALID_ARGUMENT;
  unsigned L = 1;
  unsigned pers[64];
  if (n_gens > 64) return OR_INVALID_ARGUMENT;
  for (unsigned g = 0; g < n_gens; ++g) {
    int st = or_symmetry_info(n, perms + (size_t)g * n, sectors[g], &pers[g]);
    if (st) return st;
    L = L / gcd_u(L, pers[g]) * pers[g];
  }
  /* Phase numerator of generator g: sector * L / periodicity. */
  unsigned count = 1;
  for (unsigned i = 0; i < n; ++i) out_perms[i] = i;
  out_phase[0] = 0;
  unsigned* tmp = (unsigned*)malloc(n * sizeof(unsigned));
  if (!tmp) return OR_OUT_OF_MEMORY;
  for (unsigned head = 0; head < count; ++head) {
    for (unsigned g = 0; g < n_gens; ++g) {
      compose(n, out_perms + (size_t)head * n, perms + (size_t)g * n, tmp);
      unsigned ph = (out_phase[head] + sectors[g] * (L / pers[g])) % L;
      long k = find_perm(n, out_perms, count, tmp);
      if (k >= 0) {
        if (out_phase[k] != ph) {
          free(tmp);
          return OR_INCOMPATIBLE_SYMMETRIES;
        }
        continue;
      }
      if (count == max_size) {
        free(tmp);
        return OR_GROUP_TOO_BIG;
      }
      memcpy(out_perms + (size_t)count * n, tmp, n * sizeof(unsigned));
      out_phase[count] = ph;
      ++count;
    }
  }
  free(tmp);
  *out_L = L;
  *out_size = count;
  return OR_OK;
}

/* ------------------------------------------------------------------------ */
/* Basis (src/SpinED/Internal.hs:199-236; src/SpinED.hs:178-188,315-337)    */
/* ------------------------------------------------------------------------ */

struct or_basis {
  unsigned n;
  int hw;
  int inv;          /* 0, +1, -1 */
  unsigned G;       /* permutation-group size */
  unsigned L;       /* phase modulus (even when inv == -1) */
  unsigned inv_phase;
  unsigned nbytes;  /* ceil(n / 8) */
  uint64_t mask;
  unsigned* phase;  /* [G] */
  uint64_t* table;  /* [G][nbytes][256] byte images */
  uint64_t binom[65][65];
};

static uint64_t apply_naive(unsigned n, const unsigned* p, uint64_t x) {
  uint64_t y = 0;
  for (unsigned i = 0; i < n; ++i) y |= ((x >> p[i]) & 1u) << i;
  return y;
}

int or_basis_create(or_basis** out, unsigned n, int hamming_weight, int spin_inversion,
                    unsigned group_size, const unsigned* perms, const unsigned* phase, unsigned L) {
  if (n == 0 || n > 64) return OR_INVALID_ARGUMENT;
  if (hamming_weight < -1 || hamming_weight > (int)n) return OR_INVALID_ARGUMENT;
  if (spin_inversion < -1 || spin_inversion > 1) return OR_INVALID_ARGUMENT;
  if (spin_inversion != 0 && hamming_weight != -1 && 2 * hamming_weight != (int)n)
    return OR_INVALID_ARGUMENT;
  if (group_size == 0 || group_size > OR_MAX_GROUP || L == 0) return OR_INVALID_ARGUMENT;
  or_basis* b = (or_basis*)calloc(1, sizeof(or_basis));
  if (!b) return OR_OUT_OF_MEMORY;
  b->n = n;
  b->hw = hamming_weight;
  b->inv = spin_inversion;
  b->G = group_size;
  unsigned scale = (spin_inversion == -1 && (L % 2)) ? 2u : 1u;
  b->L = L * scale;
  b->inv_phase = spin_inversion == -1 ? b->L / 2 : 0;
  b->nbytes = (n + 7) / 8;
  b->mask = n == 64 ? ~(uint64_t)0 : (((uint64_t)1 << n) - 1);
  b->phase = (unsigned*)malloc(group_size * sizeof(unsigned));
  b->table = (uint64_t*)calloc((size_t)group_size * b->nbytes * 256, sizeof(uint64_t));
  if (!b->phase || !b->table) {
    or_basis_destroy(b);
    return OR_OUT_OF_MEMORY;
  }
  for (unsigned g = 0; g < group_size; ++g) {
    const unsigned* p = perms + (size_t)g * n;
    if (!is_permutation(n, p)) {
      or_basis_destroy(b);
      return OR_INVALID_PERMUTATION;
    }
    b->phase[g] = (phase[g] * scale) % b->L;
    /* Byte tables built from the per-bit definition y_i = x_{p[i]}. */
    for (unsigned k = 0; k < b->nbytes; ++k)
      for (unsigned v = 0; v < 256; ++v) {
        uint64_t x = (uint64_t)v << (8 * k);
        x &= b->mask;
        b->table[((size_t)g * b->nbytes + k) * 256 + v] = apply_naive(n, p, x);
      }
  }
  for (unsigned i = 0; i <= 64; ++i) {
    b->binom[i][0] = 1;
    for (unsigned j = 1; j <= 64; ++j)
      b->binom[i][j] = i == 0 ? 0 : b->binom[i - 1][j - 1] + b->binom[i - 1][j];
  }
  *out = b;
  return OR_OK;
}

void or_basis_destroy(or_basis* b) {
  if (!b) return;
  free(b->phase);
  free(b->table);
  free(b);
}

uint64_t or_apply(const or_basis* b, unsigned g, uint64_t x) {
  const uint64_t* t = b->table + (size_t)g * b->nbytes * 256;
  uint64_t y = 0;
  for (unsigned k = 0; k < b->nbytes; ++k) y |= t[k * 256 + ((x >> (8 * k)) & 0xFF)];
  return y;
}

unsigned or_representative_weight(const or_basis* b, uint64_t x) {
  unsigned S = 0;
  for (unsigned g = 0; g < b->G; ++g) {
    uint64_t y = or_apply(b, g, x);
    if (y < x) return 0;
    if (y == x) {
      if (b->phase[g] != 0) return 0;
      ++S;
    }
    if (b->inv) {
      uint64_t yi = ~y & b->mask;
      if (yi < x) return 0;
      if (yi == x) {
        if ((b->phase[g] + b->inv_phase) % b->L != 0) return 0;
        ++S;
      }
    }
  }
  return S;
}

uint64_t or_state_info(const or_basis* b, uint64_t x, unsigned* phase, int* inverted) {
  uint64_t best = x;
  unsigned ph = 0;
  int inv = 0;
  for (unsigned g = 0; g < b->G; ++g) {
    uint64_t y = or_apply(b, g, x);
    if (y < best) {
      best = y;
      ph = b->phase[g];
      inv = 0;
    }
    if (b->inv) {
      uint64_t yi = ~y & b->mask;
      if (yi < best) {
        best = yi;
        ph = (b->phase[g] + b->inv_phase) % b->L;
        inv = 1;
      }
    }
  }
  if (phase) *phase = ph;
  if (inverted) *inverted = inv;
  return best;
}

uint64_t or_space_size(const or_basis* b) {
  if (b->hw >= 0) return b->binom[b->n][b->hw];
  return b->n >= 64 ? ~(uint64_t)0 : ((uint64_t)1 << b->n);
}

/* k-th word (0-based) of n bits with weight w in increasing numeric order. */
static uint64_t unrank(const or_basis* b, uint64_t k) {
  if (b->hw < 0) return k;
  uint64_t x = 0;
  unsigned m = (unsigned)b->hw;
  int c = (int)b->n - 1;
  while (m > 0) {
    while (b->binom[c][m] > k) --c;
    k -= b->binom[c][m];
    x |= (uint64_t)1 << c;
    --m;
    --c;
  }
  return x;
}

/* Next word with the same popcount (increasing order). */
static uint64_t next_same_weight(uint64_t x) {
  uint64_t t = x | (x - 1);
  unsigned tz = (unsigned)__builtin_ctzll(x);
  uint64_t lowbit_nt = ~t & (uint64_t)(-(int64_t)~t);
  uint64_t low = tz + 1 >= 64 ? 0 : ((lowbit_nt - 1) >> (tz + 1));
  return (t + 1) | low;
}

static uint64_t scan_chunk(const or_basis* b, uint64_t r0, uint64_t r1, uint64_t* reps,
                           unsigned* weights) {
  uint64_t x = unrank(b, r0), found = 0;
  for (uint64_t r = r0; r < r1; ++r) {
    unsigned S = or_representative_weight(b, x);
    if (S) {
      if (reps) {
        reps[found] = x;
        if (weights) weights[found] = S;
      }
      ++found;
    }
    if (r + 1 < r1) x = b->hw >= 0 ? next_same_weight(x) : x + 1;
  }
  return found;
}

int or_enumerate(const or_basis* b, uint64_t rank_begin, uint64_t rank_end, uint64_t* reps,
                 unsigned* weights, uint64_t capacity, uint64_t* count) {
  uint64_t space = or_space_size(b);
  if (rank_end > space) rank_end = space;
  if (rank_begin > rank_end) rank_begin = rank_end;
  const uint64_t chunk = 1u << 14;
  uint64_t n_chunks = (rank_end - rank_begin + chunk - 1) / chunk;
  uint64_t* off = (uint64_t*)calloc(n_chunks + 1, sizeof(uint64_t));
  if (!off) return OR_OUT_OF_MEMORY;
#pragma omp parallel for schedule(dynamic, 16)
  for (uint64_t c = 0; c < n_chunks; ++c) {
    uint64_t r0 = rank_begin + c * chunk;
    uint64_t r1 = r0 + chunk < rank_end ? r0 + chunk : rank_end;
    off[c + 1] = scan_chunk(b, r0, r1, NULL, NULL);
  }
  /* Inclusive prefix over chunks keeps the output in word order. */
  for (uint64_t c = 0; c < n_chunks; ++c) off[c + 1] += off[c];
  uint64_t total = off[n_chunks];
  if (reps) {
    if (total > capacity) {
      free(off);
      return OR_BUFFER_TOO_SMALL;
    }
#pragma omp parallel for schedule(dynamic, 16)
    for (uint64_t c = 0; c < n_chunks; ++c) {
      uint64_t r0 = rank_begin + c * chunk;
      uint64_t r1 = r0 + chunk < rank_end ? r0 + chunk : rank_end;
      scan_chunk(b, r0, r1, reps + off[c], weights ? weights + off[c] : NULL);
    }
  }
  free(off);
  *count = total;
  return OR_OK;
}

/* ------------------------------------------------------------------------ */
/* Operator (src/SpinED/Internal.hs:256-367,391-429)                         */
/* ------------------------------------------------------------------------ */

typedef struct {
  unsigned k;
  unsigned n_tuples;
  const uint16_t* sites; /* into op->sites */
  double diag[16][2];
  unsigned n_off[16];
  unsigned off_col[16][16];
  double off_val[16][16][2];
} or_term;

struct or_operator {
  const or_basis* b;
  unsigned n_terms;
  or_term* terms;
  uint16_t* sites;
  double* root; /* [L][2]: exp(-2 pi i k / L) */
};

int or_operator_create(or_operator** out, const or_basis* b, unsigned n_terms, const unsigned* k,
                       const unsigned* n_tuples, const double* matrices, const uint16_t* sites) {
  size_t total_sites = 0;
  for (unsigned t = 0; t < n_terms; ++t) {
    if (k[t] < 1 || k[t] > 4) return OR_INVALID_ARGUMENT;
    total_sites += (size_t)k[t] * n_tuples[t];
  }
  or_operator* op = (or_operator*)calloc(1, sizeof(or_operator));
  if (!op) return OR_OUT_OF_MEMORY;
  op->b = b;
  op->n_terms = n_terms;
  op->terms = (or_term*)calloc(n_terms ? n_terms : 1, sizeof(or_term));
  op->sites = (uint16_t*)malloc((total_sites ? total_sites : 1) * sizeof(uint16_t));
  op->root = (double*)malloc((size_t)b->L * 2 * sizeof(double));
  if (!op->terms || !op->sites || !op->root) {
    or_operator_destroy(op);
    return OR_OUT_OF_MEMORY;
  }
  memcpy(op->sites, sites, total_sites * sizeof(uint16_t));
  size_t so = 0, mo = 0;
  for (unsigned t = 0; t < n_terms; ++t) {
    or_term* T = &op->terms[t];
    T->k = k[t];
    T->n_tuples = n_tuples[t];
    T->sites = op->sites + so;
    unsigned dim = 1u << k[t];
    for (unsigned u = 0; u < n_tuples[t]; ++u)
      for (unsigned m = 0; m < k[t]; ++m) {
        uint16_t s = T->sites[(size_t)u * k[t] + m];
        if (s >= b->n) {
          or_operator_destroy(op);
          return OR_INVALID_ARGUMENT;
        }
        for (unsigned m2 = 0; m2 < m; ++m2)
          if (T->sites[(size_t)u * k[t] + m2] == s) {
            or_operator_destroy(op);
            return OR_INVALID_ARGUMENT;
          }
      }
    for (unsigned a = 0; a < dim; ++a) {
      for (unsigned a2 = 0; a2 < dim; ++a2) {
        const double* v = matrices + 2 * (mo + (size_t)a * dim + a2);
        if (a2 == a) {
          T->diag[a][0] = v[0];
          T->diag[a][1] = v[1];
        } else if (v[0] != 0.0 || v[1] != 0.0) {
          unsigned q = T->n_off[a]++;
          T->off_col[a][q] = a2;
          T->off_val[a][q][0] = v[0];
          T->off_val[a][q][1] = v[1];
        }
      }
    }
    so += (size_t)k[t] * n_tuples[t];
    mo += (size_t)dim * dim;
  }
  /* Characters exp(-2 pi i k / L) with exact values on the axes. */
  for (unsigned q = 0; q < b->L; ++q) {
    double re, im;
    if (4 * q == 0) {
      re = 1.0; im = 0.0;
    } else if (4 * q == b->L) {
      re = 0.0; im = -1.0;
    } else if (2 * q == b->L) {
      re = -1.0; im = 0.0;
    } else if (4 * q == 3 * b->L) {
      re = 0.0; im = 1.0;
    } else {
      double ang = -OR_TWO_PI * (double)q / (double)b->L;
      re = cos(ang);
      im = sin(ang);
    }
    op->root[2 * q] = re;
    op->root[2 * q + 1] = im;
  }
  *out = op;
  return OR_OK;
}

void or_operator_destroy(or_operator* op) {
  if (!op) return;
  free(op->terms);
  free(op->sites);
  free(op->root);
  free(op);
}

static int64_t find_rep(uint64_t D, const uint64_t* reps, uint64_t x) {
  uint64_t lo = 0, hi = D;
  while (lo < hi) {
    uint64_t mid = lo + (hi - lo) / 2;
    if (reps[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return (lo < D && reps[lo] == x) ? (int64_t)lo : -1;
}

static unsigned local_index(uint64_t x, const uint16_t* s, unsigned k) {
  unsigned a = 0;
  for (unsigned m = 0; m < k; ++m) a = (a << 1) | (unsigned)((x >> s[m]) & 1u);
  return a;
}

static uint64_t replace_local(uint64_t x, const uint16_t* s, unsigned k, unsigned a) {
  for (unsigned m = 0; m < k; ++m) {
    uint64_t bit = (uint64_t)((a >> (k - 1 - m)) & 1u);
    x = (x & ~((uint64_t)1 << s[m])) | (bit << s[m]);
  }
  return x;
}

/* Contributions of row i: calls emit(j, coefficient) for every element. */
typedef void (*emit_fn)(void* ctx, uint64_t j, double re, double im);

static void row_elements(const or_operator* op, uint64_t D, const uint64_t* reps,
                         const unsigned* weights, uint64_t i, emit_fn emit, void* ctx) {
  const or_basis* b = op->b;
  uint64_t r = reps[i];
  double Si = (double)weights[i];
  for (unsigned t = 0; t < op->n_terms; ++t) {
    const or_term* T = &op->terms[t];
    for (unsigned u = 0; u < T->n_tuples; ++u) {
      const uint16_t* s = T->sites + (size_t)u * T->k;
      unsigned a = local_index(r, s, T->k);
      if (T->diag[a][0] != 0.0 || T->diag[a][1] != 0.0) emit(ctx, i, T->diag[a][0], T->diag[a][1]);
      for (unsigned q = 0; q < T->n_off[a]; ++q) {
        uint64_t st = replace_local(r, s, T->k, T->off_col[a][q]);
        unsigned ph;
        uint64_t rho = or_state_info(b, st, &ph, NULL);
        int64_t j = find_rep(D, reps, rho);
        if (j < 0) continue; /* the orbit projects to zero in this sector */
        double ratio = sqrt((double)weights[j] / Si);
        const double* c = T->off_val[a][q];
        const double* chi = op->root + 2 * ph;
        double re = (c[0] * chi[0] - c[1] * chi[1]) * ratio;
        double im = (c[0] * chi[1] + c[1] * chi[0]) * ratio;
        emit(ctx, (uint64_t)j, re, im);
      }
    }
  }
}

typedef struct {
  const double* x;
  double acc[2];
} mv_ctx;

static void mv_emit(void* p, uint64_t j, double re, double im) {
  mv_ctx* c = (mv_ctx*)p;
  double xr = c->x[2 * j], xi = c->x[2 * j + 1];
  c->acc[0] += re * xr - im * xi;
  c->acc[1] += re * xi + im * xr;
}

int or_matvec_rows(const or_operator* op, uint64_t D, const uint64_t* reps, const unsigned* weights,
                   const double* x, double* y_rows, uint64_t row_begin, uint64_t row_end) {
  if (row_end > D) row_end = D;
  if (row_begin > row_end) row_begin = row_end;
#pragma omp parallel for schedule(dynamic, 256)
  for (uint64_t i = row_begin; i < row_end; ++i) {
    mv_ctx c = {x, {0.0, 0.0}};
    row_elements(op, D, reps, weights, i, mv_emit, &c);
    y_rows[2 * (i - row_begin)] = c.acc[0];
    y_rows[2 * (i - row_begin) + 1] = c.acc[1];
  }
  return OR_OK;
}

int or_matvec(const or_operator* op, uint64_t D, const uint64_t* reps, const unsigned* weights,
              const double* x, double* y, uint64_t row_begin, uint64_t row_end) {
  if (row_end > D) row_end = D;
#pragma omp parallel for schedule(dynamic, 256)
  for (uint64_t i = row_begin; i < row_end; ++i) {
    mv_ctx c = {x, {0.0, 0.0}};
    row_elements(op, D, reps, weights, i, mv_emit, &c);
    y[2 * i] = c.acc[0];
    y[2 * i + 1] = c.acc[1];
  }
  return OR_OK;
}

typedef struct {
  uint64_t n;
  uint64_t cap;
  uint64_t* col;
  double* val;
} coo_row;

static void coo_emit(void* p, uint64_t j, double re, double im) {
  coo_row* c = (coo_row*)p;
  for (uint64_t q = 0; q < c->n; ++q)
    if (c->col[q] == j) {
      c->val[2 * q] += re;
      c->val[2 * q + 1] += im;
      return;
    }
  if (c->n == c->cap) {
    c->cap = c->cap ? 2 * c->cap : 16;
    c->col = (uint64_t*)realloc(c->col, c->cap * sizeof(uint64_t));
    c->val = (double*)realloc(c->val, 2 * c->cap * sizeof(double));
  }
  c->col[c->n] = j;
  c->val[2 * c->n] = re;
  c->val[2 * c->n + 1] = im;
  ++c->n;
}

int or_matrix_coo(const or_operator* op, uint64_t D, const uint64_t* reps, const unsigned* weights,
                  uint64_t* rows, uint64_t* cols, double* vals, uint64_t capacity, uint64_t* nnz) {
  uint64_t total = 0;
  coo_row c = {0, 0, NULL, NULL};
  for (uint64_t i = 0; i < D; ++i) {
    c.n = 0;
    row_elements(op, D, reps, weights, i, coo_emit, &c);
    for (uint64_t q = 0; q < c.n; ++q) {
      if (rows) {
        if (total >= capacity) {
          free(c.col);
          free(c.val);
          return OR_BUFFER_TOO_SMALL;
        }
        rows[total] = i;
        cols[total] = c.col[q];
        vals[2 * total] = c.val[2 * q];
        vals[2 * total + 1] = c.val[2 * q + 1];
      }
      ++total;
    }
  }
  free(c.col);
  free(c.val);
  *nnz = total;
  return OR_OK;
}

uint64_t or_row_work(const or_operator* op, const uint64_t* rows, uint64_t n_rows, uint64_t* n_elements) {
  uint64_t sum = 0, count = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(^ : sum) reduction(+ : count)
  for (uint64_t i = 0; i < n_rows; ++i) {
    uint64_t r = rows[i];
    for (unsigned t = 0; t < op->n_terms; ++t) {
      const or_term* T = &op->terms[t];
      for (unsigned u = 0; u < T->n_tuples; ++u) {
        const uint16_t* st = T->sites + (size_t)u * T->k;
        unsigned a = local_index(r, st, T->k);
        for (unsigned q = 0; q < T->n_off[a]; ++q) {
          unsigned ph;
          sum ^= or_state_info(op->b, replace_local(r, st, T->k, T->off_col[a][q]), &ph, NULL) + ph;
          ++count;
        }
      }
    }
  }
  if (n_elements) *n_elements = count;
  return sum;
}

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) and the start vector.   */
/* ------------------------------------------------------------------------ */

void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int round = 0; round < 10; ++round) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static double u01_53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

void or_start_vector(uint64_t seed, uint64_t D, double* out) {
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
#pragma omp parallel for schedule(static)
  for (uint64_t blk = 0; blk < (D + 1) / 2; ++blk) {
    uint32_t ctr[4] = {(uint32_t)blk, (uint32_t)(blk >> 32), 0u, 0u}, r[4];
    or_philox4x32_10(ctr, key, r);
    out[2 * blk] = 2.0 * u01_53(r[0], r[1]) - 1.0;
    if (2 * blk + 1 < D) out[2 * blk + 1] = 2.0 * u01_53(r[2], r[3]) - 1.0;
  }
}

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
