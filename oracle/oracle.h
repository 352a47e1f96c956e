/*
 * oracle.h — CPU restatement of the SpinED exact-diagonalisation hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker: the parity tests,
 * `__graft_entry__.smoke()` and the CPU-baseline leg of `bench.py` load it to
 * produce expected values. No product code path links, loads or calls it.
 *
 * The reference (twesterhout/spin-ed) keeps its numerics in lattice-symmetries
 * (C++/OpenMP, cloned unpinned at `master`, configure:21-33) and PRIMME
 * (primme-hs, unpinned git HEAD, cabal.project:13-15). Neither is vendored, so
 * this file restates the published mathematics at the reference's call sites:
 *   ls_create_symmetry  src/SpinED/Internal.hs:69-70,99-116
 *   ls_create_group     src/SpinED/Internal.hs:120-150
 *   ls_create_spin_basis/ls_build  src/SpinED/Internal.hs:172-182,199-236
 *   ls_create_interaction{1..4}    src/SpinED/Internal.hs:258-270,350-362
 *   ls_operator_matmat  src/SpinED/Internal.hs:377-378,411-429
 *
 * Conventions (fixed here; the reference tests pin none of them):
 *   - A permutation p acts on a bit string x as y_i = x_{p[i]}.
 *   - A generator with periodicity n and sector k has character
 *     exp(-2*pi*i*k/n); characters are stored as integer phases mod L,
 *     L = lcm of the generators' periodicities.
 *   - Spin inversion with sign s maps x -> ~x (within n bits), character s.
 *   - The representative of an orbit is its numerically smallest member; a
 *     representative is kept iff the group character is trivial on its
 *     stabiliser. Its stabiliser order S (>0) fixes the norm
 *     sqrt(S / |G|), |G| counting inversion.
 *   - For a k-site term on sites (i_0..i_{k-1}) the local index is
 *     sum_m bit(i_m) << (k-1-m) (first site most significant).
 */
#ifndef SED_ORACLE_H
#define SED_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  OR_OK = 0,
  OR_INVALID_PERMUTATION = 10,
  OR_INVALID_SECTOR = 11,
  OR_INCOMPATIBLE_SYMMETRIES = 12,
  OR_GROUP_TOO_BIG = 13,
  OR_INVALID_ARGUMENT = 14,
  OR_OUT_OF_MEMORY = 15,
  OR_BUFFER_TOO_SMALL = 16,
};

/* Periodicity of a permutation and sector check (test/Spec.hs:39-43). */
int or_symmetry_info(unsigned n, const unsigned* perm, unsigned sector, unsigned* periodicity);

/* Group closure of n_gens generators of n sites each. Writes up to max_size
 * elements (perm rows of length n, phase numerators mod *L). */
int or_group_closure(unsigned n_gens, unsigned n, const unsigned* perms, const unsigned* sectors,
                     unsigned max_size, unsigned* out_perms, unsigned* out_phase, unsigned* out_L,
                     unsigned* out_size);

/* A basis: number of spins, Hamming weight (-1 none), inversion sign (0 none)
 * and the closed permutation group. */
typedef struct or_basis or_basis;
int or_basis_create(or_basis** out, unsigned n, int hamming_weight, int spin_inversion,
                    unsigned group_size, const unsigned* perms, const unsigned* phase, unsigned L);
void or_basis_destroy(or_basis* b);

/* Apply group element g (0 <= g < group_size) to x. */
uint64_t or_apply(const or_basis* b, unsigned g, uint64_t x);

/* Stabiliser order with trivial character (0 if x is not an orbit minimum or
 * the character is non-trivial on its stabiliser). */
unsigned or_representative_weight(const or_basis* b, uint64_t x);

/* Orbit minimum of x, the group element mapping x to it (phase numerator and
 * whether inversion was applied). */
uint64_t or_state_info(const or_basis* b, uint64_t x, unsigned* phase, int* inverted);

/* Enumerate representatives in ascending order. Call once with reps == NULL
 * to get the count, then with buffers of that size. rank_begin/rank_end
 * restrict the scan to a slice of the fixed-weight (or full) word ranks; pass
 * 0 and UINT64_MAX for the whole space. */
int or_enumerate(const or_basis* b, uint64_t rank_begin, uint64_t rank_end, uint64_t* reps,
                 unsigned* weights, uint64_t capacity, uint64_t* count);

/* Number of words scanned by or_enumerate for the whole space. */
uint64_t or_space_size(const or_basis* b);

/* Operator terms: n_terms interactions; term t has k[t] sites per tuple,
 * n_tuples[t] tuples, a 2^k x 2^k complex matrix (row-major, interleaved
 * re/im) and uint16 site indices, concatenated in term order. */
typedef struct or_operator or_operator;
int or_operator_create(or_operator** out, const or_basis* b, unsigned n_terms, const unsigned* k,
                       const unsigned* n_tuples, const double* matrices, const uint16_t* sites);
void or_operator_destroy(or_operator* op);

/* y = H x in the symmetry-adapted basis (pull form, complex128 arithmetic).
 * reps/weights: the sorted representatives and their stabiliser orders.
 * x, y: interleaved complex, length D each. Rows [row_begin, row_end). */
int or_matvec(const or_operator* op, uint64_t D, const uint64_t* reps, const unsigned* weights,
              const double* x, double* y, uint64_t row_begin, uint64_t row_end);

/* Rows [row_begin, row_end) of y = H x into y_rows (interleaved complex,
 * row_end - row_begin entries); reps/weights/x as for or_matvec. */
int or_matvec_rows(const or_operator* op, uint64_t D, const uint64_t* reps, const unsigned* weights,
                   const double* x, double* y_rows, uint64_t row_begin, uint64_t row_end);

/* Explicit matrix in COO form (duplicates summed per row). Call with
 * rows == NULL to get nnz. */
int or_matrix_coo(const or_operator* op, uint64_t D, const uint64_t* reps, const unsigned* weights,
                  uint64_t* rows, uint64_t* cols, double* vals, uint64_t capacity, uint64_t* nnz);

/* Work of the on-the-fly matvec for the given rows without the index
 * lookup (which needs the full representative list): generates every
 * element and canonicalises it. Returns a checksum of the representatives
 * found; used to time bounded samples of large bases on the CPU. */
uint64_t or_row_work(const or_operator* op, const uint64_t* rows, uint64_t n_rows, uint64_t* n_elements);

/* Philox4x32-10 (Salmon et al., SC'11). */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* Start vector: element i is uniform in [-1, 1) from Philox block i/2. */
void or_start_vector(uint64_t seed, uint64_t D, double* out);

/* Number of threads OpenMP will use. */
int or_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
