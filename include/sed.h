/*
 * sed.h — C ABI of libsed, the GB300 (sm_103a) exact-diagonalisation engine.
 *
 * The `ls_*` entry points have the names, argument meanings and status
 * convention of the lattice-symmetries C ABI that SpinED binds with
 * `foreign import ccall` in src/SpinED/Internal.hs; each declaration cites the
 * import it replaces. The `sed_*` entry points are additions: the device
 * eigensolver that replaces Numeric.PRIMME.eigh (src/SpinED.hs:404) and
 * device-resident variants of the matvec.
 *
 * Conventions
 *  - Every function returning int returns 0 on success and a non-zero status
 *    otherwise; ls_error_to_string() turns a status into a message that the
 *    caller frees with ls_destroy_string() (Internal.hs:47-65).
 *  - Handles are opaque and are written through an out-pointer
 *    (Internal.hs:96-97). Destroy functions accept NULL, may run on any host
 *    thread (they are GHC finalisers, Internal.hs:72-73) and never require a
 *    current CUDA context or stream.
 *  - x/y block arguments may be host memory (pageable or pinned) or device
 *    memory of the current device; the library detects which. Blocks are
 *    column-major with the given column strides (Internal.hs:411-429).
 *  - Calls that take caller buffers and return when done (ls_operator_matmat,
 *    ls_operator_expectation, ls_build_unsafe, sed_eigh, sed_eigh_batched,
 *    sed_mlp_*) first wait for all work queued on the device when any of
 *    those buffers is device memory, so a buffer the caller has just written
 *    on a stream of its own is complete before libsed reads it. Calls that
 *    take a stream argument order their work on that stream instead.
 *  - dtype codes: 0 = float32, 1 = float64, 2 = complex64, 3 = complex128
 *    (Internal.hs:404-409).
 *  - A permutation p acts on a spin configuration x as y_i = x_{p[i]}; a
 *    generator with periodicity n and sector k has eigenvalue exp(-2 pi i k/n);
 *    representatives are orbit minima.
 */
#ifndef SED_H
#define SED_H

#include <stdbool.h>
#include <stdint.h>

#if defined(__GNUC__)
#define SED_API __attribute__((visibility("default")))
#else
#define SED_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ls_symmetry ls_symmetry;
typedef struct ls_group ls_group;
typedef struct ls_spin_basis ls_spin_basis;
typedef struct ls_states ls_states;
typedef struct ls_interaction ls_interaction;
typedef struct ls_operator ls_operator;

/* Status codes (values are part of the ABI). */
enum {
  LS_SUCCESS = 0,
  LS_OUT_OF_MEMORY = 1,
  LS_INVALID_ARGUMENT = 2,
  LS_INVALID_HAMMING_WEIGHT = 3,
  LS_INVALID_SPIN_INVERSION = 4,
  LS_INVALID_NUMBER_SPINS = 5,
  LS_INVALID_PERMUTATION = 6,
  LS_INVALID_SECTOR = 7,
  LS_INVALID_STATE = 8,
  LS_INVALID_DATATYPE = 9,
  LS_PERMUTATION_TOO_LONG = 10,
  LS_INCOMPATIBLE_SYMMETRIES = 11,
  LS_NOT_A_REPRESENTATIVE = 12,
  LS_WRONG_BASIS_TYPE = 13,
  LS_CACHE_NOT_BUILT = 14,
  LS_COULD_NOT_OPEN_FILE = 15,
  LS_FILE_IO_FAILED = 16,
  LS_CACHE_IS_CORRUPT = 17,
  LS_OPERATOR_IS_COMPLEX = 18,
  LS_DIMENSION_MISMATCH = 19,
  LS_GROUP_TOO_BIG = 20,
  LS_CUDA_ERROR = 21,
  LS_NOT_CONVERGED = 22,
  LS_DEVICE_TIMEOUT = 23,
  LS_SYSTEM_ERROR = 24,
};

/* --- errors and logging -------------------------------------------------- */

/* Internal.hs:39. Returns a heap string; free it with ls_destroy_string. */
SED_API char const* ls_error_to_string(int status);
/* Internal.hs:41 */
SED_API void ls_destroy_string(char const* message);
/* Internal.hs:43 */
SED_API void ls_enable_logging(void);
/* Internal.hs:45 */
SED_API void ls_disable_logging(void);

/* --- symmetries (Internal.hs:67-116) ------------------------------------ */

/* Internal.hs:69-70. Validates that `permutation` is a permutation of
 * 0..length-1 (length <= 64) and that sector < periodicity. */
SED_API int ls_create_symmetry(ls_symmetry** ptr, unsigned length, unsigned const permutation[],
                       unsigned sector);
/* Internal.hs:72-73 */
SED_API void ls_destroy_symmetry(ls_symmetry* symmetry);
/* Internal.hs:75 */
SED_API unsigned ls_get_sector(ls_symmetry const* symmetry);
/* Internal.hs:77. Returns sector / periodicity. */
SED_API double ls_get_phase(ls_symmetry const* symmetry);
/* Internal.hs:79 */
SED_API unsigned ls_get_periodicity(ls_symmetry const* symmetry);

/* --- groups (Internal.hs:118-155) ---------------------------------------- */

/* Internal.hs:120-121. Closure of the generators; fails with
 * LS_INCOMPATIBLE_SYMMETRIES when two products give the same permutation
 * with different characters. Zero generators give the trivial group. */
SED_API int ls_create_group(ls_group** ptr, unsigned size, ls_symmetry const* generators[]);
/* Internal.hs:123-124 */
SED_API void ls_destroy_group(ls_group* group);
/* Internal.hs:126-127. Number of permutations (spin inversion not counted). */
SED_API unsigned ls_get_group_size(ls_group const* group);

/* --- spin basis (Internal.hs:157-254) ------------------------------------ */

/* Internal.hs:172-173. hamming_weight = -1 for no restriction; spin_inversion
 * in {-1, 0, +1}, 0 meaning none. */
SED_API int ls_create_spin_basis(ls_spin_basis** ptr, ls_group const* group, unsigned number_spins,
                         int hamming_weight, int spin_inversion);
/* Internal.hs:175-176 */
SED_API void ls_destroy_spin_basis(ls_spin_basis* basis);
/* Internal.hs:178-179. Enumerates the representatives on the GPU. */
SED_API int ls_build(ls_spin_basis* basis);
/* Internal.hs:181-182. Installs a caller-supplied sorted representative list
 * (host or device memory); norms are recomputed on the GPU. */
SED_API int ls_build_unsafe(ls_spin_basis* basis, uint64_t size, uint64_t const representatives[]);
/* Internal.hs:184-185 */
SED_API int ls_get_number_states(ls_spin_basis const* basis, uint64_t* out);
/* Internal.hs:187-188. Copies the representatives into host memory owned by
 * the returned states object. */
SED_API int ls_get_states(ls_states** ptr, ls_spin_basis const* basis);
/* Internal.hs:190-191. Host pointer, valid until ls_destroy_states. */
SED_API uint64_t const* ls_states_get_data(ls_states const* states);
/* Internal.hs:193-194 */
SED_API uint64_t ls_states_get_size(ls_states const* states);
/* Internal.hs:196-197 */
SED_API void ls_destroy_states(ls_states* states);

/* --- interactions (Internal.hs:256-367) ---------------------------------- */

/* Internal.hs:260-270. matrix: 2^k x 2^k complex128, row-major, interleaved
 * (re, im); sites: number_nodes tuples of k uint16 site indices. For a tuple
 * (i_0, ..., i_{k-1}) the local index is sum_m bit(i_m) << (k-1-m). */
SED_API int ls_create_interaction1(ls_interaction** ptr, void const* matrix, unsigned number_nodes,
                           uint16_t const* nodes);
SED_API int ls_create_interaction2(ls_interaction** ptr, void const* matrix, unsigned number_nodes,
                           uint16_t const* nodes);
SED_API int ls_create_interaction3(ls_interaction** ptr, void const* matrix, unsigned number_nodes,
                           uint16_t const* nodes);
SED_API int ls_create_interaction4(ls_interaction** ptr, void const* matrix, unsigned number_nodes,
                           uint16_t const* nodes);
/* Internal.hs:272-273 */
SED_API bool ls_interaction_is_real(ls_interaction const* interaction);
/* Internal.hs:275-276 */
SED_API void ls_destroy_interaction(ls_interaction* interaction);

/* --- operators (Internal.hs:369-458) ------------------------------------- */

/* Internal.hs:371-372. Binds the terms to a basis (built now or later, as
 * SpinED builds representatives after creating operators, Main.hs:19-22);
 * sites must be below number_spins and distinct within a tuple. */
SED_API int ls_create_operator(ls_operator** ptr, ls_spin_basis const* basis, unsigned number_terms,
                       ls_interaction const* const terms[]);
/* Internal.hs:374-375 */
SED_API void ls_destroy_operator(ls_operator* op);
/* Internal.hs:377-378. Y = H X for `block_size` columns of length `size`. */
SED_API int ls_operator_matmat(ls_operator const* op, int dtype, uint64_t size, uint64_t block_size,
                       void const* x, uint64_t x_stride, void* y, uint64_t y_stride);
/* Internal.hs:380-381. out[c] = <x_c|H|x_c> as complex128 (interleaved). */
SED_API int ls_operator_expectation(ls_operator const* op, int dtype, uint64_t size, uint64_t block_size,
                            void const* x, uint64_t x_stride, void* out);
/* Internal.hs:383-384. True iff every term is real and every character of the
 * sector is real. */
SED_API bool ls_operator_is_real(ls_operator const* op);

/* --- additions: device eigensolver and device-resident forms ------------- */

/* Matvec forms. SED_FORM_STREAM records (column, value code) once and then
 * streams it (an HBM-bound SpMV); SED_FORM_ON_THE_FLY regenerates every
 * element each call. SED_FORM_AUTO streams when the recorded form fits. */
enum { SED_FORM_AUTO = 0, SED_FORM_STREAM = 1, SED_FORM_ON_THE_FLY = 2 };
/* Krylov storage/arithmetic: plain FP64, or FP32-stored vectors for the bulk
 * of the iterations followed by an FP64 refinement. */
enum { SED_PRECISION_FP64 = 0, SED_PRECISION_MIXED = 1 };
/* Start vector: Philox4x32-10 uniform [-1, 1) from `seed`, or the caller's
 * vector(s) in `start`. */
enum { SED_START_RANDOM = 0, SED_START_GIVEN = 1 };

typedef void (*sed_progress_fn)(void* user, uint64_t iteration, double const* ritz_values,
                                double const* residual_estimates, unsigned count);

typedef struct sed_eigh_options {
  uint32_t struct_size;      /* sizeof(sed_eigh_options) */
  uint32_t nev;              /* number of lowest eigenpairs (number_vectors) */
  double tol;                /* ||H psi - E psi|| bound; <= 0 means 1e-8 */
  uint32_t max_iter;         /* Lanczos steps in total; 0 means 100000 */
  uint32_t max_basis;        /* stored Krylov vectors per cycle; 0 = auto */
  uint32_t block_size;       /* 1 = single-vector Lanczos */
  uint32_t precision;        /* SED_PRECISION_* */
  uint32_t start;            /* SED_START_* */
  uint32_t form;             /* SED_FORM_* */
  uint64_t seed;             /* Philox key for SED_START_RANDOM */
  void const* start_vectors; /* column-major, size x block_size, host or device */
  uint64_t start_stride;
  sed_progress_fn progress;  /* may be NULL; called between iterations */
  void* progress_user;
} sed_eigh_options;

typedef struct sed_eigh_info {
  uint64_t iterations;       /* Lanczos steps (all phases) */
  uint64_t matvecs;
  uint64_t restarts;
  uint64_t fp32_iterations;  /* steps taken with FP32-stored vectors */
  double seconds_total;
  double seconds_setup;      /* recording the stream form */
  double seconds_solve;
} sed_eigh_info;

/* Fills `opts` with defaults (nev 1, tol 1e-8, FP64, random seed 1234). */
SED_API void sed_eigh_options_init(sed_eigh_options* opts);

/* Replaces Numeric.PRIMME.eigh at src/SpinED.hs:404: lowest `opts->nev`
 * eigenpairs of `op`. eigenvalues[nev] and residuals[nev] are host arrays;
 * eigenvectors is size x nev, column-major with stride ldv, host or device,
 * of `dtype`; residuals are ||H psi - E psi|| of the returned unit vectors
 * recomputed in FP64 at the end. `info` may be NULL. */
SED_API int sed_eigh(ls_operator const* op, int dtype, sed_eigh_options const* opts, double* eigenvalues,
             void* eigenvectors, uint64_t ldv, double* residuals, sed_eigh_info* info);

/* Selects the matvec form of the operator for later calls (ls_operator_matmat,
 * sed_eigh with SED_FORM_AUTO); SED_FORM_STREAM and SED_FORM_AUTO record the
 * stream form now (AUTO silently keeps on-the-fly if it does not fit). */
SED_API int sed_operator_prepare(ls_operator* op, int form);
/* How the stream form is recorded. AUTO uses the orbit table when the
 * characters are real and the table fits in 40 % of the free device memory:
 * a map from every word of the basis's weight class (C(n, w) words, or 2^n
 * without a Hamming weight; 4 bytes each) to its representative's index and
 * character sign, filled by enumerating the orbits of the representatives,
 * after which each generated element costs one rank and one table load.
 * CANONICALISE always searches the group for each element. Both record
 * bit-identical stream forms. The setting is process-wide. */
enum { SED_RECORD_AUTO = 0, SED_RECORD_CANONICALISE = 1 };
SED_API void sed_set_record_mode(int mode);
/* 1 if the operator's stream form was recorded through the orbit table. */
SED_API int sed_operator_recorded_with_table(ls_operator const* op);

/* Bytes the stream form occupies on the device (0 if not recorded). */
SED_API uint64_t sed_operator_stream_bytes(ls_operator const* op);
/* Stored elements of the stream form (off-diagonal, per matvec). */
SED_API uint64_t sed_operator_stream_elements(ls_operator const* op);

/* Y = H X on device pointers, enqueued on `stream` (a cudaStream_t, or NULL
 * for the operator's own stream); returns without synchronising. */
SED_API int sed_operator_matmat_device(ls_operator const* op, int dtype, uint64_t size,
                               uint64_t block_size, void const* x, uint64_t x_stride, void* y,
                               uint64_t y_stride, void* stream);

/* Measurement: y = H x for a real operator, x and y FP64 device vectors of
 * the basis size, `repetitions` times back to back on the operator's stream
 * after two untimed ones; *ms_matvec is the CUDA-event time per complete
 * matvec and *ms_kernel the time per launch of the SpMV kernel alone. The
 * two differ when the matvec runs in exact fixed point (real operators with
 * real characters and at most 4 distinct off-diagonal values): its pre-pass
 * turns x into the scaled integer copy the SpMV gathers, and the Lanczos
 * solver produces that copy inside its vector update instead. */
SED_API int sed_operator_time_matvec(ls_operator const* op, void const* x, void* y, unsigned repetitions,
                                     double* ms_matvec, double* ms_kernel);

/* No counterpart in the reference: ls_operator_expectation for callers that
 * cannot let the library allocate device memory (a process whose device
 * memory belongs to its own pool allocator, or a latency-critical loop that
 * cannot afford cudaMalloc's implicit synchronisation). Computes Y = H X
 * into the caller's device buffer y (column stride y_stride) and
 * out[c] = <x_c|y_c> as complex128 (out: host or device memory). x and y
 * must be device memory; at most 64 columns per call. It performs no device
 * allocation: the operator must already be prepared (sed_operator_prepare,
 * or an earlier ls_operator_matmat); the streamed form is used if recorded,
 * else the on-the-fly form, and neither is recorded here. The work is
 * enqueued on `stream` (a cudaStream_t): pass the stream on which x was
 * written, so that the matvec reads x only after those writes. NULL selects
 * the operator's own non-blocking stream, which is ordered with nothing the
 * caller enqueued: x must then be complete (and y no longer in use) before
 * the call, e.g. after a cudaDeviceSynchronize. The call waits for `stream`
 * to finish before it returns, so `out` holds the results on return. Partial
 * sums live in a 66 KiB scratch array in the library's static device memory
 * (held on every GPU that loads the library until exit) and shared by all
 * calls: calls that overlap on the GPU race on it. Because the call
 * synchronises with `stream` before it returns, it cannot be captured in a
 * CUDA graph. */
SED_API int sed_operator_expectation_noalloc(ls_operator const* op, int dtype, uint64_t size,
                                             uint64_t block_size, void const* x, uint64_t x_stride,
                                             void* y, uint64_t y_stride, void* out, void* stream);

/* V[:, 0..kk) <- V[:, 0..m) Y in place: the basis rotation of a thick
 * restart (Ritz vectors replacing the first kk Krylov vectors). No
 * counterpart in the reference (PRIMME's restart is internal to it,
 * src/SpinED.hs:404). V is FP64, D x m column-major with stride ld >= D; Y
 * is m x kk row-major FP64; both device memory, 1 <= kk <= m <= 32. Paths:
 * SED_ROTATE_TENSOR runs it on the tensor cores (kk <= 16) by an error-free
 * split of both operands into 8-bit slices held exactly in BF16, FP32
 * accumulation in tensor memory that is exact for these slices, and integer
 * recombination (the result differs from an FP64 product by the truncation
 * of each operand to 56 bits below its row or column maximum and the final
 * rounding); SED_ROTATE_FP64 uses FP64 FMAs on the CUDA cores;
 * SED_ROTATE_AUTO takes the tensor cores when the shape allows and m >= 16
 * (where they measured faster than the FP64 pipe). The work is
 * enqueued on `stream` (a cudaStream_t; NULL = the legacy default stream)
 * and the call waits for it. sed_set_rotate_path selects the path of the
 * rotation inside sed_eigh's thick-restart solver (process-wide). */
enum { SED_ROTATE_AUTO = 0, SED_ROTATE_FP64 = 1, SED_ROTATE_TENSOR = 2 };
SED_API int sed_rotate_vectors(double* V, uint64_t ld, uint32_t m, double const* Y, uint32_t kk, uint64_t D,
                               int path, void* stream);
SED_API void sed_set_rotate_path(int path);

/* Many Hamiltonians in one persistent launch. No counterpart in the
 * reference, which solves one operator per run. The lowest opts->nev (<= 4)
 * eigenpairs of every operator by block Lanczos with block size 4
 * (opts->block_size 0 or 4; opts->max_basis / 4 stored blocks per cycle, at
 * most 16, default 12; opts->tol; opts->seed; opts->max_iter bounds the
 * matvec columns per problem). Vectors, matvec, QR and Rayleigh-Ritz are
 * FP64; the Gram-Schmidt products run in double-float arithmetic (about 48
 * significant bits). All operators must be real, built and on the current
 * device; their stream forms are recorded if needed. One cooperative kernel
 * solves all of them: its CTAs form groups that solve their problems one
 * after another; large problems get a group of several CTAs each and small
 * ones share one-CTA groups, by a cost model of a block step
 * (sed_debug_batched_layout); the launch shape (threads and CTAs per SM) is
 * picked by timing short trial runs on the first call for a given set of
 * sizes (cached afterwards). eigenvalues and residuals are
 * count x nev host arrays (row i for operator i; residuals may be NULL);
 * eigenvectors[i] (host or device, may be NULL, or the array itself NULL) is
 * D_i x nev column-major with stride ldv[i] (ldv NULL: D_i). */
typedef struct sed_batch_info {
  uint64_t block_steps_max;  /* block Lanczos steps of the slowest problem */
  uint64_t restarts_max;
  double seconds_total;
  double seconds_setup;      /* stream-form recording */
  double seconds_solve;      /* the persistent launch and the result copies */
  double kernel_ms;          /* CUDA-event time of the persistent launch */
  uint32_t grid;             /* CTAs available to the launch */
  uint32_t ctas_per_sm;
  uint32_t threads_per_cta;
  uint32_t reserved;
} sed_batch_info;
SED_API int sed_eigh_batched(unsigned count, ls_operator* const ops[], sed_eigh_options const* opts,
                             double* eigenvalues, double* residuals, void* const eigenvectors[],
                             uint64_t const ldv[], sed_batch_info* info);
/* Fixes the launch shape of sed_eigh_batched instead of tuning it: 128 or
 * 256 threads per CTA and 1 to 3 CTAs per SM (a shape that is not
 * co-resident on the device makes sed_eigh_batched fail with
 * LS_INVALID_ARGUMENT). threads_per_cta = 0 returns to tuning, which times
 * every such shape on a short trial run. Process-wide. */
SED_API void sed_set_batched_launch(unsigned threads_per_cta, unsigned ctas_per_sm);

/* Norms ||P r|| = sqrt(S / |G|) of the representatives (host array). */
SED_API int sed_basis_get_norms(ls_spin_basis const* basis, double* out);
/* Device pointer to the representatives (valid while the basis lives). */
SED_API uint64_t const* sed_basis_device_states(ls_spin_basis const* basis);
/* Index of a representative, or LS_NOT_A_REPRESENTATIVE. */
SED_API int sed_basis_index(ls_spin_basis const* basis, uint64_t representative, uint64_t* index);
/* Orbit minimum and character phase (numerator of exp(-2 pi i phase / L)). */
SED_API int sed_basis_state_info(ls_spin_basis const* basis, uint64_t bits, uint64_t* representative,
                         unsigned* phase, unsigned* phase_modulus);

/* ------------------------------------------------ learned start vector ---
 * No counterpart in the reference, which always starts PRIMME from its own
 * random vector (src/SpinED.hs:385-394). A small MLP over spin
 * configurations, x_j = +1/-1 for spin j up/down:
 *   h1 = tanh(W1 x + b1), h2 = tanh(W2 h1 + b2), (a, s) = W3 h2 + b3,
 * a ~ log|psi(x)| and s the logit of "sign psi(x) = (-1)^popcount(x &
 * sign_mask)". Weights: FP32 master copy (Adam), BF16 in the passes, FP32
 * accumulation. Parameters are one FP32 blob in the order W1 [hidden x n],
 * b1, W2 [hidden x hidden], b2, W3 [2 x hidden], b3 (row-major). The network
 * lives on the current device. Host or device pointers are accepted
 * everywhere below. */
typedef struct sed_mlp sed_mlp;
SED_API int sed_mlp_create(sed_mlp** out, unsigned n_inputs, unsigned hidden, uint64_t sign_mask, uint64_t seed);
SED_API void sed_mlp_destroy(sed_mlp* mlp);
SED_API uint64_t sed_mlp_num_params(sed_mlp const* mlp);
SED_API int sed_mlp_get_params(sed_mlp const* mlp, float* out);
SED_API int sed_mlp_set_params(sed_mlp* mlp, float const* in);
/* out[2 i], out[2 i + 1] = (a, s) for states[i]. */
SED_API int sed_mlp_forward(sed_mlp* mlp, uint64_t const* states, uint64_t n, float* out);
/* Loss L = mean_i [(a_i - t_abs_i)^2 + BCE(s_i, y_i)], y_i = [t_sign_i (1 if
 * psi_i > 0, else 0) agrees with the prior], and dL/dparams (same layout as
 * the parameters; grads may be NULL). At most 2^20 samples (a patch network:
 * at most 8 388 480 / n_sites). */
SED_API int sed_mlp_loss_grad(sed_mlp* mlp, uint64_t const* states, float const* t_abs, float const* t_sign,
                              uint64_t n, double* loss, float* grads);
/* Adam (0.9, 0.999, 1e-8) on mini-batches of `batch` samples, reshuffled
 * every epoch (floor(n / batch) batches; the rest of a shuffle is unused);
 * final_loss (may be NULL) is the loss of the last batch. On the tensor-core
 * path (sed_mlp_set_path) the shuffle is a keyed permutation made on the
 * device, at most 2^31 - 1 samples; on the SIMT path a host shuffle. Both
 * paths add every gradient sum in a fixed order: the same data, starting
 * parameters and seed give the same network bit for bit. */
SED_API int sed_mlp_train(sed_mlp* mlp, uint64_t const* states, float const* t_abs, float const* t_sign, uint64_t n,
                          unsigned epochs, unsigned batch, float lr, uint64_t seed, double* final_loss);
/* Training data from a real vector psi over the built basis: n representatives
 * drawn with probability psi_r^2 / ||psi||^2 (Philox from `seed`), labelled
 * t_abs = log|psi_r n_r| (the amplitude of the configuration itself, n_r =
 * ||P r||) and t_sign = [sigma psi_r > 0]. An eigenvector's global sign is
 * arbitrary, so sigma = +1 or -1 is chosen to make
 * sum_r prior(r) sigma psi_r |psi_r| >= 0 with prior(r) =
 * (-1)^popcount(r & sign_mask): data sets sampled from several ground states
 * then agree on the sign (pass the network's sign_mask). */
SED_API int sed_mlp_sample(ls_spin_basis const* basis, double const* psi, uint64_t n, uint64_t seed,
                           uint64_t sign_mask, uint64_t* states, float* t_abs, float* t_sign);
/* Start vector over the built basis: v_r = prior(r) sign(s_r) exp(a_r) / n_r,
 * scaled so the largest configuration amplitude is 1; out holds D doubles.
 * Pass it to sed_eigh as SED_START_GIVEN. */
SED_API int sed_mlp_start_vector(sed_mlp* mlp, ls_spin_basis const* basis, double* out);

/* Patch network: the same three layers applied to the `patch` spins around
 * each of the n_sites sites (patch_sites[i * patch + j] = the j-th site of
 * site i's patch) and summed over the sites,
 *   (a, s) = W3 sum_i tanh(W2 tanh(W1 x_i + b1) + b2) + b3,
 * with the parameter layout of sed_mlp_create for n_inputs = patch. The
 * parameters do not depend on the lattice: sed_mlp_set_patch_sites binds the
 * network to another lattice with the same patch shape (for example one
 * trained on a 4x4 torus to a 6x6 torus). patch <= 64, hidden 64, 128 or 256,
 * n_sites <= 64; training and inference run on the tensor cores only. */
SED_API int sed_mlp_create_patch(sed_mlp** out, unsigned n_sites, unsigned patch, uint16_t const* patch_sites,
                                 unsigned hidden, uint64_t sign_mask, uint64_t seed);
SED_API int sed_mlp_set_patch_sites(sed_mlp* mlp, unsigned n_sites, uint16_t const* patch_sites, uint64_t sign_mask);

/* Path of every pass. AUTO uses the tensor cores (tcgen05, BF16 operands,
 * FP32 accumulation in tensor memory) when n_inputs <= 64 and hidden is 128,
 * 256 or 512. Inference (sed_mlp_forward, sed_mlp_start_vector) then runs the
 * whole network in one fused kernel per 128 states, h1 rounded to BF16
 * between the layers and tanh the hardware approximation. Training
 * (sed_mlp_loss_grad, sed_mlp_train) runs each product as a tensor-core GEMM
 * with h1, h2 and the backward activations stored in BF16 (the bias
 * gradients sum them before the rounding). SIMT keeps every product on the
 * CUDA cores with FP32 activations. */
enum { SED_MLP_PATH_AUTO = 0, SED_MLP_PATH_SIMT = 1 };
SED_API int sed_mlp_set_path(sed_mlp* mlp, int path);
/* 1 if inference runs on the tensor cores, else 0. */
SED_API int sed_mlp_uses_tensor_cores(sed_mlp const* mlp);

/* sed_eigh keeps its largest Krylov workspace (the stored basis vectors)
 * allocated on each device between calls, because freeing tens of GB costs
 * about 20 ms per call; it is released automatically when another libsed
 * allocation runs out of memory. This frees it now (all devices). */
SED_API void sed_release_workspace(void);

/* A cap on the device memory libsed holds (all its buffers on all devices,
 * the cached Krylov workspace included); 0 removes it. An allocation that
 * would exceed it first releases the cached workspace, then fails with
 * LS_OUT_OF_MEMORY, as a cudaMalloc that runs out of memory does. The cap
 * lets a process that shares a GPU bound libsed's share of it. */
SED_API void sed_set_device_memory_limit(uint64_t bytes);
/* Device bytes libsed holds now. */
SED_API uint64_t sed_device_memory_in_use(void);

/* Bound on every wait inside libsed kernels that wait on other threads or
 * blocks: the group barriers of sed_eigh_batched's persistent kernel (20 s by
 * default) and its waits for shared-memory copies (1 s by default), and the
 * tensor-core kernels' waits on their copies and MMAs (1 s by default). A wait that runs out sets an error flag, the kernel drains
 * and returns, and the call fails with LS_DEVICE_TIMEOUT; the CUDA context
 * stays usable. seconds <= 0 restores the defaults. Process-wide. */
SED_API void sed_set_device_wait_limit(double seconds);
/* Test hook: the number of arrivals each batched group barrier waits for
 * beyond its own CTAs (0 in normal use). With n > 0 every barrier waits for
 * CTAs that do not exist, so its bounded wait runs out and sed_eigh_batched
 * reports LS_DEVICE_TIMEOUT; tests use it to exercise that path without a
 * GPU fault. Process-wide. */
SED_API void sed_debug_barrier_extra_arrivals(unsigned n);
/* Test hook: the group layout sed_eigh_batched uses on `grid` CTAs for
 * `count` problems of modelled work work[i] (a block step on n CTAs costs
 * fixed + work[i] / n) and at most max_ctas[i] CTAs each. Writes group_of[i],
 * the group of problem i, and per group g below the returned number of
 * groups its CTA count ncta[g] and problem count nprob[g] (ncta and nprob
 * hold `grid` entries). Groups take consecutive CTAs in index order.
 * Returns 0 on invalid arguments. Host only. */
SED_API unsigned sed_debug_batched_layout(unsigned count, double const* work, uint32_t const* max_ctas, double fixed,
                                          unsigned grid, uint32_t* group_of, uint32_t* ncta, uint32_t* nprob);

/* Number of libsed kernels launched by this process so far (graph replays
 * count their kernel nodes). */
SED_API uint64_t sed_kernel_launches(void);

/* Version string of the library (static storage). */
SED_API char const* sed_version(void);

#ifdef __cplusplus
}
#endif
#endif
