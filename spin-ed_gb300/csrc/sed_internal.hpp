// sed_internal.hpp — object model shared by the libsed translation units.
//
// The opaque handles of sed.h wrap reference-counted payloads: SpinED hands
// every handle to a GHC finaliser (src/SpinED/Internal.hs:116,150,228,362,402)
// and only keeps the basis alive while ls_create_operator runs
// (Internal.hs:391-402), so an operator owns a reference to its basis data.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <memory>
#include <initializer_list>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sed.h"
#include "canon.cuh"

namespace sed {

// ---------------------------------------------------------------- errors ---
int fail(int status, std::string const& message);  // records message, returns status
std::string last_message();
bool logging_enabled();
void log_line(char const* fmt, ...);

#define SED_TRY_CUDA(expr)                                                              \
  do {                                                                                  \
    cudaError_t sed_err_ = (expr);                                                      \
    if (sed_err_ != cudaSuccess)                                                        \
      return ::sed::fail(LS_CUDA_ERROR, std::string(#expr) + ": " +                     \
                                            cudaGetErrorString(sed_err_));              \
  } while (0)

// ------------------------------------------------------- device buffers ---
// Owns a device allocation; frees it on the device that made it, from any
// host thread.
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
  int device = -1;
  DeviceBuffer() = default;
  DeviceBuffer(DeviceBuffer const&) = delete;
  DeviceBuffer& operator=(DeviceBuffer const&) = delete;
  DeviceBuffer(DeviceBuffer&& o) noexcept { swap(o); }
  DeviceBuffer& operator=(DeviceBuffer&& o) noexcept {
    reset();
    swap(o);
    return *this;
  }
  ~DeviceBuffer() { reset(); }
  void swap(DeviceBuffer& o) noexcept {
    std::swap(ptr, o.ptr);
    std::swap(bytes, o.bytes);
    std::swap(device, o.device);
  }
  int allocate(size_t n);  // LS_* status
  void reset();
  template <class T>
  T* as() const {
    return static_cast<T*>(ptr);
  }
};

// A device buffer of at least `bytes` for a Krylov basis on the current
// device: the cached one when it is big enough, else a new allocation.
int krylov_take(size_t bytes, DeviceBuffer& out);
// Returns a Krylov basis buffer: the larger of it and the cached one stays
// cached (sed_eigh keeps its workspace between calls: freeing tens of GB
// costs about 20 ms per call), the other is freed.
void krylov_give(DeviceBuffer& b);

struct ScopedDevice {
  int previous = -1;
  explicit ScopedDevice(int device);
  ~ScopedDevice();
};

// ------------------------------------------------------------- symmetry ---
struct SymmetryData {
  std::vector<uint8_t> perm;  // y_i = x_{perm[i]}
  unsigned sector = 0;
  unsigned periodicity = 1;
};

struct GroupData {
  unsigned n = 0;                  // 0: trivial group of unspecified size
  std::vector<uint8_t> perms;      // [size][n], element 0 is the identity
  std::vector<uint32_t> phase;     // numerators mod L
  unsigned L = 1;
  std::vector<SymmetryData> generators;
  unsigned size() const { return n ? (unsigned)phase.size() : 1u; }
};

// Host-side symmetry plan; `view()` exposes it to canon.cuh.
struct SymPlanHost {
  unsigned n_bits = 0;
  uint64_t mask = 0;
  int inv = 0;
  unsigned L = 1;
  unsigned inv_phase = 0;
  unsigned group_order = 1;         // including inversion
  unsigned n_cosets = 1, n_h = 1, n_stages = 0, n_terms = 1;
  std::vector<uint64_t> benes_mask;  // [n_cosets][n_stages]
  std::vector<uint64_t> full_nets;   // [n_cosets][SED_MAX_STAGES] unpruned networks
  std::vector<uint8_t> pos;          // [n_cosets][64] landing position of each bit
  std::vector<uint32_t> benes_shift; // [n_stages]
  std::vector<uint64_t> h_mask;      // [n_h][n_terms]
  std::vector<uint32_t> h_rot;       // [n_h][n_terms] left-rotate amounts
  std::vector<uint32_t> coset_phase; // [n_cosets]
  std::vector<uint32_t> h_phase;     // [n_h]
  // H = <g1> x <g2> as nested cyclic loops (cyc = 0: explicit list above)
  unsigned cyc = 0;
  unsigned cyc_ord[2] = {1, 1};
  unsigned cyc_phase[2] = {0, 0};
  unsigned cyc_rot[2][2] = {{0, 0}, {0, 0}};
  uint64_t cyc_mask[2][2] = {{0, 0}, {0, 0}};
  // row structure (see PlanView::rows)
  unsigned rows = 0, row_bits = 0, n_rows = 1, rot_phase = 0, shift_phase = 0;
  uint64_t row_mask = 0;
  std::vector<uint16_t> row_min, row_set;
  std::vector<uint64_t> rot_mask, sh_mask;
  std::vector<uint32_t> rot_rot, rot_exp, sh_rot, sh_exp;
  // line tables (see PlanView::line_fast)
  unsigned line_fast = 0, line_cols = 0, col_s = 0;
  uint64_t col_m = 0, col_k = 0;
  std::vector<uint16_t> line_row, line_col;
  PlanView view() const;
};

// self_check: also run check_plan (otherwise the caller runs it before the
// plan's first use; ls_build overlaps it with the basis scan).
int build_plan(GroupData const& group, unsigned n_bits, int spin_inversion, SymPlanHost& out,
               bool self_check = true);
int check_plan(SymPlanHost const& plan);

// ---------------------------------------------------------------- basis ---
struct BasisData {
  int device = -1;
  unsigned n = 0;
  int hw = -1;
  int inv = 0;
  GroupData group;
  SymPlanHost plan;
  bool plan_checked = false;  // check_plan has passed (run by the first ls_build or host lookup)
  // device copy of the plan arrays (one allocation) and the view onto it
  DeviceBuffer plan_buf;
  PlanView plan_dev{};
  DeviceBuffer binom;  // [65][65] uint64
  // built state
  bool built = false;
  uint64_t D = 0;
  DeviceBuffer reps;     // uint64[D]
  DeviceBuffer weights;  // uint32[D] stabiliser orders
  DeviceBuffer prefix;   // uint64[(1 << prefix_bits) + 1]
  unsigned prefix_bits = 0, prefix_shift = 0;
  std::vector<uint32_t> s_values;  // distinct stabiliser orders (ascending)
  std::mutex mu;
  IndexView index_view() const;
};

int basis_upload_plan(BasisData& b, cudaStream_t stream);
int basis_build_index(BasisData& b, cudaStream_t stream);

// ----------------------------------------------------------- interaction ---
struct InteractionData {
  unsigned k = 2;
  std::vector<double> matrix;  // interleaved complex, (2^k)^2 entries
  std::vector<uint16_t> sites; // [n_tuples][k]
  bool is_real = true;
};

// -------------------------------------------------------------- operator ---
struct StreamForm {
  bool ready = false;
  bool packed = true;           // u32 entries: col | code << col_bits
  unsigned col_bits = 0;
  uint64_t n_slices = 0;
  uint64_t n_entries = 0;       // padded slots
  uint64_t n_elements = 0;      // generated off-diagonal elements
  DeviceBuffer slice_ptr;       // uint64[n_slices + 1] (slot offsets)
  DeviceBuffer entries;         // uint32[n_entries] (packed) or col array
  DeviceBuffer values;          // double[n_entries] (unpacked form)
  DeviceBuffer diag;            // double or double2 [D]
  DeviceBuffer row_class;       // uint8[D] stabiliser class of the row
  DeviceBuffer table;           // value table for codes (double or double2)
  DeviceBuffer inv_sqrt_s;      // double[n classes]
  unsigned n_codes = 0;
  double seconds = 0;
  bool orbit_table = false;     // recorded through the orbit table
  // FP32 companions for the mixed-precision Krylov phase (real operators)
  DeviceBuffer diag_f;   // float[D]
  DeviceBuffer table_f;  // float[n_codes]
  DeviceBuffer invs_f;   // float[n classes]
  uint64_t bytes() const {
    return slice_ptr.bytes + entries.bytes + values.bytes + diag.bytes + row_class.bytes +
           table.bytes + inv_sqrt_s.bytes;
  }
};

struct OperatorTables;  // value tables, defined in operator.cu

struct OperatorData {
  std::shared_ptr<BasisData> basis;
  std::vector<InteractionData> terms;
  bool is_real = true;
  // device term tables
  DeviceBuffer term_buf;
  TermsView terms_dev{};
  std::vector<double> off_values;  // distinct off-diagonal matrix values (re, im)
  uint64_t row_bound = 0;          // most off-diagonal elements any row can generate
  StreamForm stream;
  std::unique_ptr<OperatorTables> tables;
  int form = SED_FORM_AUTO;  // selected by sed_operator_prepare
  cudaStream_t cuda_stream = nullptr;
  // fixed-point matvec workspace (see operator_impl.cuh): u for fix_cols
  // columns, then per column the max |x| bit pattern and the exponent F;
  // fix_event orders its reuse across the callers' streams
  DeviceBuffer fix_u;
  DeviceBuffer fix_slots;
  uint32_t fix_cols = 0;
  cudaEvent_t fix_event = nullptr;
  bool fix_event_recorded = false;
  // the FP32-stored Krylov phase's gather copy: u_j in int32, then its slots
  DeviceBuffer fix_u32;
  DeviceBuffer fix_slots32;
  std::mutex mu;
  ~OperatorData();
};

int operator_upload_terms(OperatorData& op);
// Entry points that take caller buffers and run on a libsed stream call this
// first: when any of the pointers is device memory, it waits for all work
// already queued on the device, since the caller may have written the buffer
// (or may still be reading it) on a stream of its own. Host pointers need no
// wait. Returns a status.
int wait_for_caller(std::initializer_list<void const*> buffers);
int operator_record_stream(OperatorData& op, cudaStream_t stream);
int operator_apply_device(OperatorData& op, int dtype, uint64_t block, void const* x,
                          uint64_t ldx, void* y, uint64_t ldy, cudaStream_t stream, int form);
// Fixed-point matvec workspace for `cols` columns (no-op when the operator
// does not qualify or already has it), and a host wait for the last use of
// that workspace on any caller's stream.
int fix_reserve(OperatorData& op, uint32_t cols);
int fix_wait(OperatorData& op);
// FP32 companions of the stream form (mixed-precision Krylov phase).
int operator_prepare_fp32(OperatorData& op, cudaStream_t stream);

bool characters_real(BasisData const& b);
uint64_t host_binom(unsigned n, unsigned k);
// How the stream form is recorded (sed_set_record_mode).
extern int g_record_mode;

// sed_eigh's thick-restart solver (real operators, 0 < max_basis <= 32).
int solve_thick(OperatorData& op, int out_dtype, sed_eigh_options const& o, double* evals, void* evecs, uint64_t ldv,
                double* rnorms, sed_eigh_info* info);

// Bound on device-side waits (sed_set_device_wait_limit): the caller's
// limit in nanoseconds, or `default_ns` when none is set.
uint64_t device_wait_ns(uint64_t default_ns);
// Extra arrivals each batched group barrier waits for (0 in normal use; a
// test sets it so that the bounded barrier wait runs out).
extern std::atomic<uint32_t> g_barrier_extra_arrivals;

// Kernel-launch accounting (sed_kernel_launches): every launch site calls
// note_launches(1); launches made while capturing a graph are not counted,
// the graph's kernel nodes are counted at each replay instead.
void note_launches(uint64_t n);
void set_capturing(bool on);
int current_device(int* device);

}  // namespace sed

struct ls_symmetry {
  sed::SymmetryData d;
};
struct ls_group {
  sed::GroupData d;
};
struct ls_spin_basis {
  std::shared_ptr<sed::BasisData> d;
};
struct ls_states {
  std::unique_ptr<uint64_t[]> data;  // host copy of the representatives (not zero-filled first)
  uint64_t size = 0;
};
struct ls_interaction {
  sed::InteractionData d;
};
struct ls_operator {
  std::shared_ptr<sed::OperatorData> d;
};
