// capi.cu — error channel, logging and device-memory plumbing of libsed.
//
// Status convention of src/SpinED/Internal.hs:47-65: a non-zero status is
// turned into text by ls_error_to_string and freed by ls_destroy_string. The
// text carries the description of the code plus the detail recorded by the
// failing call on the same host thread.
#include <atomic>
#include <cstdarg>
#include <cstdlib>
#include <cstring>

#include "sed_internal.hpp"

namespace sed {
namespace {

thread_local int t_last_status = 0;
thread_local std::string t_last_message;
std::atomic<bool> g_logging{false};
std::atomic<uint64_t> g_launches{0};
thread_local bool t_capturing = false;

char const* describe(int status) {
  switch (status) {
    case LS_SUCCESS: return "success";
    case LS_OUT_OF_MEMORY: return "failed to allocate memory";
    case LS_INVALID_ARGUMENT: return "invalid argument";
    case LS_INVALID_HAMMING_WEIGHT: return "invalid Hamming weight";
    case LS_INVALID_SPIN_INVERSION: return "invalid spin inversion";
    case LS_INVALID_NUMBER_SPINS: return "invalid number of spins";
    case LS_INVALID_PERMUTATION: return "argument is not a valid permutation";
    case LS_INVALID_SECTOR: return "sector exceeds the periodicity of the operator";
    case LS_INVALID_STATE: return "invalid basis state";
    case LS_INVALID_DATATYPE: return "invalid datatype";
    case LS_PERMUTATION_TOO_LONG: return "permutation is too long";
    case LS_INCOMPATIBLE_SYMMETRIES: return "symmetries are incompatible";
    case LS_NOT_A_REPRESENTATIVE: return "argument is not a representative";
    case LS_WRONG_BASIS_TYPE: return "wrong basis type";
    case LS_CACHE_NOT_BUILT: return "basis cache has not been built";
    case LS_COULD_NOT_OPEN_FILE: return "could not open file";
    case LS_FILE_IO_FAILED: return "file input/output failed";
    case LS_CACHE_IS_CORRUPT: return "cache is corrupt";
    case LS_OPERATOR_IS_COMPLEX: return "operator is complex but a real datatype was requested";
    case LS_DIMENSION_MISMATCH: return "dimensions do not match";
    case LS_GROUP_TOO_BIG: return "symmetry group is too big";
    case LS_CUDA_ERROR: return "CUDA error";
    case LS_NOT_CONVERGED: return "eigensolver did not converge";
    case LS_DEVICE_TIMEOUT: return "a device-side wait timed out";
    case LS_SYSTEM_ERROR: return "internal error";
    default: return "unknown error";
  }
}

}  // namespace

int fail(int status, std::string const& message) {
  t_last_status = status;
  t_last_message = message;
  if (g_logging.load(std::memory_order_relaxed))
    std::fprintf(stderr, "[libsed] error %d: %s\n", status, message.c_str());
  return status;
}

std::string last_message() { return t_last_message; }
void note_launches(uint64_t n) {
  if (!t_capturing) g_launches.fetch_add(n, std::memory_order_relaxed);
}
void set_capturing(bool on) { t_capturing = on; }
bool logging_enabled() { return g_logging.load(std::memory_order_relaxed); }

void log_line(char const* fmt, ...) {
  if (!logging_enabled()) return;
  va_list ap;
  va_start(ap, fmt);
  std::fprintf(stderr, "[libsed] ");
  std::vfprintf(stderr, fmt, ap);
  std::fprintf(stderr, "\n");
  va_end(ap);
}

// One cached Krylov workspace per device (see krylov_take / krylov_give).
namespace {
constexpr int kCacheDevices = 64;
std::mutex g_cache_mu;
DeviceBuffer g_krylov_cache[kCacheDevices];

// Frees the cached workspace of `device` (all devices for -1).
void release_cache(int device) {
  std::lock_guard<std::mutex> lk(g_cache_mu);
  for (int d = 0; d < kCacheDevices; ++d)
    if (device < 0 || d == device) g_krylov_cache[d].reset();
}
}  // namespace

int krylov_take(size_t bytes, DeviceBuffer& out) {
  int dev = -1;
  if (int st = current_device(&dev)) return st;
  if (dev >= 0 && dev < kCacheDevices) {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    if (g_krylov_cache[dev].ptr && g_krylov_cache[dev].bytes >= bytes) {
      out = std::move(g_krylov_cache[dev]);
      return LS_SUCCESS;
    }
  }
  return out.allocate(bytes);
}

void krylov_give(DeviceBuffer& b) {
  if (!b.ptr) return;
  int const dev = b.device;
  if (dev >= 0 && dev < kCacheDevices) {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    if (b.bytes > g_krylov_cache[dev].bytes) std::swap(g_krylov_cache[dev], b);
  }
  b.reset();
}

namespace {
// Device bytes held by libsed buffers (all devices) and the caller's cap on
// them (sed_set_device_memory_limit; 0 = none).
std::atomic<uint64_t> g_dev_bytes{0};
std::atomic<uint64_t> g_dev_limit{0};

bool over_limit(size_t n) {
  uint64_t const lim = g_dev_limit.load();
  return lim && g_dev_bytes.load() + n > lim;
}
}  // namespace

std::atomic<uint64_t> g_wait_ns{0};
std::atomic<uint32_t> g_barrier_extra_arrivals{0};

uint64_t device_wait_ns(uint64_t default_ns) {
  uint64_t const w = g_wait_ns.load();
  return w ? w : default_ns;
}

int DeviceBuffer::allocate(size_t n) {
  reset();
  if (int st = current_device(&device)) return st;
  if (over_limit(n)) {
    release_cache(device);  // the cached Krylov workspace counts towards the cap
    if (over_limit(n))
      return fail(LS_OUT_OF_MEMORY, "libsed device-memory limit of " + std::to_string(g_dev_limit.load()) +
                                        " bytes: " + std::to_string(g_dev_bytes.load()) + " in use, " +
                                        std::to_string(n) + " more requested");
  }
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, n ? n : 1);
  if (e == cudaErrorMemoryAllocation) {
    // the cached Krylov workspace may hold the memory: free it and retry once
    cudaGetLastError();
    release_cache(device);
    e = cudaMalloc(&p, n ? n : 1);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(e == cudaErrorMemoryAllocation ? LS_OUT_OF_MEMORY : LS_CUDA_ERROR,
                "cudaMalloc(" + std::to_string(n) + " bytes): " + cudaGetErrorString(e));
  }
  ptr = p;
  bytes = n;
  g_dev_bytes.fetch_add(n);
  return LS_SUCCESS;
}

void DeviceBuffer::reset() {
  if (ptr) {
    int prev = -1;
    cudaGetDevice(&prev);
    if (device >= 0 && device != prev) cudaSetDevice(device);
    cudaFree(ptr);
    if (device >= 0 && device != prev && prev >= 0) cudaSetDevice(prev);
    g_dev_bytes.fetch_sub(bytes);
  }
  ptr = nullptr;
  bytes = 0;
}

ScopedDevice::ScopedDevice(int device) {
  cudaGetDevice(&previous);
  if (device >= 0 && device != previous) cudaSetDevice(device);
}
ScopedDevice::~ScopedDevice() {
  int now = -1;
  cudaGetDevice(&now);
  if (previous >= 0 && now != previous) cudaSetDevice(previous);
}

int current_device(int* device) {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail(LS_CUDA_ERROR, std::string("no CUDA device is available: ") +
                                   (e == cudaSuccess ? "device count is 0" : cudaGetErrorString(e)));
  }
  e = cudaGetDevice(device);
  if (e != cudaSuccess) return fail(LS_CUDA_ERROR, cudaGetErrorString(e));
  return LS_SUCCESS;
}

}  // namespace sed

using namespace sed;

extern "C" {

void sed_release_workspace(void) { release_cache(-1); }
void sed_set_device_memory_limit(uint64_t bytes) { g_dev_limit.store(bytes); }
void sed_set_device_wait_limit(double seconds) {
  g_wait_ns.store(seconds > 0 ? (uint64_t)(seconds * 1e9) : 0);
}
void sed_debug_barrier_extra_arrivals(unsigned n) { g_barrier_extra_arrivals.store(n); }
uint64_t sed_device_memory_in_use(void) { return g_dev_bytes.load(); }


char const* ls_error_to_string(int status) {
  std::string s = describe(status);
  if (status != LS_SUCCESS && status == t_last_status && !t_last_message.empty())
    s += ": " + t_last_message;
  char* out = static_cast<char*>(std::malloc(s.size() + 1));
  if (out) std::memcpy(out, s.c_str(), s.size() + 1);
  return out;
}

void ls_destroy_string(char const* message) { std::free(const_cast<char*>(message)); }
void ls_enable_logging(void) { g_logging.store(true); }
void ls_disable_logging(void) { g_logging.store(false); }
char const* sed_version(void) { return "libsed 0.1.0 (sm_103a)"; }
uint64_t sed_kernel_launches(void) { return g_launches.load(); }

}  // extern "C"
