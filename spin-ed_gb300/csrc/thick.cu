// thick.cu — thick-restart Lanczos for a small number of stored Krylov
// vectors (sed_eigh with 0 < max_basis <= 32 on a real operator).
//
// A cycle extends the basis v_0 .. v_{m-1} one vector at a time:
//   w = H v_k ; c = V^T w ; w -= V c (twice: CGS2) ; T[0..k][k] = c
//   beta = ||w|| ; v_{k+1} = w / beta ; T[k+1][k] = beta
// T is symmetric (tridiagonal plus, after a restart, an arrowhead), so every
// projection is kept. When the basis is full the m x m problem is solved on
// the host (cyclic Jacobi, FP64) and the lowest `keep` Ritz vectors replace
// v_0 .. v_{keep-1} in place (one pass over V, row by row), v_m becomes
// v_keep, and T restarts as diag(theta) — the next step's projections supply
// the arrowhead couplings beta_m y_{m-1,i} (Wu & Simon's thick restart).
// Converged pairs (estimate beta |y_{last,i}| <= tol / 2) are checked with
// their true residual ||H psi - theta psi|| computed in FP64.
//
// Storage S = double (SED_PRECISION_FP64) or float (SED_PRECISION_MIXED).
// With float the Krylov vectors and w are stored in FP32 and the phase
// computes in FP32 (the streamed FP32 SpMV; FP32 products in the
// projections with per-block partial sums in FP64), while T, its
// eigensolve, the Ritz vectors and their residuals are FP64. The FP32 phase
// stops at the FP32 floor (a residual of about 1e-6 of |theta|); its FP64
// Ritz vector then starts an FP64 thick-restart phase with at most 10 stored
// vectors that refines it to the tolerance.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "operator_impl.cuh"

namespace sed {
namespace {

constexpr int kMaxThick = 32;
constexpr int kDotCols = 8;

template <class S>
__device__ __forceinline__ double ldv(S const* p, uint64_t i) { return (double)p[i]; }

// Arithmetic type of the projections: FP64 for FP64 storage; for FP32
// storage FP32 products and per-thread sums (GB300's FP64 pipe is slower
// than HBM for these streams, and converting every FP32 element to FP64
// would occupy it too), with the per-thread partials summed in FP64.
template <class S>
struct Arith {
  using T = double;
};
template <>
struct Arith<float> {
  using T = float;
};

// partial[(g * gridDim.x + b) * kDotCols + c] = sum over this block's rows
// of V[:, NC g + c] . w for c < NC (columns >= ncols give 0); blockIdx.y = g.
// NC is a template parameter: on GB300 a predicated-off FP64 FMA still takes
// its issue slot on the slow FP64 pipe, so the column count of a launch is
// matched exactly instead of padding to a fixed width.
template <class S, int NC>
__global__ void __launch_bounds__(256) k_tdots(S const* __restrict__ V, uint64_t ld, uint32_t ncols,
                                               S const* __restrict__ w, uint64_t D, double* __restrict__ partial) {
  using T = typename Arith<S>::T;
  __shared__ double red[8][NC];
  uint32_t const c0 = blockIdx.y * NC;
  uint32_t const nc = ncols - c0 < (uint32_t)NC ? ncols - c0 : (uint32_t)NC;
  S const* const Vc = V + (uint64_t)c0 * ld;
  T acc[NC] = {};
  if (nc == (uint32_t)NC) {
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < D; r += (uint64_t)gridDim.x * blockDim.x) {
      T const wr = (T)w[r];
#pragma unroll
      for (int c = 0; c < NC; ++c) acc[c] = fma((T)Vc[(uint64_t)c * ld + r], wr, acc[c]);
    }
  } else {  // short last group (at most NC - 1 predicated-off columns)
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < D; r += (uint64_t)gridDim.x * blockDim.x) {
      T const wr = (T)w[r];
#pragma unroll
      for (int c = 0; c < NC; ++c)
        if (c < (int)nc) acc[c] = fma((T)Vc[(uint64_t)c * ld + r], wr, acc[c]);
    }
  }
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    double x = (double)acc[c];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][c] = x;
  }
  __syncthreads();
  if (threadIdx.x < NC) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q][threadIdx.x];
    partial[((uint64_t)blockIdx.y * gridDim.x + blockIdx.x) * kDotCols + threadIdx.x] = s;
  }
}

// Launch of k_tdots over ncols columns in g = ceil(ncols / 8) groups of
// NC = ceil(ncols / g) columns; returns NC.
template <class S>
int launch_tdots(S const* V, uint64_t ld, uint32_t ncols, S const* w, uint64_t D, double* partial, unsigned vb,
                 cudaStream_t stream) {
  uint32_t const g = (ncols + kDotCols - 1) / kDotCols;
  int const nc = (int)((ncols + g - 1) / g);
  dim3 const grid(vb, g);
  switch (nc) {
#define SED_TDOTS(N) \
  case N: { k_tdots<S, N><<<grid, 256, 0, stream>>>(V, ld, ncols, w, D, partial); note_launches(1); } break;
    SED_TDOTS(1) SED_TDOTS(2) SED_TDOTS(3) SED_TDOTS(4) SED_TDOTS(5) SED_TDOTS(6) SED_TDOTS(7) SED_TDOTS(8)
#undef SED_TDOTS
  }
  return nc;
}

// w -= sum_{c < ncols} V[:, c] coef[c]  (FP64 arithmetic)
template <class S>
__global__ void k_tupdate(S const* __restrict__ V, uint64_t ld, uint32_t ncols, double const* __restrict__ coef,
                          S* __restrict__ w, uint64_t D) {
  using T = typename Arith<S>::T;
  __shared__ T cf[kMaxThick + 1];
  for (uint32_t c = threadIdx.x; c < ncols; c += blockDim.x) cf[c] = (T)coef[c];
  __syncthreads();
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < D; r += (uint64_t)gridDim.x * blockDim.x) {
    T x = (T)w[r];
    for (uint32_t c = 0; c < ncols; ++c) x = fma(-(T)V[(uint64_t)c * ld + r], cf[c], x);
    w[r] = (S)x;
  }
}

template <class S>
__global__ void k_tscale(S const* __restrict__ w, uint64_t D, double f, S* __restrict__ out) {
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < D; r += (uint64_t)gridDim.x * blockDim.x)
    out[r] = (S)(ldv(w, r) * f);
}

// In place, row by row: V[:, c] <- sum_{i < m} V[:, i] Y[i * kk + c] for
// c < kk <= 4 KB. The kk sums of a row are independent chains, one FMA of
// each per V value; KB is a template parameter so that at most three
// predicated-off FMAs per V value take FP64 issue slots.
template <class S, int KB>
__global__ void k_trotate(S* __restrict__ V, uint64_t ld, uint32_t m, double const* __restrict__ Y, uint32_t kk,
                          uint64_t D) {
  constexpr int KC = 4 * KB;
  __shared__ double y[kMaxThick * KC];
  for (uint32_t e = threadIdx.x; e < m * KC; e += blockDim.x) {
    uint32_t const i = e / KC, c = e % KC;
    y[e] = c < kk ? Y[i * kk + c] : 0.0;
  }
  __syncthreads();
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < D; r += (uint64_t)gridDim.x * blockDim.x) {
    double acc[KC];
#pragma unroll
    for (int c = 0; c < KC; ++c) acc[c] = 0.0;
    for (uint32_t i = 0; i < m; ++i) {
      double const vi = ldv(V, (uint64_t)i * ld + r);
#pragma unroll
      for (int c = 0; c < KC; ++c) acc[c] = fma(vi, y[i * KC + c], acc[c]);
    }
#pragma unroll
    for (int c = 0; c < KC; ++c)
      if (c < (int)kk) V[(uint64_t)c * ld + r] = (S)acc[c];
  }
}

template <class S>
void launch_trotate(S* V, uint64_t ld, uint32_t m, double const* Y, uint32_t kk, uint64_t D, unsigned vb,
                    cudaStream_t stream) {
  switch ((kk + 3) / 4) {
#define SED_TROT(N) \
  case N: { k_trotate<S, N><<<vb, 256, 0, stream>>>(V, ld, m, Y, kk, D); note_launches(1); } break;
    SED_TROT(1) SED_TROT(2) SED_TROT(3) SED_TROT(4) SED_TROT(5) SED_TROT(6) SED_TROT(7) SED_TROT(8)
#undef SED_TROT
  }
}

// V[:, 0..kk) <- V[:, 0..m) Y: on the tensor cores for FP64 storage when
// the shape allows it (and the path setting does not forbid it), else the
// FP64-FMA kernel above. `err` is a device int for the tensor-core kernel's
// bounded waits; a set flag is reported as LS_DEVICE_TIMEOUT.
template <class S>
int rotate_basis(S* V, uint64_t ld, uint32_t m, double const* Y, uint32_t kk, uint64_t D, unsigned vb,
                 cudaStream_t stream, int path, int* err) {
  if constexpr (std::is_same<S, double>::value) {
    // AUTO takes the tensor cores where they measured faster than the FP64
    // pipe (m >= 16: 68 against 82 ms for m = 32, kk = 16 on 1e8 rows; at
    // m = 12, kk = 6 the two tie, 16.1 against 15.7 ms)
    bool const tc = path == SED_ROTATE_TENSOR || (path == SED_ROTATE_AUTO && m >= 16);
    if (tc && rotate_tc_eligible(m, kk)) {
      SED_TRY_CUDA(cudaMemsetAsync(err, 0, 4, stream));
      if (int st = rotate_tc(V, ld, m, Y, kk, D, stream, err)) return st;
      int h = 0;
      SED_TRY_CUDA(cudaMemcpyAsync(&h, err, 4, cudaMemcpyDeviceToHost, stream));
      SED_TRY_CUDA(cudaStreamSynchronize(stream));
      if (h) return fail(LS_DEVICE_TIMEOUT, "basis rotation: a wait on the tensor cores timed out");
      return LS_SUCCESS;
    }
  }
  if (path == SED_ROTATE_TENSOR)
    return fail(LS_INVALID_ARGUMENT, "basis rotation on the tensor cores needs FP64, m <= 32 and kk <= 16");
  launch_trotate<S>(V, ld, m, Y, kk, D, vb, stream);
  SED_TRY_CUDA(cudaGetLastError());
  return LS_SUCCESS;
}

// psi = sum_{i < m} V[:, i] y[i]  (FP64 output)
template <class S>
__global__ void k_tritz(S const* __restrict__ V, uint64_t ld, uint32_t m, double const* __restrict__ yv, uint64_t D,
                        double* __restrict__ psi) {
  __shared__ double y[kMaxThick];
  for (uint32_t e = threadIdx.x; e < m; e += blockDim.x) y[e] = yv[e];
  __syncthreads();
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < D; r += (uint64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (uint32_t i = 0; i < m; ++i) s = fma(ldv(V, (uint64_t)i * ld + r), y[i], s);
    psi[r] = s;
  }
}

// partial[b] = (sum (w - theta psi)^2, sum psi^2) over this block's rows
__global__ void k_tresid(double const* __restrict__ psi, double const* __restrict__ w, double theta, uint64_t D,
                         double* __restrict__ partial) {
  __shared__ double red[2][8];
  double a = 0.0, b = 0.0;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < D; r += (uint64_t)gridDim.x * blockDim.x) {
    double const d = w[r] - theta * psi[r];
    a = fma(d, d, a);
    b = fma(psi[r], psi[r], b);
  }
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if (lane == 0) {
    red[0][warp] = a;
    red[1][warp] = b;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[threadIdx.x][q];
    partial[2 * blockIdx.x + threadIdx.x] = s;
  }
}

template <class S>
__global__ void k_trandom(S* __restrict__ x, uint64_t D, uint64_t seed) {
  for (uint64_t blk = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; blk < (D + 1) / 2;
       blk += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t c[4] = {(uint32_t)blk, (uint32_t)(blk >> 32), 0u, 0u};
    philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    x[2 * blk] = (S)(2.0 * u01_53(c[0], c[1]) - 1.0);
    if (2 * blk + 1 < D) x[2 * blk + 1] = (S)(2.0 * u01_53(c[2], c[3]) - 1.0);
  }
}

template <class S>
__global__ void k_tconvert(double const* __restrict__ a, uint64_t D, S* __restrict__ b) {
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < D; r += (uint64_t)gridDim.x * blockDim.x)
    b[r] = (S)a[r];
}

// Cyclic Jacobi eigendecomposition of the symmetric n x n matrix A (row
// major, destroyed); eigenvalues ascending in w, eigenvectors as columns of
// Z (row major n x n).
void jacobi_host(std::vector<double> A, int n, std::vector<double>& w, std::vector<double>& Z) {
  Z.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) Z[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, dia = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) (i == j ? dia : off) += A[(size_t)i * n + j] * A[(size_t)i * n + j];
    if (off <= 1e-32 * dia || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double const apq = A[(size_t)p * n + q];
        if (apq == 0.0) continue;
        double const tau = (A[(size_t)q * n + q] - A[(size_t)p * n + p]) / (2.0 * apq);
        double const t = (tau >= 0.0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        double const c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        for (int k = 0; k < n; ++k) {  // rows p, q
          double const ap = A[(size_t)p * n + k], aq = A[(size_t)q * n + k];
          A[(size_t)p * n + k] = c * ap - s * aq;
          A[(size_t)q * n + k] = s * ap + c * aq;
        }
        for (int k = 0; k < n; ++k) {  // columns p, q
          double const ap = A[(size_t)k * n + p], aq = A[(size_t)k * n + q];
          A[(size_t)k * n + p] = c * ap - s * aq;
          A[(size_t)k * n + q] = s * ap + c * aq;
          double const zp = Z[(size_t)k * n + p], zq = Z[(size_t)k * n + q];
          Z[(size_t)k * n + p] = c * zp - s * zq;
          Z[(size_t)k * n + q] = s * zp + c * zq;
        }
      }
  }
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int a, int b) { return A[(size_t)a * n + a] < A[(size_t)b * n + b]; });
  w.resize(n);
  std::vector<double> Zs((size_t)n * n);
  for (int c = 0; c < n; ++c) {
    w[c] = A[(size_t)order[c] * n + order[c]];
    for (int r = 0; r < n; ++r) Zs[(size_t)r * n + c] = Z[(size_t)r * n + order[c]];
  }
  Z.swap(Zs);
}

int elem_bytes_of(int dtype) { return dtype == 0 ? 4 : dtype == 1 ? 8 : dtype == 2 ? 8 : 16; }

__global__ void k_tout(double const* __restrict__ a, uint64_t D, int dtype, void* __restrict__ out) {
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < D; r += (uint64_t)gridDim.x * blockDim.x) {
    double const v = a[r];
    switch (dtype) {
      case 0: static_cast<float*>(out)[r] = (float)v; break;
      case 1: static_cast<double*>(out)[r] = v; break;
      case 2: static_cast<float2*>(out)[r] = make_float2((float)v, 0.0f); break;
      default: static_cast<double2*>(out)[r] = make_double2(v, 0.0); break;
    }
  }
}

// FP64 device vector -> dst (host or device) of the given dtype.
int store_vector(double const* v, uint64_t D, int dtype, void* dst, cudaStream_t stream) {
  DeviceBuffer tmp;
  size_t const bytes = D * (size_t)elem_bytes_of(dtype);
  if (int st = tmp.allocate(bytes)) return st;
  { k_tout<<<grid_size(D, 0, 4), 256, 0, stream>>>(v, D, dtype, tmp.ptr); note_launches(1); }
  SED_TRY_CUDA(cudaGetLastError());
  SED_TRY_CUDA(cudaMemcpyAsync(dst, tmp.ptr, bytes, cudaMemcpyDefault, stream));
  SED_TRY_CUDA(cudaStreamSynchronize(stream));
  return LS_SUCCESS;
}

struct ThickResult {
  std::vector<double> theta, resid;
  uint64_t steps = 0, matvecs = 0, restarts = 0;
  bool converged = false;
};

// One thick-restart run with storage S. start: FP64 D-vector (device) or
// null for the Philox start. With rel_floor = 0 it stops when the nev lowest
// true residuals are <= tol_true; with rel_floor > 0 (the FP32 phase) it
// stops as soon as every estimate is below max(tol_true / 2, rel_floor
// max(1, |theta_0|)). The nev Ritz vectors (FP64, normalised) are left in psi
// (D x nev).
template <class S>
int thick_run(OperatorData& op, cudaStream_t stream, uint32_t m, uint32_t nev, double tol_true, double rel_floor,
              double const* start, uint64_t seed, uint64_t max_steps, double* psi, ThickResult& out) {
  uint64_t const D = op.basis->D;
  int const dtype = std::is_same<S, float>::value ? 0 : 1;
  int const dev = op.basis->device;
  unsigned const vb = grid_size(D, dev, 4);
  uint32_t const groups = (m + 1 + kDotCols - 1) / kDotCols;
  DeviceBuffer Vb, wb, w64, part, coef, Yb, rt_err;
  if (int st = rt_err.allocate(4)) return st;
  if (int st = Vb.allocate((size_t)(m + 1) * D * sizeof(S))) return st;
  if (int st = wb.allocate(D * sizeof(S))) return st;
  if (int st = w64.allocate(D * 8)) return st;
  if (int st = part.allocate((size_t)groups * vb * kDotCols * 8 + 16 * (size_t)vb)) return st;
  if (int st = coef.allocate((kMaxThick + 1) * 8)) return st;
  if (int st = Yb.allocate((size_t)kMaxThick * kMaxThick * 8)) return st;
  S* V = Vb.as<S>();
  S* w = wb.as<S>();
  std::vector<double> hp((size_t)groups * vb * kDotCols);
  // res[c] = V[:, first + c] . x for c < ncols
  auto dots_at = [&](uint32_t first, uint32_t ncols, S const* x, std::vector<double>& res) -> int {
    uint32_t const g = (ncols + kDotCols - 1) / kDotCols;
    int const nc = launch_tdots<S>(V + (uint64_t)first * D, D, ncols, x, D, part.as<double>(), vb, stream);
    SED_TRY_CUDA(cudaGetLastError());
    SED_TRY_CUDA(cudaMemcpyAsync(hp.data(), part.ptr, (size_t)g * vb * kDotCols * 8, cudaMemcpyDeviceToHost, stream));
    SED_TRY_CUDA(cudaStreamSynchronize(stream));
    res.assign(ncols, 0.0);
    for (uint32_t gg = 0; gg < g; ++gg)
      for (unsigned b = 0; b < vb; ++b)
        for (int c = 0; c < nc; ++c)
          if (gg * nc + c < ncols) res[gg * nc + c] += hp[((size_t)gg * vb + b) * kDotCols + c];
    return LS_SUCCESS;
  };
  auto dots = [&](uint32_t ncols, S const* x, std::vector<double>& res) -> int { return dots_at(0, ncols, x, res); };
  auto norm = [&](S const* x, double& nrm) -> int {
    // ||x||: dots of column 0 of a one-column "V" = x itself
    launch_tdots<S>(x, D, 1, x, D, part.as<double>(), vb, stream);
    SED_TRY_CUDA(cudaMemcpyAsync(hp.data(), part.ptr, (size_t)vb * kDotCols * 8, cudaMemcpyDeviceToHost, stream));
    SED_TRY_CUDA(cudaStreamSynchronize(stream));
    double s = 0.0;
    for (unsigned b = 0; b < vb; ++b) s += hp[(size_t)b * kDotCols];
    nrm = std::sqrt(s);
    return LS_SUCCESS;
  };
  // v_0
  if (start) {
    { k_tconvert<S><<<vb, 256, 0, stream>>>(start, D, V); note_launches(1); }
  } else {
    { k_trandom<S><<<vb, 256, 0, stream>>>(V, D, seed); note_launches(1); }
  }
  double n0 = 0.0;
  if (int st = norm(V, n0)) return st;
  if (!(n0 > 0.0)) return fail(LS_INVALID_ARGUMENT, "sed_eigh: zero start vector");
  { k_tscale<S><<<vb, 256, 0, stream>>>(V, D, 1.0 / n0, V); note_launches(1); }

  std::vector<double> T((size_t)(m + 1) * (m + 1), 0.0);
  auto Tij = [&](uint32_t i, uint32_t j) -> double& { return T[(size_t)i * (m + 1) + j]; };
  uint32_t k = 0;      // index of the newest basis vector
  uint32_t arrow = 0;  // index of the continuation vector after the last restart (0: none)
  std::vector<double> c, c2, theta, Z;
  out = ThickResult{};
  while (true) {
    // ---- one Lanczos step from v_k
    if constexpr (std::is_same<S, float>::value) {
      if (op.stream.ready && op.stream.diag_f.ptr) {
        if (int st = operator_apply32(op, V + (uint64_t)k * D, w, stream)) return st;
      } else if (int st = operator_apply_device(op, dtype, 1, V + (uint64_t)k * D, D, w, D, stream, SED_FORM_AUTO)) {
        return st;
      }
    } else if (int st = operator_apply_device(op, dtype, 1, V + (uint64_t)k * D, D, w, D, stream, SED_FORM_AUTO)) {
      return st;
    }
    ++out.matvecs;
    ++out.steps;
    // Orthogonalisation, two passes. Away from the continuation vector of a
    // restart, H v_k has (in exact arithmetic) components along v_{k-1} and
    // v_k only, so the first pass projects out those two; the second pass
    // runs against the whole basis and removes what rounding left along any
    // stored vector. On the step from the continuation vector (whose column
    // of the projected matrix is an arrowhead over the kept Ritz vectors)
    // both passes are full.
    uint32_t const first = k > arrow ? k - 1 : 0;
    if (int st = dots_at(first, k + 1 - first, w, c)) return st;
    SED_TRY_CUDA(cudaMemcpyAsync(coef.ptr, c.data(), (k + 1 - first) * 8, cudaMemcpyHostToDevice, stream));
    { k_tupdate<S><<<vb, 256, 0, stream>>>(V + (uint64_t)first * D, D, k + 1 - first, coef.as<double>(), w, D); note_launches(1); }
    c.insert(c.begin(), first, 0.0);
    if (int st = dots(k + 1, w, c2)) return st;
    SED_TRY_CUDA(cudaMemcpyAsync(coef.ptr, c2.data(), (k + 1) * 8, cudaMemcpyHostToDevice, stream));
    { k_tupdate<S><<<vb, 256, 0, stream>>>(V, D, k + 1, coef.as<double>(), w, D); note_launches(1); }
    for (uint32_t i = 0; i <= k; ++i) {
      double const v = c[i] + c2[i];
      if (i == k) Tij(k, k) = v;
      else Tij(i, k) = Tij(k, i) = v;
    }
    double beta = 0.0;
    if (int st = norm(w, beta)) return st;
    bool const breakdown = !(beta > 1e-14 * std::max(1.0, std::fabs(Tij(k, k))));
    if (!breakdown) {
      { k_tscale<S><<<vb, 256, 0, stream>>>(w, D, 1.0 / beta, V + (uint64_t)(k + 1) * D); note_launches(1); }
      Tij(k + 1, k) = Tij(k, k + 1) = beta;
    } else {
      beta = 0.0;
    }
    uint32_t const n = k + 1;  // order of the projected problem
    bool const full = n >= m || breakdown || out.steps >= max_steps;
    if (!full && n % 4 != 0) {
      k = n;
      continue;
    }
    // ---- Rayleigh-Ritz on T[0..n)
    std::vector<double> A((size_t)n * n);
    for (uint32_t i = 0; i < n; ++i)
      for (uint32_t j = 0; j < n; ++j) A[(size_t)i * n + j] = Tij(i, j);
    jacobi_host(A, (int)n, theta, Z);
    uint32_t const want = std::min<uint32_t>(nev, n);
    double worst = 0.0;
    for (uint32_t i = 0; i < want; ++i) worst = std::max(worst, std::fabs(beta * Z[(size_t)(n - 1) * n + i]));
    double const target =
        rel_floor > 0.0 ? std::max(0.5 * tol_true, rel_floor * std::max(1.0, std::fabs(theta[0]))) : 0.5 * tol_true;
    bool const est_ok = worst <= target;
    bool const last = out.steps >= max_steps;
    if (est_ok || last) {
      // Ritz vectors and true residuals (FP64)
      bool all = true;
      out.theta.assign(want, 0.0);
      out.resid.assign(want, 0.0);
      for (uint32_t i = 0; i < want; ++i) {
        std::vector<double> y(n);
        for (uint32_t q = 0; q < n; ++q) y[q] = Z[(size_t)q * n + i];
        SED_TRY_CUDA(cudaMemcpyAsync(coef.ptr, y.data(), n * 8, cudaMemcpyHostToDevice, stream));
        double* pi = psi + (uint64_t)i * D;
        { k_tritz<S><<<vb, 256, 0, stream>>>(V, D, n, coef.as<double>(), D, pi); note_launches(1); }
        if (int st = operator_apply_device(op, 1, 1, pi, D, w64.ptr, D, stream, SED_FORM_AUTO)) return st;
        ++out.matvecs;
        { k_tresid<<<vb, 256, 0, stream>>>(pi, w64.as<double>(), theta[i], D, part.as<double>()); note_launches(1); }
        SED_TRY_CUDA(cudaMemcpyAsync(hp.data(), part.ptr, 2 * (size_t)vb * 8, cudaMemcpyDeviceToHost, stream));
        SED_TRY_CUDA(cudaStreamSynchronize(stream));
        double rr = 0.0, pp = 0.0;
        for (unsigned b = 0; b < vb; ++b) {
          rr += hp[2 * b];
          pp += hp[2 * b + 1];
        }
        out.theta[i] = theta[i];
        out.resid[i] = std::sqrt(rr / pp);
        if (!(out.resid[i] <= tol_true)) all = false;
      }
      if (all || (rel_floor > 0.0 && est_ok) || last) {
        out.converged = all || (rel_floor > 0.0 && est_ok);
        return LS_SUCCESS;
      }
    }
    if (full) {
      // ---- thick restart: keep the lowest `keep` Ritz vectors, then v_n
      uint32_t const keep = std::min<uint32_t>(n - 1, std::max<uint32_t>(nev + 1, m / 2));
      std::vector<double> Y((size_t)n * keep);
      for (uint32_t q = 0; q < n; ++q)
        for (uint32_t cidx = 0; cidx < keep; ++cidx) Y[(size_t)q * keep + cidx] = Z[(size_t)q * n + cidx];
      SED_TRY_CUDA(cudaMemcpyAsync(Yb.ptr, Y.data(), Y.size() * 8, cudaMemcpyHostToDevice, stream));
      if (int st = rotate_basis<S>(V, D, n, Yb.as<double>(), keep, D, vb, stream, g_rotate_path, rt_err.as<int>()))
        return st;
      if (breakdown) {
        // no continuation vector: a fresh random direction, orthogonalised
        { k_trandom<S><<<vb, 256, 0, stream>>>(V + (uint64_t)keep * D, D, seed + 7919 * (out.restarts + 1)); note_launches(1); }
        for (int pass = 0; pass < 2; ++pass) {
          if (int st = dots(keep, V + (uint64_t)keep * D, c)) return st;
          SED_TRY_CUDA(cudaMemcpyAsync(coef.ptr, c.data(), keep * 8, cudaMemcpyHostToDevice, stream));
          { k_tupdate<S><<<vb, 256, 0, stream>>>(V, D, keep, coef.as<double>(), V + (uint64_t)keep * D, D); note_launches(1); }
        }
        double nn = 0.0;
        if (int st = norm(V + (uint64_t)keep * D, nn)) return st;
        { k_tscale<S><<<vb, 256, 0, stream>>>(V + (uint64_t)keep * D, D, 1.0 / nn, V + (uint64_t)keep * D); note_launches(1); }
      } else {
        SED_TRY_CUDA(cudaMemcpyAsync(V + (uint64_t)keep * D, V + (uint64_t)n * D, D * sizeof(S),
                                     cudaMemcpyDeviceToDevice, stream));
      }
      std::fill(T.begin(), T.end(), 0.0);
      for (uint32_t i = 0; i < keep; ++i) Tij(i, i) = theta[i];
      k = keep;
      arrow = keep;
      ++out.restarts;
      continue;
    }
    k = n;
  }
}

}  // namespace

// sed_eigh's thick-restart path (real operators, 0 < max_basis <= 32).
int solve_thick(OperatorData& op, int out_dtype, sed_eigh_options const& o, double* evals, void* evecs, uint64_t ldv,
                double* rnorms, sed_eigh_info* info) {
  auto t0 = std::chrono::steady_clock::now();
  uint64_t const D = op.basis->D;
  uint32_t const nev = o.nev;
  double const tol = o.tol > 0 ? o.tol : 1e-8;
  uint32_t m = std::min<uint32_t>(o.max_basis, kMaxThick);
  m = (uint32_t)std::min<uint64_t>(m, D);
  if (m < nev + 2 && D > nev + 1) return fail(LS_INVALID_ARGUMENT, "sed_eigh: max_basis must exceed nev + 1");
  cudaStream_t stream = op.cuda_stream;
  auto ts = std::chrono::steady_clock::now();
  int const form = o.form == SED_FORM_AUTO ? op.form : (int)o.form;
  if (form != SED_FORM_ON_THE_FLY) {
    int st = operator_record_stream(op, stream);
    if (st && form == SED_FORM_STREAM) return st;
  }
  int const saved_form = op.form;
  op.form = op.stream.ready && form != SED_FORM_ON_THE_FLY ? SED_FORM_STREAM : SED_FORM_ON_THE_FLY;
  struct FormGuard {
    OperatorData& o;
    int f;
    ~FormGuard() { o.form = f; }
  } form_guard{op, saved_form};
  double const setup = std::chrono::duration<double>(std::chrono::steady_clock::now() - ts).count();
  uint64_t const max_iter = o.max_iter ? o.max_iter : 100000;
  DeviceBuffer psi, start;
  if (int st = psi.allocate((size_t)nev * D * 8)) return st;
  double const* start_ptr = nullptr;
  if (o.start == SED_START_GIVEN && o.start_vectors) {
    if (int st = start.allocate(D * 8)) return st;
    SED_TRY_CUDA(cudaMemcpyAsync(start.ptr, o.start_vectors, D * 8, cudaMemcpyDefault, stream));
    start_ptr = start.as<double>();
  }
  ThickResult r32, r64;
  uint64_t fp32_steps = 0;
  if (o.precision == SED_PRECISION_MIXED) {
    if (op.stream.ready)
      if (int st = operator_prepare_fp32(op, stream)) return st;
    // FP32-stored phase down to the FP32 floor, then FP64 refinement of its
    // Ritz vector with at most 10 stored FP64 vectors
    if (int st = thick_run<float>(op, stream, m, nev, tol, 1e-6, start_ptr, o.seed, max_iter, psi.as<double>(), r32))
      return st;
    fp32_steps = r32.steps;
    uint32_t const mb = std::max<uint32_t>(nev + 2, std::min<uint32_t>(m, 10));
    if (int st = thick_run<double>(op, stream, mb, nev, tol, 0.0, psi.as<double>(), o.seed,
                                   max_iter > r32.steps ? max_iter - r32.steps : 1, psi.as<double>(), r64))
      return st;
  } else {
    if (int st = thick_run<double>(op, stream, m, nev, tol, 0.0, start_ptr, o.seed, max_iter, psi.as<double>(), r64))
      return st;
  }
  // output
  if (evecs) {
    size_t const es = (size_t)elem_bytes_of(out_dtype);
    for (uint32_t i = 0; i < nev; ++i)
      if (int st = store_vector(psi.as<double>() + (uint64_t)i * D, D, out_dtype,
                                static_cast<char*>(evecs) + (size_t)i * ldv * es, stream))
        return st;
  }
  SED_TRY_CUDA(cudaStreamSynchronize(stream));
  for (uint32_t i = 0; i < nev; ++i) {
    if (evals) evals[i] = i < r64.theta.size() ? r64.theta[i] : 0.0;
    if (rnorms) rnorms[i] = i < r64.resid.size() ? r64.resid[i] : 1e300;
  }
  double const total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (info) {
    info->iterations = r32.steps + r64.steps;
    info->matvecs = r32.matvecs + r64.matvecs;
    info->restarts = r32.restarts + r64.restarts;
    info->fp32_iterations = fp32_steps;
    info->seconds_total = total;
    info->seconds_setup = setup;
    info->seconds_solve = total - setup;
  }
  if (logging_enabled())
    log_line("sed_eigh (thick restart, m = %u): E0 = %.15g, residual %.3e, %llu steps (%llu FP32), %llu restarts, %.3f s",
             m, r64.theta.empty() ? 0.0 : r64.theta[0], r64.resid.empty() ? 0.0 : r64.resid[0],
             (unsigned long long)(r32.steps + r64.steps), (unsigned long long)fp32_steps,
             (unsigned long long)(r32.restarts + r64.restarts), total);
  if (!r64.converged)
    return fail(LS_NOT_CONVERGED, "thick restart: residual " +
                                      std::to_string(r64.resid.empty() ? 1e300 : r64.resid[0]) + " above tolerance");
  return LS_SUCCESS;
}

}  // namespace sed

using namespace sed;

extern "C" {

void sed_set_rotate_path(int path) {
  g_rotate_path = (path == SED_ROTATE_FP64 || path == SED_ROTATE_TENSOR) ? path : SED_ROTATE_AUTO;
}

int sed_rotate_vectors(double* V, uint64_t ld, uint32_t m, double const* Y, uint32_t kk, uint64_t D, int path,
                       void* stream) {
  if (!V || !Y || m == 0 || kk == 0 || kk > m || m > (uint32_t)kMaxThick || (D && ld < D))
    return fail(LS_INVALID_ARGUMENT, "sed_rotate_vectors: needs 1 <= kk <= m <= 32, ld >= D and device pointers");
  if (path < SED_ROTATE_AUTO || path > SED_ROTATE_TENSOR) return fail(LS_INVALID_ARGUMENT, "sed_rotate_vectors: bad path");
  if (D == 0) return LS_SUCCESS;
  try {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int dev = 0;
    SED_TRY_CUDA(cudaGetDevice(&dev));
    DeviceBuffer err;
    if (int st = err.allocate(4)) return st;
    if (int st = rotate_basis<double>(V, ld, m, Y, kk, D, grid_size(D, dev, 4), s, path, err.as<int>())) return st;
    SED_TRY_CUDA(cudaStreamSynchronize(s));
    return LS_SUCCESS;
  } catch (std::exception const& e) {
    return fail(LS_SYSTEM_ERROR, e.what());
  }
}

}  // extern "C"
