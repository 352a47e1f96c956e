// lanczos.cu — the device eigensolver behind sed_eigh, replacing the PRIMME
// call at src/SpinED.hs:404 (options at src/SpinED.hs:383-394: smallest
// eigenvalues, tolerance, basis and block sizes, per-iteration monitor).
//
// Single-vector Lanczos with every Krylov vector resident in HBM:
//   w = H v_k (streamed SpMV; its epilogue also yields alpha_k = <v_k, w>)
//   w -= alpha_k v_k + beta_{k-1} v_{k-1}      (+ CGS2 against V when nev > 1)
//   beta_k = ||w||, v_{k+1} = w / beta_k
// The step index lives in device memory, so one CUDA graph holding `check`
// steps is replayed for the whole run. Every `check` steps a one-block kernel
// solves the tridiagonal T_k for its lowest eigenpair(s) on the device
// (Rayleigh-quotient iteration seeded with the previous Ritz vector and
// certified by a division-free positive-definiteness test of T - (theta -
// delta) I; Sturm multisection otherwise) and flags convergence when
// beta_k |s_k| <= tol / 2. The Ritz vector psi = V s is then formed in one
// pass and its true residual ||H psi - E psi|| recomputed in FP64; the run
// restarts from psi until that residual meets the tolerance.
//
// Precision SED_PRECISION_MIXED runs the bulk of the iterations with FP32
// Krylov vectors and FP32 SpMV arithmetic (reductions, alpha/beta, the
// tridiagonal solve stay FP64), then refines the FP32 Ritz vector with the
// FP64 iteration above.
#include <chrono>
#include <cmath>
#include <cstring>

#include "operator_impl.cuh"

namespace sed {
namespace {

constexpr unsigned kMaxNev = 16;
constexpr unsigned kRedThreads = 1024;
constexpr unsigned kVecBlocks = 152 * 8;  // grid of the vector kernels

struct LzHeader {
  uint32_t k;       // newest normalised Krylov vector
  uint32_t stop;    // 0 running, 1 converged, 2 storage full, 3 breakdown
  uint32_t m_max;   // stored vectors
  uint32_t check;   // convergence check period
  uint32_t nev;
  uint32_t size;    // order of T at the last solve
  uint32_t steps;   // Lanczos steps taken
  uint32_t have_s;  // previous Ritz vector of T available
  uint32_t reorth;  // CGS2 against all stored vectors
  uint32_t fallbacks;
  double tol_est;
  double theta[kMaxNev];
  double est[kMaxNev];
};

// ------------------------------------------------------------ vector ops --

template <class X>
__device__ __forceinline__ typename Store<X>::V ld(X const* p, uint64_t i) { return Store<X>::load(p, i); }

template <class X>
__device__ __forceinline__ double norm2(X const* p, uint64_t i) {
  auto const v = Store<X>::load(p, i);
  return dot_re(v, v);
}

// Sums n partials into out (mode 0: alpha[k] = s; mode 1: beta[k] = sqrt(s)).
__global__ void k_reduce(double const* __restrict__ partial, unsigned n, LzHeader* h,
                         double* __restrict__ arr, int mode) {
  __shared__ double red[kRedThreads / 32];
  if (h->stop) return;
  // eight independent sums per thread keep eight loads in flight (the
  // partials of a one-row-per-thread SpMV number D / 256); fixed order
  double a[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  unsigned i = threadIdx.x;
  for (; i + 7 * blockDim.x < n; i += 8 * blockDim.x)
#pragma unroll
    for (unsigned q = 0; q < 8; ++q) a[q] += partial[i + q * blockDim.x];
  for (; i < n; i += blockDim.x) a[0] += partial[i];
  double s = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
  s = block_sum(s, red);
  if (threadIdx.x == 0) {
    uint32_t const k = h->k;
    if (mode == 0) {
      arr[k] += s;  // alpha[k] (zeroed before the SpMV)
    } else {
      arr[k] = sqrt(s);
    }
  }
}

template <class X>
__global__ void k_zero_alpha(LzHeader const* h, double* alpha, unsigned long long* wmax) {
  if (h->stop) return;
  alpha[h->k] = 0.0;
  if (wmax) *wmax = 0;  // fused fixed-point step: k_update's max |w| starts here
}

// Fused fixed-point Lanczos step (FP64, one vector): k_update leaves max |w|
// (bit pattern) in *wmax and k_scale_next writes, next to v_{k+1} = w /
// beta_k, the next matvec's gather copy u = round(sqrt(S) v_{k+1} 2^F) and
// F, so that matvec skips its own pre-pass. `on` is false otherwise.
struct FixStep {
  bool on;
  unsigned long long* wmax;
  int64_t* F;
  int64_t* u;
  uint8_t const* row_class;
  FixView fv;
};

// w = w - alpha_k v_k - beta_{k-1} v_{k-1}; partial ||w||^2.
template <class X>
__global__ void k_update(X* __restrict__ V, uint64_t ld_v, uint64_t D, LzHeader const* h,
                         double const* __restrict__ alpha, double const* __restrict__ beta,
                         double* __restrict__ partial, unsigned long long* __restrict__ wmax) {
  using Vt = typename Store<X>::V;
  __shared__ double red[kBlock / 32];
  __shared__ unsigned long long redm[kBlock / 32];
  if (h->stop) return;
  unsigned long long m = 0;
  uint32_t const k = h->k;
  X* w = V + (uint64_t)(k + 1) * ld_v;
  X const* v = V + (uint64_t)k * ld_v;
  X const* vp = k ? V + (uint64_t)(k - 1) * ld_v : v;
  double const a = alpha[k];
  double const b = k ? beta[k - 1] : 0.0;
  double part = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D;
       i += (uint64_t)gridDim.x * blockDim.x) {
    Vt wi = Store<X>::load(w, i);
    Vt const vi = Store<X>::load(v, i), vpi = Store<X>::load(vp, i);
    if constexpr (std::is_same<Vt, double>::value) {
      wi = fma(-a, vi, fma(-b, vpi, wi));
    } else {
      wi.re = fma(-a, vi.re, fma(-b, vpi.re, wi.re));
      wi.im = fma(-a, vi.im, fma(-b, vpi.im, wi.im));
    }
    Store<X>::store(w, i, wi);
    part += dot_re(wi, wi);
    if constexpr (std::is_same<Vt, double>::value)
      m = max(m, (unsigned long long)__double_as_longlong(wi) & 0x7FFFFFFFFFFFFFFFull);
  }
  double const tot = block_sum(part, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
  if (wmax) {
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) redm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      for (unsigned q = 1; q < kBlock / 32; ++q) m = max(m, redm[q]);
      atomicMax(wmax, m);
    }
  }
}

// Classical Gram-Schmidt pass against V[0..k]: c_j = <V_j, w> (partials per
// block and vector, 16 vectors per blockIdx.y). The vector count NJ of the
// block's group is a template parameter of the loop body, chosen on the
// device from k: a predicated-off FP64 FMA still takes its issue slot on
// GB300's slow FP64 pipe, so the body never pads to 16.
template <int NJ, class X>
__device__ __forceinline__ void cgs_dots_body(X const* __restrict__ V, uint64_t ld_v, uint64_t D, X const* w,
                                              uint32_t j0, double* red, double* __restrict__ partial) {
  double acc[NJ];
#pragma unroll
  for (int j = 0; j < NJ; ++j) acc[j] = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D;
       i += (uint64_t)gridDim.x * blockDim.x) {
    auto const wi = Store<X>::load(w, i);
#pragma unroll
    for (int j = 0; j < NJ; ++j) acc[j] += dot_re(Store<X>::load(V + (uint64_t)(j0 + j) * ld_v, i), wi);
  }
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    double const t = block_sum(acc[j], red);
    if (threadIdx.x == 0) partial[(uint64_t)(j0 + j) * gridDim.x + blockIdx.x] = t;
  }
}

template <class X>
__global__ void k_cgs_dots(X const* __restrict__ V, uint64_t ld_v, uint64_t D, LzHeader const* h,
                           double* __restrict__ partial /* [m_max][gridDim.x] */) {
  __shared__ double red[kBlock / 32];
  if (h->stop) return;
  uint32_t const k = h->k;
  uint32_t const j0 = blockIdx.y * 16;
  if (j0 > k) return;  // uniform per block
  uint32_t const nj = min(16u, k + 1 - j0);
  X const* w = V + (uint64_t)(k + 1) * ld_v;
  switch (nj) {
#define SED_CGS(N) \
  case N: cgs_dots_body<N, X>(V, ld_v, D, w, j0, red, partial); break;
    SED_CGS(1) SED_CGS(2) SED_CGS(3) SED_CGS(4) SED_CGS(5) SED_CGS(6) SED_CGS(7) SED_CGS(8)
    SED_CGS(9) SED_CGS(10) SED_CGS(11) SED_CGS(12) SED_CGS(13) SED_CGS(14) SED_CGS(15) SED_CGS(16)
#undef SED_CGS
  }
}

__global__ void k_cgs_reduce(double const* __restrict__ partial, unsigned nb, LzHeader const* h,
                             double* __restrict__ coef, double* __restrict__ alpha) {
  __shared__ double red[kRedThreads / 32];
  if (h->stop) return;
  uint32_t const k = h->k;
  for (uint32_t j = 0; j <= k; ++j) {
    double s = 0.0;
    for (unsigned i = threadIdx.x; i < nb; i += blockDim.x) s += partial[(uint64_t)j * nb + i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) {
      coef[j] = s;
      if (j == k) alpha[k] += s;  // the projection on v_k corrects alpha_k
    }
  }
}

// w -= sum_j c_j V_j; partial ||w||^2.
template <class X>
__global__ void k_cgs_update(X* __restrict__ V, uint64_t ld_v, uint64_t D, LzHeader const* h,
                             double const* __restrict__ coef, double* __restrict__ partial) {
  using Vt = typename Store<X>::V;
  __shared__ double red[kBlock / 32];
  __shared__ double c[2048];
  if (h->stop) return;
  uint32_t const k = h->k;
  for (uint32_t j = threadIdx.x; j <= k; j += blockDim.x) c[j] = coef[j];
  __syncthreads();
  X* w = V + (uint64_t)(k + 1) * ld_v;
  double part = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D;
       i += (uint64_t)gridDim.x * blockDim.x) {
    Vt wi = Store<X>::load(w, i);
    for (uint32_t j = 0; j <= k; ++j) {
      Vt const vj = Store<X>::load(V + (uint64_t)j * ld_v, i);
      if constexpr (std::is_same<Vt, double>::value) {
        wi = fma(-c[j], vj, wi);
      } else {
        wi.re = fma(-c[j], vj.re, wi.re);
        wi.im = fma(-c[j], vj.im, wi.im);
      }
    }
    Store<X>::store(w, i, wi);
    part += dot_re(wi, wi);
  }
  double const tot = block_sum(part, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

template <class X>
__global__ void k_scale_next(X* __restrict__ V, uint64_t ld_v, uint64_t D, LzHeader const* h,
                             double const* __restrict__ beta, FixStep fx) {
  __shared__ double fac[kFixMaxClasses];
  if (h->stop) return;
  uint32_t const k = h->k;
  double const b = beta[k];
  if (!(b > 0.0)) return;
  double const inv = 1.0 / b;
  X* w = V + (uint64_t)(k + 1) * ld_v;
  if constexpr (std::is_same<X, double>::value) {
    if (fx.on) {
      // max |v_j| = fl(max |w_j| inv): the rounding of v_j = w_j inv is
      // monotone in |w_j|, so this bounds every |v_j| exactly
      double const vmax = __longlong_as_double((long long)*fx.wmax) * inv;
      int64_t const F = fix_exponent((uint64_t)__double_as_longlong(fabs(vmax)), fx.fv.bound);
      if (blockIdx.x == 0 && threadIdx.x == 0) *fx.F = F;
      int64_t const F1 = (F == kFixBad || (F >= -1000 && F <= 1000)) ? 0 : F / 2;
      double const p1 = fix_pow2(F1);
      double const p2 = F == kFixBad ? 0.0 : fix_pow2(F - F1);
      for (uint32_t c = threadIdx.x; c < fx.fv.n_div; c += blockDim.x) fac[c] = fx.fv.sqrt_s[c] * p2;
      __syncthreads();
      for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D;
           i += (uint64_t)gridDim.x * blockDim.x) {
        double const v = inv * w[i];
        w[i] = v;
        fx.u[i] = F == kFixBad ? 0 : fix_round((F1 ? v * p1 : v) * fac[fx.row_class[i]]);
      }
      return;
    }
  }
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D;
       i += (uint64_t)gridDim.x * blockDim.x) {
    auto v = Store<X>::load(w, i);
    Store<X>::store(w, i, mulv(inv, v));
  }
}

// ------------------------------------------------------- tridiagonal ----
// T: diagonal a[0..n), off-diagonal b[0..n-1). All routines run in one thread
// unless stated otherwise; work arrays hold 5 n doubles.

// True iff T - x I is positive definite (all leading minors > 0), computed
// without divisions by the three-term recurrence of the minors with exact
// power-of-two rescaling.
__device__ bool tri_pos_def(double const* a, double const* b, uint32_t n, double x) {
  double p0 = 1.0, p1 = a[0] - x;
  if (!(p1 > 0.0)) return false;
  for (uint32_t i = 1; i < n; ++i) {
    double const p2 = (a[i] - x) * p1 - b[i - 1] * b[i - 1] * p0;
    if (!(p2 > 0.0)) return false;
    p0 = p1;
    p1 = p2;
    if (p1 > 0x1p+400) {
      p0 *= 0x1p-400;
      p1 *= 0x1p-400;
    } else if (p1 < 0x1p-400 && p0 < 0x1p-400) {
      p0 *= 0x1p+400;
      p1 *= 0x1p+400;
    }
  }
  return true;
}

// Number of eigenvalues of T below x (Sturm count of negative pivots).
__device__ uint32_t tri_count(double const* a, double const* b, uint32_t n, double x) {
  uint32_t c = 0;
  double d = a[0] - x;
  if (d < 0.0) ++c;
  for (uint32_t i = 1; i < n; ++i) {
    if (d == 0.0) d = 1e-300;
    d = (a[i] - x) - b[i - 1] * b[i - 1] / d;
    if (d < 0.0) ++c;
  }
  return c;
}

// Solves (T - sigma I) z = r in place (r -> z) by Gaussian elimination with
// partial pivoting on the tridiagonal (the dgttrf/dgtts2 scheme); exactly
// singular pivots are perturbed.
__device__ void tri_solve(double const* a, double const* b, uint32_t n, double sigma, double* r,
                          double* dl, double* d, double* du, double* du2, uint8_t* piv) {
  for (uint32_t i = 0; i < n; ++i) d[i] = a[i] - sigma;
  for (uint32_t i = 0; i + 1 < n; ++i) {
    dl[i] = b[i];
    du[i] = b[i];
  }
  double const tiny = 1e-300;
  for (uint32_t i = 0; i + 1 < n; ++i) {
    if (i + 2 < n) du2[i] = 0.0;
    if (fabs(d[i]) >= fabs(dl[i])) {
      if (d[i] == 0.0) d[i] = tiny;
      double const f = dl[i] / d[i];
      dl[i] = f;
      d[i + 1] -= f * du[i];
      piv[i] = 0;
    } else {
      double const f = d[i] / dl[i];
      d[i] = dl[i];
      dl[i] = f;
      double const t = du[i];
      du[i] = d[i + 1];
      d[i + 1] = t - f * d[i + 1];
      if (i + 2 < n) {
        du2[i] = du[i + 1];
        du[i + 1] = -f * du[i + 1];
      }
      piv[i] = 1;
    }
  }
  if (d[n - 1] == 0.0) d[n - 1] = tiny;
  for (uint32_t i = 0; i + 1 < n; ++i) {
    if (piv[i]) {
      double const t = r[i];
      r[i] = r[i + 1];
      r[i + 1] = t - dl[i] * r[i];
    } else {
      r[i + 1] -= dl[i] * r[i];
    }
  }
  r[n - 1] /= d[n - 1];
  if (n > 1) r[n - 2] = (r[n - 2] - du[n - 2] * r[n - 1]) / d[n - 2];
  for (int i = (int)n - 3; i >= 0; --i) r[i] = (r[i] - du[i] * r[i + 1] - du2[i] * r[i + 2]) / d[i];
}

__device__ double tri_rayleigh(double const* a, double const* b, uint32_t n, double const* s) {
  double num = 0.0, den = 0.0;
  for (uint32_t i = 0; i < n; ++i) {
    double ts = a[i] * s[i];
    if (i) ts += b[i - 1] * s[i - 1];
    if (i + 1 < n) ts += b[i] * s[i + 1];
    num += s[i] * ts;
    den += s[i] * s[i];
  }
  return num / den;
}

__device__ void normalise(double* s, uint32_t n) {
  double m = 0.0;
  for (uint32_t i = 0; i < n; ++i) m += s[i] * s[i];
  double const inv = 1.0 / sqrt(m);
  for (uint32_t i = 0; i < n; ++i) s[i] *= inv;
}

// One block: lowest nev eigenpairs of T_n (n = k + 1) every `check` steps,
// convergence flags, then k += 1.
__global__ void k_tridiag(LzHeader* h, double const* __restrict__ alpha,
                          double const* __restrict__ beta, double* __restrict__ S /* [nev][m_max] */,
                          double* __restrict__ work) {
  __shared__ double lohi[2];
  __shared__ uint32_t sh_flag;
  __shared__ double bounds[2];
  if (h->stop) return;
  uint32_t const k = h->k;
  uint32_t const n = k + 1;
  uint32_t const m_max = h->m_max;
  double const bk = beta[k];
  bool const full = k + 2 >= m_max;
  double anorm = 0.0;
  bool const breakdown = !(bk > 0.0) || !isfinite(bk);
  bool const do_check = ((n % h->check) == 0) || full || breakdown;
  if (!do_check) {
    __syncthreads();
    if (threadIdx.x == 0) {
      h->steps += 1;
      h->k = k + 1;
    }
    return;
  }
  uint32_t const nev = min(h->nev, n);
  double* dl = work;
  double* d = work + m_max;
  double* du = work + 2 * m_max;
  double* du2 = work + 3 * m_max;
  uint8_t* piv = reinterpret_cast<uint8_t*>(work + 4 * m_max);
  // Gershgorin bounds.
  if (threadIdx.x == 0) {
    double lo = 1e300, hi = -1e300;
    for (uint32_t i = 0; i < n; ++i) {
      double r = (i ? fabs(beta[i - 1]) : 0.0) + (i + 1 < n ? fabs(beta[i]) : 0.0);
      lo = fmin(lo, alpha[i] - r);
      hi = fmax(hi, alpha[i] + r);
    }
    bounds[0] = lo;
    bounds[1] = hi;
  }
  __syncthreads();
  anorm = fmax(fabs(bounds[0]), fabs(bounds[1]));
  bool all_ok = true;
  for (uint32_t j = 0; j < nev; ++j) {
    double* s = S + (uint64_t)j * m_max;
    // Fast path (nev == 1): Rayleigh-quotient iteration from the previous
    // Ritz vector, certified by a positive-definiteness test.
    if (threadIdx.x == 0) sh_flag = 0;
    __syncthreads();
    if (nev == 1 && h->have_s && threadIdx.x == 0) {
      uint32_t const prev = h->size;
      for (uint32_t i = prev; i < n; ++i) s[i] = 0.0;
      normalise(s, n);
      double sigma = tri_rayleigh(alpha, beta, n, s);
      for (int it = 0; it < 3; ++it) {
        tri_solve(alpha, beta, n, sigma, s, dl, d, du, du2, piv);
        normalise(s, n);
        double const ns = tri_rayleigh(alpha, beta, n, s);
        bool const done = fabs(ns - sigma) <= 1e-15 * fmax(1.0, fabs(ns));
        sigma = ns;
        if (done) break;
      }
      double const delta = 1e-12 * fmax(1.0, anorm);
      if (tri_pos_def(alpha, beta, n, sigma - delta)) {
        h->theta[0] = sigma;
        sh_flag = 1;
      }
    }
    __syncthreads();
    if (!sh_flag) {
      // Sturm multisection for the j-th eigenvalue, all threads.
      if (threadIdx.x == 0) {
        lohi[0] = bounds[0] - 1e-12 * fmax(1.0, anorm);
        lohi[1] = bounds[1] + 1e-12 * fmax(1.0, anorm);
      }
      __syncthreads();
      for (int round = 0; round < 24; ++round) {
        double const lo = lohi[0], hi = lohi[1];
        if (hi - lo <= 2e-16 * fmax(fabs(lo), fabs(hi)) + 1e-300) break;
        double const x = lo + (hi - lo) * (double)(threadIdx.x + 1) / (double)(blockDim.x + 1);
        bool const above = tri_count(alpha, beta, n, x) > j;  // x above eigenvalue j
        unsigned const ballot = __ballot_sync(0xffffffffu, above);
        __syncthreads();
        if (threadIdx.x == 0) {
          int const first = ballot ? __ffs(ballot) - 1 : (int)blockDim.x;
          double const nlo = first == 0 ? lo : lo + (hi - lo) * (double)first / (double)(blockDim.x + 1);
          double const nhi = first == (int)blockDim.x ? hi : lo + (hi - lo) * (double)(first + 1) / (double)(blockDim.x + 1);
          lohi[0] = nlo;
          lohi[1] = nhi;
        }
        __syncthreads();
      }
      if (threadIdx.x == 0) {
        double const theta = 0.5 * (lohi[0] + lohi[1]);
        // Inverse iteration, orthogonalised against lower pairs.
        for (uint32_t i = 0; i < n; ++i) s[i] = 1.0 + 1e-3 * (double)((i * 7919u + j * 104729u) % 1000u) / 1000.0;
        for (int it = 0; it < 3; ++it) {
          for (uint32_t q = 0; q < j; ++q) {
            double const* sq = S + (uint64_t)q * m_max;
            double dp = 0.0;
            for (uint32_t i = 0; i < n; ++i) dp += sq[i] * s[i];
            for (uint32_t i = 0; i < n; ++i) s[i] -= dp * sq[i];
          }
          normalise(s, n);
          tri_solve(alpha, beta, n, theta, s, dl, d, du, du2, piv);
          normalise(s, n);
        }
        h->theta[j] = tri_rayleigh(alpha, beta, n, s);
        h->fallbacks += 1;
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      double const est = fabs(bk * s[n - 1]);
      h->est[j] = breakdown ? 0.0 : est;
      if (!(h->est[j] <= h->tol_est)) all_ok = false;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    h->size = n;
    h->have_s = 1;
    h->steps += 1;
    if (breakdown)
      h->stop = 3;
    else if (nev == h->nev && all_ok)
      h->stop = 1;
    else if (full)
      h->stop = 2;
    else
      h->k = k + 1;
  }
}

// out_i = sum_{j < n} s_j V_j[i]
template <class X, class Y>
__global__ void k_ritz(X const* __restrict__ V, uint64_t ld_v, uint64_t D, double const* __restrict__ s,
                       uint32_t n, Y* __restrict__ out) {
  __shared__ double c[2048];
  for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) c[j] = s[j];
  __syncthreads();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D;
       i += (uint64_t)gridDim.x * blockDim.x) {
    typename Store<Y>::V acc = zero<typename Store<Y>::V>();
    for (uint32_t j = 0; j < n; ++j) {
      auto const v = Store<X>::load(V + (uint64_t)j * ld_v, i);
      if constexpr (std::is_same<typename Store<Y>::V, double>::value) {
        acc = fma(c[j], v, acc);
      } else {
        acc.re = fma(c[j], v.re, acc.re);
        acc.im = fma(c[j], v.im, acc.im);
      }
    }
    Store<Y>::store(out, i, acc);
  }
}

// partial dots for <x,x>, <x,y> and ||y - e x||^2 (mode 0: first two; 1: last)
template <class X>
__global__ void k_dots(X const* __restrict__ x, X const* __restrict__ y, uint64_t D, double e,
                       int mode, double* __restrict__ partial) {
  __shared__ double red[kBlock / 32];
  double p0 = 0.0, p1 = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D;
       i += (uint64_t)gridDim.x * blockDim.x) {
    auto const xi = Store<X>::load(x, i);
    auto const yi = Store<X>::load(y, i);
    if (mode == 0) {
      p0 += dot_re(xi, xi);
      p1 += dot_re(xi, yi);
    } else {
      auto const r = addv(yi, mulv(-e, xi));
      p0 += dot_re(r, r);
    }
  }
  double const t0 = block_sum(p0, red);
  double const t1 = block_sum(p1, red);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = t0;
    partial[2 * blockIdx.x + 1] = t1;
  }
}

template <class X>
__global__ void k_scale(X* __restrict__ x, uint64_t D, double f) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D;
       i += (uint64_t)gridDim.x * blockDim.x)
    Store<X>::store(x, i, mulv(f, Store<X>::load(x, i)));
}

template <class X, class Y>
__global__ void k_convert(X const* __restrict__ x, uint64_t D, Y* __restrict__ y) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D;
       i += (uint64_t)gridDim.x * blockDim.x) {
    auto const v = Store<X>::load(x, i);
    if constexpr (std::is_same<decltype(v), typename Store<Y>::V const>::value) {
      Store<Y>::store(y, i, v);
    } else if constexpr (std::is_same<typename Store<Y>::V, cplx>::value) {
      Store<Y>::store(y, i, cplx{(double)v, 0.0});
    } else {
      Store<Y>::store(y, i, v.re);
    }
  }
}

// Element i of the start vector is uniform in [-1, 1) from Philox block i/2.
template <class X>
__global__ void k_random(X* __restrict__ x, uint64_t D, uint64_t seed) {
  for (uint64_t blk = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; blk < (D + 1) / 2;
       blk += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t c[4] = {(uint32_t)blk, (uint32_t)(blk >> 32), 0u, 0u};
    philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    double const v0 = 2.0 * u01_53(c[0], c[1]) - 1.0;
    double const v1 = 2.0 * u01_53(c[2], c[3]) - 1.0;
    if constexpr (std::is_same<typename Store<X>::V, double>::value) {
      Store<X>::store(x, 2 * blk, v0);
      if (2 * blk + 1 < D) Store<X>::store(x, 2 * blk + 1, v1);
    } else {
      Store<X>::store(x, 2 * blk, cplx{v0, 0.0});
      if (2 * blk + 1 < D) Store<X>::store(x, 2 * blk + 1, cplx{v1, 0.0});
    }
  }
}

// ------------------------------------------------------------- driver ----

struct Workspace {
  DeviceBuffer V, header, alpha, beta, s, work, partial, cgs_partial, coef, ritz, y, scratch;
};

int elem_bytes(int dtype) { return dtype == 0 ? 4 : dtype == 1 ? 8 : dtype == 2 ? 8 : 16; }

template <class X>
double host_sum(DeviceBuffer const& partial, unsigned n, unsigned stride, unsigned off, cudaStream_t s,
                int* st) {
  std::vector<double> h((size_t)n * stride);
  cudaError_t e = cudaMemcpyAsync(h.data(), partial.ptr, h.size() * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    *st = fail(LS_CUDA_ERROR, std::string("reading partial sums: ") + cudaGetErrorString(e));
    return 0.0;
  }
  double t = 0.0;
  for (unsigned i = 0; i < n; ++i) t += h[(size_t)i * stride + off];
  return t;
}

template <class X>
struct Solver {
  OperatorData& op;
  int dtype;  // storage dtype of X
  uint64_t D;
  cudaStream_t stream;
  Workspace ws;
  uint32_t m_max = 0;
  unsigned spmv_blocks = 0;
  unsigned vblocks = 0;
  cudaGraphExec_t graph = nullptr;
  size_t graph_kernels = 0;
  LzHeader* hh = nullptr;  // pinned host mirror
  FixStep fx{};            // fused fixed-point step (FP64, one vector, stream form)

  Solver(OperatorData& o, int dt, cudaStream_t s) : op(o), dtype(dt), D(o.basis->D), stream(s) {}
  ~Solver() {
    if (graph) cudaGraphExecDestroy(graph);
    if (hh) cudaFreeHost(hh);
    krylov_give(ws.V);
  }

  X* V() const { return ws.V.as<X>(); }
  LzHeader* hdr() const { return ws.header.as<LzHeader>(); }

  int init(uint32_t m, uint32_t nev, uint32_t check, double tol_est, bool reorth) {
    m_max = m;
    int dev = op.basis->device;
    vblocks = grid_size(D, dev, 8);
    if (int st = krylov_take((size_t)m_max * D * sizeof(X), ws.V)) return st;
    if (int st = ws.header.allocate(sizeof(LzHeader))) return st;
    if (int st = ws.alpha.allocate((size_t)m_max * 8)) return st;
    if (int st = ws.beta.allocate((size_t)m_max * 8)) return st;
    if (int st = ws.s.allocate((size_t)kMaxNev * m_max * 8)) return st;
    if (int st = ws.work.allocate((size_t)5 * m_max * 8 + 64)) return st;
    uint64_t const nb = std::max<uint64_t>((D + kBlock - 1) / kBlock + 64, vblocks);
    if (int st = ws.partial.allocate(nb * 16)) return st;
    if (reorth) {
      if (int st = ws.cgs_partial.allocate((size_t)m_max * vblocks * 8)) return st;
      if (int st = ws.coef.allocate((size_t)m_max * 8)) return st;
    }
    if (int st = ws.ritz.allocate(D * sizeof(X))) return st;
    if (int st = ws.y.allocate(D * sizeof(X))) return st;
    SED_TRY_CUDA(cudaMallocHost(&hh, sizeof(LzHeader)));
    std::memset(hh, 0, sizeof(LzHeader));
    hh->m_max = m_max;
    hh->check = check;
    hh->nev = nev;
    hh->tol_est = tol_est;
    hh->reorth = reorth ? 1u : 0u;
    SED_TRY_CUDA(cudaMemcpyAsync(hdr(), hh, sizeof(LzHeader), cudaMemcpyHostToDevice, stream));
    SED_TRY_CUDA(cudaMemsetAsync(ws.alpha.ptr, 0, (size_t)m_max * 8, stream));
    SED_TRY_CUDA(cudaMemsetAsync(ws.beta.ptr, 0, (size_t)m_max * 8, stream));
    FixSlots fs;
    if (std::is_same<X, double>::value && !reorth && fix_slots(op, &fs))
      fx = FixStep{true, fs.max_bits, fs.F, fs.u, fs.row_class, fs.view};
    return LS_SUCCESS;
  }

  // Fused step: the matvec's pre-pass for the current v_k, needed whenever
  // v_k was not produced by k_scale_next (the start and every restart) or
  // the workspace was used by another matvec since.
  int prescale() {
    if (!fx.on) return LS_SUCCESS;
    Indirect ind;
    ind.k = &hdr()->k;
    ind.stop = &hdr()->stop;
    ind.ld = D;
    return fix_prescale(op, reinterpret_cast<double const*>(V()), ind, stream);
  }

  // One Lanczos step (all kernels read k from the header).
  int enqueue_step() {
    LzHeader* h = hdr();
    { k_zero_alpha<X><<<1, 1, 0, stream>>>(h, ws.alpha.as<double>(), fx.on ? fx.wmax : nullptr); note_launches(1); }
    Indirect ind;
    ind.k = &h->k;
    ind.stop = &h->stop;
    ind.ld = D;
    ind.partial = ws.partial.as<double>();
    ind.prescaled = fx.on;
    if (int st = operator_apply_krylov(op, dtype, V(), ind, stream, &spmv_blocks)) return st;
    { k_reduce<<<1, kRedThreads, 0, stream>>>(ws.partial.as<double>(), spmv_blocks, h, ws.alpha.as<double>(), 0); note_launches(1); }
    { k_update<X><<<vblocks, kBlock, 0, stream>>>(V(), D, D, h, ws.alpha.as<double>(), ws.beta.as<double>(),
                                                ws.partial.as<double>(), fx.on ? fx.wmax : nullptr); note_launches(1); }
    if (hh->reorth) {
      for (int pass = 0; pass < 2; ++pass) {
        dim3 grid(vblocks, (m_max + 15) / 16);
        { k_cgs_dots<X><<<grid, kBlock, 0, stream>>>(V(), D, D, h, ws.cgs_partial.as<double>()); note_launches(1); }
        { k_cgs_reduce<<<1, kRedThreads, 0, stream>>>(ws.cgs_partial.as<double>(), vblocks, h,
                                                    ws.coef.as<double>(), ws.alpha.as<double>()); note_launches(1); }
        { k_cgs_update<X><<<vblocks, kBlock, 0, stream>>>(V(), D, D, h, ws.coef.as<double>(),
                                                        ws.partial.as<double>()); note_launches(1); }
      }
    }
    { k_reduce<<<1, kRedThreads, 0, stream>>>(ws.partial.as<double>(), vblocks, h, ws.beta.as<double>(), 1); note_launches(1); }
    { k_scale_next<X><<<vblocks, kBlock, 0, stream>>>(V(), D, D, h, ws.beta.as<double>(), fx); note_launches(1); }
    { k_tridiag<<<1, 32, 0, stream>>>(h, ws.alpha.as<double>(), ws.beta.as<double>(), ws.s.as<double>(),
                                    ws.work.as<double>()); note_launches(1); }
    SED_TRY_CUDA(cudaGetLastError());
    return LS_SUCCESS;
  }

  int capture(uint32_t steps) {
    cudaGraph_t g;
    SED_TRY_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    set_capturing(true);
    int st = LS_SUCCESS;
    for (uint32_t i = 0; i < steps && st == LS_SUCCESS; ++i) st = enqueue_step();
    set_capturing(false);
    cudaError_t e = cudaStreamEndCapture(stream, &g);
    if (st) {
      if (e == cudaSuccess) cudaGraphDestroy(g);
      return st;
    }
    SED_TRY_CUDA(e);
    size_t n_nodes = 0;
    cudaGraphGetNodes(g, nullptr, &n_nodes);
    graph_kernels = n_nodes;
    e = cudaGraphInstantiate(&graph, g, 0);
    cudaGraphDestroy(g);
    SED_TRY_CUDA(e);
    return LS_SUCCESS;
  }

  int read_header() {
    SED_TRY_CUDA(cudaMemcpyAsync(hh, hdr(), sizeof(LzHeader), cudaMemcpyDeviceToHost, stream));
    SED_TRY_CUDA(cudaStreamSynchronize(stream));
    return LS_SUCCESS;
  }

  int write_header() {
    SED_TRY_CUDA(cudaMemcpyAsync(hdr(), hh, sizeof(LzHeader), cudaMemcpyHostToDevice, stream));
    return LS_SUCCESS;
  }

  // Writes x (device, type X) to dst (host or device) as `out_dtype`.
  int store(X const* x, int out_dtype, void* dst) {
    int const own = std::is_same<X, double>::value ? 1 : 3;
    if (out_dtype == own) {
      SED_TRY_CUDA(cudaMemcpyAsync(dst, x, D * sizeof(X), cudaMemcpyDefault, stream));
      SED_TRY_CUDA(cudaStreamSynchronize(stream));
      return LS_SUCCESS;
    }
    size_t const es = (size_t)elem_bytes(out_dtype);
    if (!ws.scratch.ptr || ws.scratch.bytes < D * es)
      if (int st = ws.scratch.allocate(D * es)) return st;
    switch (out_dtype) {
      case 0: { k_convert<X, float><<<vblocks, kBlock, 0, stream>>>(x, D, ws.scratch.as<float>()); note_launches(1); } break;
      case 1: { k_convert<X, double><<<vblocks, kBlock, 0, stream>>>(x, D, ws.scratch.as<double>()); note_launches(1); } break;
      case 2: { k_convert<X, float2><<<vblocks, kBlock, 0, stream>>>(x, D, ws.scratch.as<float2>()); note_launches(1); } break;
      default: { k_convert<X, double2><<<vblocks, kBlock, 0, stream>>>(x, D, ws.scratch.as<double2>()); note_launches(1); } break;
    }
    SED_TRY_CUDA(cudaGetLastError());
    SED_TRY_CUDA(cudaMemcpyAsync(dst, ws.scratch.ptr, D * es, cudaMemcpyDefault, stream));
    SED_TRY_CUDA(cudaStreamSynchronize(stream));
    return LS_SUCCESS;
  }

  // ||x||, normalises x in place.
  int normalise_vec(X* x, double* out_norm) {
    { k_dots<X><<<vblocks, kBlock, 0, stream>>>(x, x, D, 0.0, 0, ws.partial.as<double>()); note_launches(1); }
    SED_TRY_CUDA(cudaGetLastError());
    int st = LS_SUCCESS;
    double const n2 = host_sum<X>(ws.partial, vblocks, 2, 0, stream, &st);
    if (st) return st;
    double const nrm = std::sqrt(n2);
    if (!(nrm > 0.0)) return fail(LS_INVALID_ARGUMENT, "start vector is zero");
    { k_scale<X><<<vblocks, kBlock, 0, stream>>>(x, D, 1.0 / nrm); note_launches(1); }
    SED_TRY_CUDA(cudaGetLastError());
    if (out_norm) *out_norm = nrm;
    return LS_SUCCESS;
  }

  // y = H x with residual: returns E = <x,Hx>/<x,x> and ||Hx - E x||/||x||.
  int residual(X* x, double* E, double* r) {
    if (int st = operator_apply_device(op, dtype, 1, x, D, ws.y.ptr, D, stream, SED_FORM_AUTO)) return st;
    { k_dots<X><<<vblocks, kBlock, 0, stream>>>(x, ws.y.as<X>(), D, 0.0, 0, ws.partial.as<double>()); note_launches(1); }
    int st = LS_SUCCESS;
    std::vector<double> h(2 * (size_t)vblocks);
    SED_TRY_CUDA(cudaMemcpyAsync(h.data(), ws.partial.ptr, h.size() * 8, cudaMemcpyDeviceToHost, stream));
    SED_TRY_CUDA(cudaStreamSynchronize(stream));
    double xx = 0.0, xy = 0.0;
    for (unsigned i = 0; i < vblocks; ++i) {
      xx += h[2 * i];
      xy += h[2 * i + 1];
    }
    *E = xy / xx;
    { k_dots<X><<<vblocks, kBlock, 0, stream>>>(x, ws.y.as<X>(), D, *E, 1, ws.partial.as<double>()); note_launches(1); }
    double const rr = host_sum<X>(ws.partial, vblocks, 2, 0, stream, &st);
    if (st) return st;
    *r = std::sqrt(rr / xx);
    return LS_SUCCESS;
  }
};

// ------------------------------------------------- mixed precision ----
// FP32 Lanczos steps: vectors and their updates in FP32, reductions per warp
// in FP32 and per block in FP64.
__global__ void k_update32(float* __restrict__ V, uint64_t ld_v, uint64_t D, LzHeader const* h,
                           double const* __restrict__ alpha, double const* __restrict__ beta,
                           double* __restrict__ partial) {
  __shared__ double red[kBlock / 32];
  if (h->stop) return;
  uint32_t const k = h->k;
  float* w = V + (uint64_t)(k + 1) * ld_v;
  float const* v = V + (uint64_t)k * ld_v;
  float const* vp = k ? V + (uint64_t)(k - 1) * ld_v : v;
  float const a = (float)alpha[k];
  float const b = k ? (float)beta[k - 1] : 0.0f;
  float part = 0.0f;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D;
       i += (uint64_t)gridDim.x * blockDim.x) {
    float const wi = fmaf(-a, v[i], fmaf(-b, vp[i], w[i]));
    w[i] = wi;
    part = fmaf(wi, wi, part);
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  double const tot = block_sum((threadIdx.x & 31) == 0 ? (double)part : 0.0, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

__global__ void k_scale_next32(float* __restrict__ V, uint64_t ld_v, uint64_t D, LzHeader const* h,
                               double const* __restrict__ beta) {
  if (h->stop) return;
  uint32_t const k = h->k;
  double const b = beta[k];
  if (!(b > 0.0)) return;
  float const inv = (float)(1.0 / b);
  float* w = V + (uint64_t)(k + 1) * ld_v;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D;
       i += (uint64_t)gridDim.x * blockDim.x)
    w[i] *= inv;
}

// out = s_0 psi + sum_{j=1}^{n-1} s_j V_j, accumulated in FP64.
__global__ void k_ritz_mixed(double const* __restrict__ psi, float const* __restrict__ V, uint64_t ld_v,
                             uint64_t D, double const* __restrict__ s, uint32_t n, double* __restrict__ out) {
  __shared__ double c[2048];
  for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) c[j] = s[j];
  __syncthreads();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D;
       i += (uint64_t)gridDim.x * blockDim.x) {
    double acc = c[0] * psi[i];
    for (uint32_t j = 1; j < n; ++j) acc = fma(c[j], (double)V[(uint64_t)j * ld_v + i], acc);
    out[i] = acc;
  }
}

// v0 = (float) psi, v1 = (float) ((y - theta psi) / rn)
__global__ void k_start_cycle(double const* __restrict__ psi, double const* __restrict__ y, uint64_t D,
                              double theta, double inv_rn, float* __restrict__ v0, float* __restrict__ v1) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D;
       i += (uint64_t)gridDim.x * blockDim.x) {
    double const p = psi[i];
    v0[i] = (float)p;
    v1[i] = (float)((y[i] - theta * p) * inv_rn);
  }
}

uint32_t auto_basis(uint64_t D, size_t elem, uint32_t nev, uint32_t requested) {
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  uint64_t const cap_mem = (uint64_t)(0.6 * (double)free_b) / std::max<uint64_t>(1, D * elem);
  uint64_t m = requested ? requested : 400;
  m = std::min<uint64_t>(m, cap_mem);
  m = std::min<uint64_t>(m, D + 1);
  m = std::min<uint64_t>(m, 2048);
  m = std::max<uint64_t>(m, std::min<uint64_t>(D + 1, nev + 2));
  return (uint32_t)m;
}

template <class X>
int solve(OperatorData& op, int out_dtype, sed_eigh_options const& o, double* evals, void* evecs,
          uint64_t ldv, double* rnorms, sed_eigh_info* info) {
  int const dtype = std::is_same<X, double>::value ? 1 : 3;
  auto t0 = std::chrono::steady_clock::now();
  BasisData& b = *op.basis;
  uint64_t const D = b.D;
  uint32_t const nev = o.nev;
  cudaStream_t stream = op.cuda_stream;
  double const tol = o.tol > 0 ? o.tol : 1e-8;
  uint64_t const max_iter = o.max_iter ? o.max_iter : 100000;
  // Stream form when it fits.
  auto ts = std::chrono::steady_clock::now();
  int const form = o.form == SED_FORM_AUTO ? op.form : (int)o.form;
  if (form != SED_FORM_ON_THE_FLY) {
    int st = operator_record_stream(op, stream);
    if (st && form == SED_FORM_STREAM) return st;
  }
  int const saved_form = op.form;
  op.form = form;
  struct FormGuard {
    OperatorData& o;
    int f;
    ~FormGuard() { o.form = f; }
  } form_guard{op, saved_form};
  double const setup = std::chrono::duration<double>(std::chrono::steady_clock::now() - ts).count();
  bool const reorth = nev > 1;
  uint32_t const m = auto_basis(D, sizeof(X), nev, o.max_basis);
  uint32_t const check = m < 64 ? 1u : 4u;
  Solver<X> S(op, dtype, stream);
  if (int st = S.init(m, nev, check, 0.5 * tol, reorth)) return st;
  // Start vector.
  if (o.start == SED_START_GIVEN && o.start_vectors) {
    size_t const es = sizeof(X);
    SED_TRY_CUDA(cudaMemcpyAsync(S.V(), o.start_vectors, D * es, cudaMemcpyDefault, stream));
  } else {
    { k_random<X><<<S.vblocks, kBlock, 0, stream>>>(S.V(), D, o.seed); note_launches(1); }
    SED_TRY_CUDA(cudaGetLastError());
  }
  if (int st = S.normalise_vec(S.V(), nullptr)) return st;
  if (int st = S.capture(check)) return st;
  if (int st = S.prescale()) return st;
  uint64_t steps = 0, matvecs = 0, restarts = 0;
  std::vector<double> E(nev, 0.0), R(nev, 1e300);
  bool converged = false;
  std::vector<double> theta_h(nev), est_h(nev);
  while (!converged) {
    SED_TRY_CUDA(cudaGraphLaunch(S.graph, stream));
    note_launches(S.graph_kernels);
    if (int st = S.read_header()) return st;
    if (o.progress) {
      for (uint32_t j = 0; j < nev; ++j) {
        theta_h[j] = S.hh->theta[j];
        est_h[j] = S.hh->est[j];
      }
      o.progress(o.progress_user, steps + S.hh->steps, theta_h.data(), est_h.data(), nev);
    }
    uint32_t const stop = S.hh->stop;
    if (!stop) {
      if (steps + S.hh->steps >= max_iter) break;
      continue;
    }
    steps += S.hh->steps;
    matvecs += S.hh->steps;
    uint32_t const n = S.hh->size;
    // Ritz vectors and their true residuals.
    bool all_ok = true;
    for (uint32_t j = 0; j < nev; ++j) {
      { k_ritz<X, X><<<S.vblocks, kBlock, 0, stream>>>(S.V(), D, D, S.ws.s.template as<double>() + (uint64_t)j * m,
                                                     n, S.ws.ritz.template as<X>()); note_launches(1); }
      SED_TRY_CUDA(cudaGetLastError());
      if (int st = S.normalise_vec(S.ws.ritz.template as<X>(), nullptr)) return st;
      double e = 0.0, r = 0.0;
      if (int st = S.residual(S.ws.ritz.template as<X>(), &e, &r)) return st;
      ++matvecs;
      E[j] = e;
      R[j] = r;
      if (!(r <= tol)) all_ok = false;
      if (evecs)
        if (int st = S.store(S.ws.ritz.template as<X>(), out_dtype, static_cast<char*>(evecs) +
                             (size_t)j * ldv * elem_bytes(out_dtype))) return st;
    }
    if (all_ok || stop == 3 || steps >= max_iter) {
      converged = all_ok || stop == 3;
      break;
    }
    // Restart from the (sum of the) Ritz vectors.
    ++restarts;
    if (nev == 1) {
      SED_TRY_CUDA(cudaMemcpyAsync(S.V(), S.ws.ritz.ptr, D * sizeof(X), cudaMemcpyDeviceToDevice, stream));
    } else {
      { k_ritz<X, X><<<S.vblocks, kBlock, 0, stream>>>(S.V(), D, D, S.ws.s.template as<double>(), n, S.ws.ritz.template as<X>()); note_launches(1); }
      // sum of all nev Ritz directions
      std::vector<double> ones(n, 0.0);
      std::vector<double> sh((size_t)nev * m);
      SED_TRY_CUDA(cudaMemcpy(sh.data(), S.ws.s.ptr, sh.size() * 8, cudaMemcpyDeviceToHost));
      for (uint32_t j = 0; j < nev; ++j)
        for (uint32_t i = 0; i < n; ++i) ones[i] += sh[(size_t)j * m + i];
      SED_TRY_CUDA(cudaMemcpy(S.ws.work.ptr, ones.data(), n * 8, cudaMemcpyHostToDevice));
      { k_ritz<X, X><<<S.vblocks, kBlock, 0, stream>>>(S.V(), D, D, S.ws.work.template as<double>(), n,
                                                     S.ws.ritz.template as<X>()); note_launches(1); }
      SED_TRY_CUDA(cudaMemcpyAsync(S.V(), S.ws.ritz.ptr, D * sizeof(X), cudaMemcpyDeviceToDevice, stream));
    }
    if (int st = S.normalise_vec(S.V(), nullptr)) return st;
    uint32_t const keep_nev = S.hh->nev;
    std::memset(S.hh, 0, sizeof(LzHeader));
    S.hh->m_max = m;
    S.hh->check = check;
    S.hh->nev = keep_nev;
    S.hh->tol_est = 0.5 * tol;
    S.hh->reorth = reorth ? 1u : 0u;
    if (int st = S.write_header()) return st;
    if (int st = S.prescale()) return st;  // the residual matvecs used the workspace
  }
  SED_TRY_CUDA(cudaStreamSynchronize(stream));
  for (uint32_t j = 0; j < nev; ++j) {
    if (evals) evals[j] = E[j];
    if (rnorms) rnorms[j] = R[j];
  }
  double const total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (info) {
    info->iterations = steps;
    info->matvecs = matvecs;
    info->restarts = restarts;
    info->fp32_iterations = 0;
    info->seconds_total = total;
    info->seconds_setup = setup;
    info->seconds_solve = total - setup;
  }
  if (logging_enabled())
    log_line("sed_eigh: E0 = %.15g, residual %.3e, %llu steps, %llu restarts, %.3f s", E[0], R[0],
             (unsigned long long)steps, (unsigned long long)restarts, total);
  if (!converged) return fail(LS_NOT_CONVERGED, "residual " + std::to_string(R[0]) + " above tolerance after " +
                                                   std::to_string(steps) + " steps");
  return LS_SUCCESS;
}

// Mixed precision: FP64 anchor psi, FP32 Krylov cycles (see the file head).
int solve_mixed(OperatorData& op, int out_dtype, sed_eigh_options const& o, double* evals, void* evecs,
                uint64_t ldv, double* rnorms, sed_eigh_info* info) {
  auto t0 = std::chrono::steady_clock::now();
  uint64_t const D = op.basis->D;
  cudaStream_t stream = op.cuda_stream;
  double const tol = o.tol > 0 ? o.tol : 1e-8;
  uint64_t const max_iter = o.max_iter ? o.max_iter : 100000;
  auto ts = std::chrono::steady_clock::now();
  if (int st = operator_record_stream(op, stream)) return st;
  if (int st = operator_prepare_fp32(op, stream)) return st;
  double const setup = std::chrono::duration<double>(std::chrono::steady_clock::now() - ts).count();
  int const saved_form = op.form;
  op.form = SED_FORM_STREAM;
  struct FormGuard {
    OperatorData& o;
    int f;
    ~FormGuard() { o.form = f; }
  } form_guard{op, saved_form};
  uint32_t const m = std::max<uint32_t>(3, auto_basis(D, 4, 1, o.max_basis ? o.max_basis : 300));
  uint32_t const check = m < 64 ? 1u : 4u;
  unsigned const vb = grid_size(D, op.basis->device, 8);
  DeviceBuffer psi, y, V, hdr_b, alpha, beta, sbuf, work, partial;
  if (int st = psi.allocate(D * 8)) return st;
  if (int st = y.allocate(D * 8)) return st;
  struct KrylovGuard {
    DeviceBuffer& b;
    ~KrylovGuard() { krylov_give(b); }
  } krylov_guard{V};
  if (int st = krylov_take((size_t)m * D * 4, V)) return st;
  if (int st = hdr_b.allocate(sizeof(LzHeader))) return st;
  if (int st = alpha.allocate((size_t)m * 8)) return st;
  if (int st = beta.allocate((size_t)m * 8)) return st;
  if (int st = sbuf.allocate((size_t)kMaxNev * m * 8)) return st;
  if (int st = work.allocate((size_t)5 * m * 8 + 64)) return st;
  uint64_t const nb = std::max<uint64_t>((D + kBlock - 1) / kBlock + 64, vb);
  if (int st = partial.allocate(nb * 16)) return st;
  LzHeader* hh = nullptr;
  SED_TRY_CUDA(cudaMallocHost(&hh, sizeof(LzHeader)));
  struct HostGuard {
    LzHeader* p;
    ~HostGuard() { cudaFreeHost(p); }
  } host_guard{hh};
  LzHeader* h = hdr_b.as<LzHeader>();
  float* Vf = V.as<float>();
  // FP64 start vector
  if (o.start == SED_START_GIVEN && o.start_vectors)
    SED_TRY_CUDA(cudaMemcpyAsync(psi.ptr, o.start_vectors, D * 8, cudaMemcpyDefault, stream));
  else
    { k_random<double><<<vb, kBlock, 0, stream>>>(psi.as<double>(), D, o.seed); note_launches(1); }
  auto sum2 = [&](int mode, double e, double& a, double& b) -> int {
    { k_dots<double><<<vb, kBlock, 0, stream>>>(psi.as<double>(), y.as<double>(), D, e, mode, partial.as<double>()); note_launches(1); }
    std::vector<double> hs(2 * (size_t)vb);
    SED_TRY_CUDA(cudaMemcpyAsync(hs.data(), partial.ptr, hs.size() * 8, cudaMemcpyDeviceToHost, stream));
    SED_TRY_CUDA(cudaStreamSynchronize(stream));
    a = b = 0.0;
    for (unsigned i = 0; i < vb; ++i) {
      a += hs[2 * i];
      b += hs[2 * i + 1];
    }
    return LS_SUCCESS;
  };
  // normalise psi: y <- psi so that mode 0 gives <psi,psi>
  SED_TRY_CUDA(cudaMemcpyAsync(y.ptr, psi.ptr, D * 8, cudaMemcpyDeviceToDevice, stream));
  double nn = 0, dummy = 0;
  if (int st = sum2(0, 0.0, nn, dummy)) return st;
  { k_scale<double><<<vb, kBlock, 0, stream>>>(psi.as<double>(), D, 1.0 / std::sqrt(nn)); note_launches(1); }
  // graph of `check` FP32 steps
  cudaGraphExec_t graph = nullptr;
  size_t graph_kernels = 0;
  {
    cudaGraph_t g;
    SED_TRY_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    set_capturing(true);
    int st = LS_SUCCESS;
    unsigned spmv_blocks = 0;
    for (uint32_t i = 0; i < check && st == LS_SUCCESS; ++i) {
      k_zero_alpha<float><<<1, 1, 0, stream>>>(h, alpha.as<double>(), nullptr);
      Indirect ind;
      ind.k = &h->k;
      ind.stop = &h->stop;
      ind.ld = D;
      ind.partial = partial.as<double>();
      st = operator_apply_krylov32(op, Vf, ind, stream, &spmv_blocks);
      if (st) break;
      k_reduce<<<1, kRedThreads, 0, stream>>>(partial.as<double>(), spmv_blocks, h, alpha.as<double>(), 0);
      k_update32<<<vb, kBlock, 0, stream>>>(Vf, D, D, h, alpha.as<double>(), beta.as<double>(), partial.as<double>());
      k_reduce<<<1, kRedThreads, 0, stream>>>(partial.as<double>(), vb, h, beta.as<double>(), 1);
      k_scale_next32<<<vb, kBlock, 0, stream>>>(Vf, D, D, h, beta.as<double>());
      k_tridiag<<<1, 32, 0, stream>>>(h, alpha.as<double>(), beta.as<double>(), sbuf.as<double>(), work.as<double>());
    }
    set_capturing(false);
    cudaError_t e = cudaStreamEndCapture(stream, &g);
    if (st) {
      if (e == cudaSuccess) cudaGraphDestroy(g);
      return st;
    }
    SED_TRY_CUDA(e);
    cudaGraphGetNodes(g, nullptr, &graph_kernels);
    e = cudaGraphInstantiate(&graph, g, 0);
    cudaGraphDestroy(g);
    SED_TRY_CUDA(e);
  }
  struct GraphGuard {
    cudaGraphExec_t g;
    ~GraphGuard() {
      if (g) cudaGraphExecDestroy(g);
    }
  } graph_guard{graph};
  uint64_t steps32 = 0, matvecs = 0, cycles = 0;
  double E = 0.0, R = 1e300;
  bool converged = false;
  while (true) {
    // FP64: theta = <psi, H psi>, r = H psi - theta psi
    if (int st = operator_apply_device(op, 1, 1, psi.ptr, D, y.ptr, D, stream, SED_FORM_STREAM)) return st;
    ++matvecs;
    double pp = 0, py = 0;
    if (int st = sum2(0, 0.0, pp, py)) return st;
    E = py / pp;
    double rr = 0, unused = 0;
    if (int st = sum2(1, E, rr, unused)) return st;
    R = std::sqrt(rr / pp);
    if (o.progress) o.progress(o.progress_user, steps32 + matvecs, &E, &R, 1);
    if (R <= tol) {
      converged = true;
      break;
    }
    if (steps32 >= max_iter || cycles >= 64) break;
    // FP32 cycle from v0 = psi, v1 = r / ||r||
    double const rn = R * std::sqrt(pp);
    { k_start_cycle<<<vb, kBlock, 0, stream>>>(psi.as<double>(), y.as<double>(), D, E, 1.0 / rn, Vf, Vf + D); note_launches(1); }
    std::memset(hh, 0, sizeof(LzHeader));
    hh->k = 1;
    hh->m_max = m;
    hh->check = check;
    hh->nev = 1;
    hh->tol_est = std::max(0.5 * tol, 2e-6 * rn);
    SED_TRY_CUDA(cudaMemcpyAsync(h, hh, sizeof(LzHeader), cudaMemcpyHostToDevice, stream));
    double const a0 = E, b0 = rn;
    SED_TRY_CUDA(cudaMemcpyAsync(alpha.ptr, &a0, 8, cudaMemcpyHostToDevice, stream));
    SED_TRY_CUDA(cudaMemcpyAsync(beta.ptr, &b0, 8, cudaMemcpyHostToDevice, stream));
    SED_TRY_CUDA(cudaStreamSynchronize(stream));
    while (true) {
      SED_TRY_CUDA(cudaGraphLaunch(graph, stream));
      note_launches(graph_kernels);
      SED_TRY_CUDA(cudaMemcpyAsync(hh, h, sizeof(LzHeader), cudaMemcpyDeviceToHost, stream));
      SED_TRY_CUDA(cudaStreamSynchronize(stream));
      if (hh->stop) break;
      if (steps32 + hh->steps >= max_iter) break;
    }
    steps32 += hh->steps;
    ++cycles;
    uint32_t const n = hh->size ? hh->size : 1;
    if (!hh->stop) break;  // out of steps
    { k_ritz_mixed<<<vb, kBlock, 0, stream>>>(psi.as<double>(), Vf, D, D, sbuf.as<double>(), n, y.as<double>()); note_launches(1); }
    SED_TRY_CUDA(cudaMemcpyAsync(psi.ptr, y.ptr, D * 8, cudaMemcpyDeviceToDevice, stream));
    double pn = 0, d2 = 0;
    if (int st = sum2(0, 0.0, pn, d2)) return st;  // y == psi here
    { k_scale<double><<<vb, kBlock, 0, stream>>>(psi.as<double>(), D, 1.0 / std::sqrt(pn)); note_launches(1); }
  }
  // output
  if (evecs) {
    int const own = 1;
    char* dst = static_cast<char*>(evecs);
    if (out_dtype == own) {
      SED_TRY_CUDA(cudaMemcpyAsync(dst, psi.ptr, D * 8, cudaMemcpyDefault, stream));
    } else {
      DeviceBuffer tmp;
      if (int st = tmp.allocate(D * (size_t)elem_bytes(out_dtype))) return st;
      switch (out_dtype) {
        case 0: { k_convert<double, float><<<vb, kBlock, 0, stream>>>(psi.as<double>(), D, tmp.as<float>()); note_launches(1); } break;
        case 2: { k_convert<double, float2><<<vb, kBlock, 0, stream>>>(psi.as<double>(), D, tmp.as<float2>()); note_launches(1); } break;
        default: { k_convert<double, double2><<<vb, kBlock, 0, stream>>>(psi.as<double>(), D, tmp.as<double2>()); note_launches(1); } break;
      }
      SED_TRY_CUDA(cudaMemcpyAsync(dst, tmp.ptr, D * (size_t)elem_bytes(out_dtype), cudaMemcpyDefault, stream));
    }
  }
  SED_TRY_CUDA(cudaStreamSynchronize(stream));
  if (evals) evals[0] = E;
  if (rnorms) rnorms[0] = R;
  double const total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (info) {
    info->iterations = steps32 + matvecs;
    info->matvecs = steps32 + matvecs;
    info->restarts = cycles;
    info->fp32_iterations = steps32;
    info->seconds_total = total;
    info->seconds_setup = setup;
    info->seconds_solve = total - setup;
  }
  if (logging_enabled())
    log_line("sed_eigh (mixed): E0 = %.15g, residual %.3e, %llu FP32 steps, %llu FP64 matvecs, %llu cycles, %.3f s",
             E, R, (unsigned long long)steps32, (unsigned long long)matvecs, (unsigned long long)cycles, total);
  if (!converged)
    return fail(LS_NOT_CONVERGED, "mixed precision: residual " + std::to_string(R) + " above tolerance");
  return LS_SUCCESS;
}

}  // namespace
}  // namespace sed

using namespace sed;

extern "C" {

void sed_eigh_options_init(sed_eigh_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->struct_size = sizeof(sed_eigh_options);
  o->nev = 1;
  o->tol = 1e-8;
  o->block_size = 1;
  o->precision = SED_PRECISION_FP64;
  o->start = SED_START_RANDOM;
  o->form = SED_FORM_AUTO;
  o->seed = 1234;
}

int sed_eigh(ls_operator const* op, int dtype, sed_eigh_options const* opts, double* eigenvalues,
             void* eigenvectors, uint64_t ldv, double* residuals, sed_eigh_info* info) {
  if (!op) return fail(LS_INVALID_ARGUMENT, "sed_eigh: NULL operator");
  sed_eigh_options o;
  sed_eigh_options_init(&o);
  if (opts) {
    if (opts->struct_size != sizeof(sed_eigh_options))
      return fail(LS_INVALID_ARGUMENT, "sed_eigh: options struct_size mismatch");
    o = *opts;
  }
  if (o.nev == 0 || o.nev > kMaxNev) return fail(LS_INVALID_ARGUMENT, "nev must be in 1..16");
  if (dtype < 0 || dtype > 3) return fail(LS_INVALID_DATATYPE, "dtype must be 0..3");
  OperatorData& d = *op->d;
  std::lock_guard<std::mutex> lock(d.mu);
  if (!d.basis->built) return fail(LS_CACHE_NOT_BUILT, "basis has not been built (call ls_build)");
  if (!d.is_real && dtype < 2) return fail(LS_OPERATOR_IS_COMPLEX, "operator is complex; use dtype 2 or 3");
  uint64_t const D = d.basis->D;
  if (D == 0) return fail(LS_INVALID_ARGUMENT, "sed_eigh: the basis is empty");
  if (o.nev > D) return fail(LS_INVALID_ARGUMENT, "nev exceeds the dimension");
  if (eigenvectors && ldv < D) return fail(LS_INVALID_ARGUMENT, "ldv is smaller than the dimension");
  try {
    ScopedDevice dev(d.basis->device);
    if (int st = operator_ensure_ready(d)) return st;
    if (int st = wait_for_caller({o.start == SED_START_GIVEN ? o.start_vectors : nullptr, eigenvectors})) return st;
    if (int st = fix_wait(d)) return st;  // matvecs still queued on callers' streams share the workspace
    if (dtype >= 2 || !d.is_real) return solve<double2>(d, dtype, o, eigenvalues, eigenvectors, ldv, residuals, info);
    if (o.max_basis > 0 && o.max_basis <= 32 && o.block_size <= 1)
      return solve_thick(d, dtype, o, eigenvalues, eigenvectors, ldv, residuals, info);
    if (o.precision == SED_PRECISION_MIXED && o.nev == 1 && o.form != SED_FORM_ON_THE_FLY)
      return solve_mixed(d, dtype, o, eigenvalues, eigenvectors, ldv, residuals, info);
    return solve<double>(d, dtype, o, eigenvalues, eigenvectors, ldv, residuals, info);
  } catch (std::exception const& e) {
    return fail(LS_SYSTEM_ERROR, e.what());
  }
}

}  // extern "C"
