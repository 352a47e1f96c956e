// util.cuh — small device helpers shared by the libsed kernels.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

namespace sed {

constexpr unsigned kBlock = 256;

struct cplx {
  double re, im;
};

__host__ __device__ __forceinline__ cplx operator+(cplx a, cplx b) { return {a.re + b.re, a.im + b.im}; }
__host__ __device__ __forceinline__ cplx operator-(cplx a, cplx b) { return {a.re - b.re, a.im - b.im}; }
__host__ __device__ __forceinline__ cplx operator*(cplx a, cplx b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__host__ __device__ __forceinline__ cplx operator*(double a, cplx b) { return {a * b.re, a * b.im}; }
__host__ __device__ __forceinline__ cplx conj(cplx a) { return {a.re, -a.im}; }

template <class V>
__host__ __device__ __forceinline__ V zero();
template <>
__host__ __device__ __forceinline__ double zero<double>() { return 0.0; }
template <>
__host__ __device__ __forceinline__ cplx zero<cplx>() { return {0.0, 0.0}; }

// acc += a * b
__device__ __forceinline__ void mac(double& acc, double a, double b) { acc = fma(a, b, acc); }
__device__ __forceinline__ void mac(cplx& acc, cplx a, cplx b) {
  acc.re = fma(a.re, b.re, fma(-a.im, b.im, acc.re));
  acc.im = fma(a.re, b.im, fma(a.im, b.re, acc.im));
}
// Rounded products and sums (no contraction into FMA), so that every kernel
// that evaluates the same expression gets the same bits.
__device__ __forceinline__ double mulv(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ cplx mulv(cplx a, cplx b) {
  return {__dsub_rn(__dmul_rn(a.re, b.re), __dmul_rn(a.im, b.im)),
          __dadd_rn(__dmul_rn(a.re, b.im), __dmul_rn(a.im, b.re))};
}
__device__ __forceinline__ cplx mulv(double a, cplx b) { return {__dmul_rn(a, b.re), __dmul_rn(a, b.im)}; }
__device__ __forceinline__ double addv(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ cplx addv(cplx a, cplx b) { return {__dadd_rn(a.re, b.re), __dadd_rn(a.im, b.im)}; }

// Storage types of the four dtypes (src/SpinED/Internal.hs:404-409).
template <class T>
struct Store;
template <>
struct Store<float> {
  using V = double;
  static __device__ __forceinline__ double load(float const* p, uint64_t i) { return (double)p[i]; }
  static __device__ __forceinline__ void store(float* p, uint64_t i, double v) { p[i] = (float)v; }
};
template <>
struct Store<double> {
  using V = double;
  static __device__ __forceinline__ double load(double const* p, uint64_t i) { return p[i]; }
  static __device__ __forceinline__ void store(double* p, uint64_t i, double v) { p[i] = v; }
};
template <>
struct Store<float2> {
  using V = cplx;
  static __device__ __forceinline__ cplx load(float2 const* p, uint64_t i) {
    float2 const v = p[i];
    return {(double)v.x, (double)v.y};
  }
  static __device__ __forceinline__ void store(float2* p, uint64_t i, cplx v) {
    p[i] = make_float2((float)v.re, (float)v.im);
  }
};
template <>
struct Store<double2> {
  using V = cplx;
  static __device__ __forceinline__ cplx load(double2 const* p, uint64_t i) {
    double2 const v = p[i];
    return {v.x, v.y};
  }
  static __device__ __forceinline__ void store(double2* p, uint64_t i, cplx v) {
    p[i] = make_double2(v.re, v.im);
  }
};

__device__ __forceinline__ double dot_re(double a, double b) { return a * b; }
__device__ __forceinline__ double dot_re(cplx a, cplx b) { return fma(a.re, b.re, a.im * b.im); }

// Sum of v over the block; the result is valid in thread 0. red holds one
// double per warp. Every thread of the block must call it.
__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (unsigned w = 0; w < (blockDim.x + 31) / 32; ++w) s += red[w];
  __syncthreads();
  return s;
}

// Krylov indirection: with k != nullptr, kernels read the step index from
// device memory so that one captured graph serves every Lanczos step.
struct Indirect {
  uint32_t const* k = nullptr;
  uint32_t const* stop = nullptr;
  uint64_t ld = 0;
  double* partial = nullptr;
  // fixed-point matvec: u and F of x were written by the step that produced
  // x (Lanczos' scale kernel), so the matvec skips its own pre-pass
  bool prescaled = false;
};

inline unsigned grid_size(uint64_t work, int device, unsigned per_sm = 16, unsigned block = kBlock) {
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  uint64_t const want = (work + block - 1) / block;
  uint64_t const cap = (uint64_t)sms * per_sm;
  return (unsigned)std::max<uint64_t>(1, std::min(want, cap));
}

// Exclusive scan of v[0..n) in place by one block of 1024 threads; v[n] = total.
static __global__ void k_scan_u64(uint64_t* __restrict__ v, uint64_t n) {
  __shared__ uint64_t sums[1024];
  unsigned const T = blockDim.x;
  uint64_t const per = (n + T - 1) / T;
  uint64_t const b = min(n, (uint64_t)threadIdx.x * per), e = min(n, b + per);
  uint64_t s = 0;
  for (uint64_t i = b; i < e; ++i) s += v[i];
  sums[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t acc = 0;
    for (unsigned i = 0; i < T; ++i) {
      uint64_t const t = sums[i];
      sums[i] = acc;
      acc += t;
    }
    v[n] = acc;
  }
  __syncthreads();
  uint64_t acc = sums[threadIdx.x];
  for (uint64_t i = b; i < e; ++i) {
    uint64_t const t = v[i];
    v[i] = acc;
    acc += t;
  }
}

// Philox4x32-10 (Salmon et al., SC'11): ten rounds on the counter c with key
// (k0, k1), in place.
__device__ __forceinline__ void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint32_t const hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    uint32_t const hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
    uint32_t const n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

__device__ __forceinline__ double u01_53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

}  // namespace sed
