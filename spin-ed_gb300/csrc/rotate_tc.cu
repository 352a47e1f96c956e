// rotate_tc.cu — V[:, 0..kk) <- V[:, 0..m) Y in FP64 on the tensor cores: the
// basis rotation of a thick restart (Ritz vectors of T replacing the first
// kk Krylov vectors in place), a D x m by m x kk product with D up to 1e9
// and m <= 32, which on GB300's FP64 pipe (about 0.5 TFMA/s) takes several
// times longer than streaming V through HBM.
//
// Method: error-free splitting of FP64 operands into small-integer slices
// whose products the tensor cores sum exactly (Ozaki, Ogita, Oishi & Rump,
// Numer. Algorithms 59 (2012); in the integer-slice form of Ootomo, Ozaki &
// Yokota, IJHPCA (2024)):
//   - row r of V is scaled by its largest exponent: |V_rk| < 2^R_r, and
//     M_rk = floor(|V_rk| 2^(56 - R_r)) < 2^56 is cut into seven 8-bit
//     slices, M = sum_s A_s 2^(8 (6 - s)); column j of Y likewise (N, B_t);
//   - every slice value (|A| <= 255, sign included) is exact in BF16;
//   - the products group by g = s + t: P_g = sum_{s+t=g} sum_k A_s B_t has at
//     most 7 x 32 x 255^2 < 2^24 in magnitude, so the FP32 accumulation of
//     tcgen05.mma (kind::f16, BF16 operands) is exact; groups g > 7 are
//     below 2^-55 of the leading term and are dropped;
//   - sum_k V_rk Y_kj = 2^(R_r + R_j - 72) T with T = sum_{g<=7} P_g
//     2^(8 (7 - g)), an integer of at most 83 bits assembled exactly in two
//     int64 words, converted to FP64 with one rounding and scaled exactly.
// The result differs from an FP64 GEMM only by the truncation of the
// operands to 56 bits relative to their row/column maxima (< 2^-55) and the
// final rounding.
//
// Layout: one CTA of 128 threads per 128-row tile (thread = row = TMEM
// lane), persistent over tiles. A (128 rows x 7 KS slices-by-k, BF16) and B
// (16 columns of Y x the same K) sit in shared memory in the K-major 128-byte
// swizzled layout of tc.cuh; 8 TMEM accumulators of 16 columns, one per
// group g. Every wait is bounded; a wait that runs out sets the error flag,
// waits (bounded) for the MMAs in flight and frees TMEM.
#include <algorithm>
#include <cmath>

#include "operator_impl.cuh"
#include "tc.cuh"

namespace sed {
namespace {

constexpr int kRtRows = 128;       // rows per tile: TMEM lanes, one thread each
constexpr int kRtSlices = 7;       // 8-bit slices of a 56-bit magnitude
constexpr int kRtGroups = 8;       // s + t <= 7
constexpr int kRtN = 16;           // output columns (kk <= 16)
constexpr uint32_t kRtCols = 128;  // TMEM columns: 8 groups x 16
constexpr int kRtMaxM = 32;
constexpr uint64_t kRtWaitNs = 1000000000ull;  // default wait bound: 1 s

struct RtArgs {
  double* V;
  uint64_t ld, D;
  double const* Y;  // m x kk, row-major
  uint32_t m, kk;
  int* error;
  uint64_t wait_ns;
};

__device__ __forceinline__ int rt_expo(double v) {  // biased exponent, 1 for subnormals and zero
  int const e = (int)(((uint64_t)__double_as_longlong(v) >> 52) & 0x7FF);
  return e ? e : 1;
}

// floor(|v| 2^(56 - R)) with R = Emax - 1022 (Emax: the largest biased
// exponent of the row or column): an integer below 2^56.
__device__ __forceinline__ uint64_t rt_mag(double v, int Emax) {
  uint64_t const b = (uint64_t)__double_as_longlong(v);
  int const e = (int)((b >> 52) & 0x7FF);
  uint64_t const m = (b & 0xFFFFFFFFFFFFFull) | (e ? (1ull << 52) : 0ull);
  int const sh = (e ? e : 1) - Emax + 3;  // <= 3
  if (sh >= 0) return m << sh;
  return sh <= -64 ? 0 : m >> (-sh);
}

// BF16 bits of the integer n (0..255) with the given sign.
__device__ __forceinline__ uint32_t rt_bf16(uint32_t n, uint32_t neg) {
  if (n == 0) return 0;
  uint32_t const e = 31 - __clz(n);  // 0..7
  return (neg << 15) | ((127 + e) << 7) | ((n << (7 - e)) & 0x7Fu);
}

// Writes one operand row into `base` (ROWS rows, KT tiles of 64 K columns):
// K element s KS + k holds slice s of magnitude mag[k] (k < m; zero padding
// elsewhere), signed by bit k of negmask. All indices are compile-time.
template <int KS, int KT, int ROWS>
__device__ __forceinline__ void rt_put_row(uint8_t* base, uint32_t r, uint64_t const (&mag)[KS], uint32_t negmask,
                                           uint32_t m) {
#pragma unroll
  for (int e0 = 0; e0 < KT * 64; e0 += 8) {  // one 16-byte chunk: 8 consecutive K elements
    uint32_t w[4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      uint32_t half[2];
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        int const e = e0 + 2 * h + p;
        int const s = e / KS, k = e % KS;
        uint32_t bits = 0;
        if (s < kRtSlices && (uint32_t)k < m)
          bits = rt_bf16((uint32_t)(mag[k] >> (8 * (6 - s))) & 0xFFu, (negmask >> k) & 1u);
        half[p] = bits;
      }
      w[h] = half[0] | (half[1] << 16);
    }
    int const kt = e0 >> 6, c = (e0 & 63) >> 3;
    *reinterpret_cast<uint4*>(base + kt * ROWS * 128 + r * 128 + ((c ^ (r & 7)) << 4)) =
        make_uint4(w[0], w[1], w[2], w[3]);
  }
}

__device__ __forceinline__ double rt_ldexp(double a, int p) {
  if (p >= -1000 && p <= 1000) return a * fix_pow2(p);
  int const h = p / 2;
  return (a * fix_pow2(h)) * fix_pow2(p - h);
}

// KS: K columns per slice (16 or 32, at least m); KT: 64-column K tiles.
template <int KS>
__global__ void __launch_bounds__(kRtRows) k_rotate_tc(RtArgs a) {
  constexpr int KT = (kRtSlices * KS + 63) / 64;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t done, drain;
  __shared__ uint32_t tmem_slot;
  __shared__ int bad_col[kRtN];
  __shared__ int ecol[kRtN];
  uint8_t* const smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* const A = smem;                               // 128 rows x KT x 128 B
  uint8_t* const B = smem + (size_t)KT * kRtRows * 128;  // 16 rows x KT x 128 B
  int const t = threadIdx.x, warp = t >> 5;
  uint32_t const m = a.m;

  if (t == 0) {
    tc::mbar_init(&done, 1);
    tc::mbar_init(&drain, 1);
    tc::fence_mbar_init();
  }
  // B: thread j < 16 writes column j of Y as row j (zero rows beyond kk)
  if (t < kRtN) {
    double y[KS];
    int emax = 1, bad = 0;
#pragma unroll
    for (int k = 0; k < KS; ++k) {
      y[k] = ((uint32_t)k < m && (uint32_t)t < a.kk) ? a.Y[(uint64_t)k * a.kk + t] : 0.0;
      int const e = rt_expo(y[k]);
      if (e == 0x7FF) bad = 1;
      emax = max(emax, e);
    }
    uint64_t mag[KS];
    uint32_t neg = 0;
#pragma unroll
    for (int k = 0; k < KS; ++k) {
      mag[k] = bad ? 0 : rt_mag(y[k], emax);
      neg |= (y[k] < 0.0 ? 1u : 0u) << k;
    }
    rt_put_row<KS, KT, kRtN>(B, (uint32_t)t, mag, neg, m);
    bad_col[t] = bad;
    ecol[t] = emax;
  }
  __syncwarp();  // warp 0 diverged above; the allocation is warp-wide
  if (warp == 0) tc::tmem_alloc(&tmem_slot, kRtCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  uint32_t const tmem = tmem_slot;
  uint32_t const idesc = tc::idesc_bf16_f32(kRtRows, kRtN);
  uint32_t const a0 = tc::smem_u32(A), b0 = tc::smem_u32(B);
  uint64_t const tiles = (a.D + kRtRows - 1) / kRtRows;
  bool ok = true;
  uint32_t it = 0;
  for (uint64_t tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x, ++it) {
    uint64_t const row = tile * kRtRows + (uint64_t)t;
    bool const live = row < a.D;
    // ---- this thread's row of V: scale, slices into A
    double v[KS];
    int emax = 1, bad = 0;
#pragma unroll
    for (int k = 0; k < KS; ++k) {
      v[k] = (live && (uint32_t)k < m) ? __ldcs(a.V + (uint64_t)k * a.ld + row) : 0.0;
      int const e = rt_expo(v[k]);
      if (e == 0x7FF) bad = 1;
      emax = max(emax, e);
    }
    {
      uint64_t mag[KS];
      uint32_t neg = 0;
#pragma unroll
      for (int k = 0; k < KS; ++k) {
        mag[k] = bad ? 0 : rt_mag(v[k], emax);
        neg |= (v[k] < 0.0 ? 1u : 0u) << k;
      }
      rt_put_row<KS, KT, kRtRows>(A, (uint32_t)t, mag, neg, m);
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // ---- one thread issues the MMAs: group g accumulates A_s B_{g-s}
    if (warp == 0) {
      if (tc::elect_one()) {
        for (int g = 0; g < kRtGroups; ++g) {
          uint32_t const d = tmem + (uint32_t)(g * kRtN);
          bool first = true;
          for (int s = max(0, g - (kRtSlices - 1)); s <= min(g, kRtSlices - 1); ++s) {
            int const tt = g - s;
            for (uint32_t kh = 0; kh < (uint32_t)KS / 16; ++kh) {
              uint32_t const ea = (uint32_t)(s * KS) + 16 * kh, eb = (uint32_t)(tt * KS) + 16 * kh;
              uint32_t const aa = a0 + (ea >> 6) * kRtRows * 128 + ((ea & 63) >> 4) * 32;
              uint32_t const bb = b0 + (eb >> 6) * kRtN * 128 + ((eb & 63) >> 4) * 32;
              tc::mma_bf16(d, tc::desc_sw128(aa), tc::desc_sw128(bb), idesc, first ? 0u : 1u);
              first = false;
            }
          }
        }
        tc::mma_commit(&done);
      }
      __syncwarp();
    }
    // ---- every thread: wait for the MMAs, read its lane's 8 x 16 sums
    if (!tc::mbar_wait(&done, it & 1u, a.wait_ns)) {
      ok = false;
      atomicExch(a.error, 1);
    }
    tc::fence_after_sync();
    ok = __syncthreads_and(ok);
    if (!ok) break;
    int64_t hi[kRtN], lo[kRtN];
#pragma unroll
    for (int j = 0; j < kRtN; ++j) hi[j] = lo[j] = 0;
    uint32_t const lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
    for (int q = 0; q < kRtGroups / 2; ++q) {  // two groups per 32-column load
      float p[32];
      tc::tmem_ld32(lane_addr + (uint32_t)(q * 32), p);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        int const g = 2 * q + h, sh = 8 * (7 - g);
#pragma unroll
        for (int j = 0; j < kRtN; ++j) {
          int64_t const pv = (int64_t)__float2int_rz(p[h * kRtN + j]);  // an exact integer below 2^24
          if (sh >= 32) {
            hi[j] += pv << (sh - 32);
          } else {
            hi[j] += pv >> (32 - sh);
            lo[j] += (int64_t)(((uint64_t)pv << sh) & 0xFFFFFFFFull);
          }
        }
      }
    }
    tc::fence_before_sync();
    // ---- T = hi 2^32 + lo, one rounding to FP64, exact scaling; in place
    if (live) {
#pragma unroll
      for (int j = 0; j < kRtN; ++j) {
        if ((uint32_t)j >= a.kk) break;
        int64_t const h = hi[j] + (lo[j] >> 32);
        int64_t const l = lo[j] & 0xFFFFFFFFll;
        double r;
        if (bad || bad_col[j]) {
          r = __longlong_as_double(0x7FF8000000000000ll);
        } else {
          double const T = __fma_rn((double)h, 4294967296.0, (double)l);
          r = rt_ldexp(T, (emax - 1022) + (ecol[j] - 1022) - 72);
        }
        __stcs(a.V + (uint64_t)j * a.ld + row, r);
      }
    }
    __syncthreads();  // every lane has read TMEM before the next tile's MMAs overwrite it
  }
  if (!ok && warp == 0) {
    // the MMAs of the tile whose wait ran out may still run: the thread that
    // issued them commits once more to a barrier of its own and waits
    // (bounded) for that single phase before TMEM is released
    if (tc::elect_one()) {
      tc::mma_commit(&drain);
      tc::mbar_wait(&drain, 0, a.wait_ns);
    }
    __syncwarp();
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kRtCols);
  }
}

}  // namespace

int g_rotate_path = SED_ROTATE_AUTO;

bool rotate_tc_eligible(uint32_t m, uint32_t kk) {
  return m >= 1 && m <= (uint32_t)kRtMaxM && kk >= 1 && kk <= (uint32_t)kRtN;
}

int rotate_tc(double* V, uint64_t ld, uint32_t m, double const* Y, uint32_t kk, uint64_t D, cudaStream_t stream,
              int* error_flag) {
  if (!rotate_tc_eligible(m, kk)) return fail(LS_INVALID_ARGUMENT, "rotate_tc: needs m <= 32 and kk <= 16");
  if (D == 0) return LS_SUCCESS;
  int dev = 0;
  SED_TRY_CUDA(cudaGetDevice(&dev));
  int sms = 152;
  SED_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  RtArgs a{};
  a.V = V;
  a.ld = ld;
  a.D = D;
  a.Y = Y;
  a.m = m;
  a.kk = kk;
  a.error = error_flag;
  a.wait_ns = device_wait_ns(kRtWaitNs);
  uint64_t const tiles = (D + kRtRows - 1) / kRtRows;
  unsigned const grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)sms * 3);  // 3 x 128 TMEM columns per SM
  if (m <= 16) {
    size_t const smem = 1024 + (size_t)((kRtSlices * 16 + 63) / 64) * (kRtRows + kRtN) * 128;
    SED_TRY_CUDA(cudaFuncSetAttribute(k_rotate_tc<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_rotate_tc<16><<<grid, kRtRows, smem, stream>>>(a);
  } else {
    size_t const smem = 1024 + (size_t)((kRtSlices * 32 + 63) / 64) * (kRtRows + kRtN) * 128;
    SED_TRY_CUDA(cudaFuncSetAttribute(k_rotate_tc<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_rotate_tc<32><<<grid, kRtRows, smem, stream>>>(a);
  }
  note_launches(1);
  SED_TRY_CUDA(cudaGetLastError());
  return LS_SUCCESS;
}

}  // namespace sed
