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

// (h 2^32 + l) 2^sc as a double, rounded to nearest even, from integer
// operations only (h: |h| < 2^51; l in [0, 2^32)); results outside the normal
// range go through FP64 arithmetic, which rounds the same way.
__device__ __forceinline__ double rt_ldexp(double a, int p);
__device__ __forceinline__ double rt_compose(int64_t h, int64_t l, int sc) {
  __int128 const T = ((__int128)h << 32) + (__int128)l;
  if (T == 0) return 0.0;
  uint64_t const sign = T < 0 ? 1ull : 0ull;
  unsigned __int128 const u = (unsigned __int128)(T < 0 ? -T : T);
  uint64_t const uh = (uint64_t)(u >> 64), ul = (uint64_t)u;
  int const top = uh ? 127 - __clzll((long long)uh) : 63 - __clzll((long long)ul);
  uint64_t mant;
  int e = top;
  if (top <= 52) {
    mant = ul << (52 - top);
  } else {
    int const r = top - 52;  // 1 .. 30
    mant = (uint64_t)(u >> r);
    uint64_t const rem = ul & ((1ull << r) - 1ull), half = 1ull << (r - 1);
    if (rem > half || (rem == half && (mant & 1ull))) ++mant;
    if (mant >> 53) {
      mant >>= 1;
      ++e;
    }
  }
  int const biased = e + sc + 1023;
  if (biased < 1 || biased > 2046)
    return rt_ldexp(__fma_rn((double)h, 4294967296.0, (double)l), sc);
  return __longlong_as_double((long long)((sign << 63) | ((uint64_t)biased << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

__device__ __forceinline__ double rt_ldexp(double a, int p) {
  if (p >= -1000 && p <= 1000) return a * fix_pow2(p);
  int const h = p / 2;
  return (a * fix_pow2(h)) * fix_pow2(p - h);
}

// KS: K columns per slice (16 or 32, at least m); KT: 64-column K tiles; NJ:
// output columns handled (8 when kk <= 8, else 16; the MMA is always N = 16).
template <int KS, int NJ>
__global__ void __launch_bounds__(kRtRows, (KS == 16 && NJ == 8) ? 4 : 3) k_rotate_tc(RtArgs a) {
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
    uint64_t yb[KS];
    int emax = 1, bad = 0;
#pragma unroll
    for (int k = 0; k < KS; ++k) {
      yb[k] = ((uint32_t)k < m && (uint32_t)t < a.kk) ? (uint64_t)__double_as_longlong(a.Y[(uint64_t)k * a.kk + t]) : 0ull;
      int const e = (int)((yb[k] >> 52) & 0x7FF);
      if (e == 0x7FF) bad = 1;
      emax = max(emax, e ? e : 1);
    }
    uint64_t mag[KS];
    uint32_t neg = 0;
#pragma unroll
    for (int k = 0; k < KS; ++k) {
      mag[k] = bad ? 0 : rt_mag(__longlong_as_double((long long)yb[k]), emax);
      neg |= (uint32_t)(yb[k] >> 63) << k;
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
    // ---- this thread's row of V: scale, slices into A (integer operations)
    int emax = 1, bad = 0;
    uint32_t neg = 0;
    {
      uint64_t vb[KS];
#pragma unroll
      for (int k = 0; k < KS; ++k) {
        vb[k] = (live && (uint32_t)k < m) ? (uint64_t)__double_as_longlong(__ldcs(a.V + (uint64_t)k * a.ld + row)) : 0ull;
        int const e = (int)((vb[k] >> 52) & 0x7FF);
        if (e == 0x7FF) bad = 1;
        emax = max(emax, e ? e : 1);
        neg |= (uint32_t)(vb[k] >> 63) << k;
      }
      uint64_t mag[KS];
#pragma unroll
      for (int k = 0; k < KS; ++k) mag[k] = bad ? 0 : rt_mag(__longlong_as_double((long long)vb[k]), emax);
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
    // ---- every thread: wait for the MMAs, read its lane's 8 groups x NJ sums
    if (!tc::mbar_wait(&done, it & 1u, a.wait_ns)) {
      ok = false;
      atomicExch(a.error, 1);
    }
    tc::fence_after_sync();
    ok = __syncthreads_and(ok);
    if (!ok) break;
    int64_t hi[NJ], lo[NJ];
#pragma unroll
    for (int j = 0; j < NJ; ++j) hi[j] = lo[j] = 0;
    uint32_t const lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
    for (int g = 0; g < kRtGroups; ++g) {
      float p[NJ];
      tc::tmem_ld(lane_addr + (uint32_t)(g * kRtN), p);
      int const sh = 8 * (7 - g);
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        int64_t const pv = (int64_t)__float2int_rz(p[j]);  // an exact integer below 2^24
        if (sh >= 32) {
          hi[j] += pv << (sh - 32);
        } else {
          hi[j] += pv >> (32 - sh);
          lo[j] += (int64_t)(((uint64_t)pv << sh) & 0xFFFFFFFFull);
        }
      }
    }
    tc::fence_before_sync();
    // ---- T = hi 2^32 + lo rounded to FP64 and scaled, in place
    if (live) {
      int const scr = emax - 1022 - 72;
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        if ((uint32_t)j >= a.kk) break;
        double const r = (bad || bad_col[j])
                             ? __longlong_as_double(0x7FF8000000000000ll)
                             : rt_compose(hi[j] + (lo[j] >> 32), lo[j] & 0xFFFFFFFFll, scr + (ecol[j] - 1022));
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
  unsigned const grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)sms * 4);  // 4 x 128 TMEM columns per SM
  auto go = [&](auto kern, int ks) -> int {
    size_t const smem = 1024 + (size_t)((kRtSlices * ks + 63) / 64) * (kRtRows + kRtN) * 128;
    SED_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, kRtRows, smem, stream>>>(a);
    return LS_SUCCESS;
  };
  int st;
  if (m <= 16) st = kk <= 8 ? go(k_rotate_tc<16, 8>, 16) : go(k_rotate_tc<16, 16>, 16);
  else st = kk <= 8 ? go(k_rotate_tc<32, 8>, 32) : go(k_rotate_tc<32, 16>, 32);
  if (st) return st;
  note_launches(1);
  SED_TRY_CUDA(cudaGetLastError());
  return LS_SUCCESS;
}

}  // namespace sed
