// tc_gemm.cu — BF16 GEMM on tcgen05 with TMA operand loads, for the
// training step of the learned start vector (mlp.cu).
//
// One CTA computes a 128 x BN tile of D = A B^T over its share of K (the K
// splits of a weight gradient are written as separate slabs). Warp-specialised:
// warp 4 streams 64-deep K slabs of A and B through a 4-stage ring with TMA,
// warp 5 issues the MMAs (M = 128, N = BN, K = 16) into BN tensor-memory
// columns, warps 0-3 wait for the last MMA and run the epilogue, thread t on
// accumulator row t.
//
// Operand orientation. An operand whose rows run along K in memory (K-major,
// "a[m][k]") is copied as one box of 64 K x 128 (or BN) rows: 128-byte rows,
// 8-row swizzle atoms, the layout of desc_sw128. An operand stored the other
// way round ("a[k][m]", M-major) is copied as boxes of 64 M x 64 K: each
// 128-byte row holds 64 consecutive M for one k, and the tensor cores read
// it through an MN-major descriptor (desc_sw128_mn, 8192 bytes from one
// 64-wide M block to the next) with the transpose bit of the instruction
// descriptor set. So the backward products (K = the batch) read the
// activations where the forward pass wrote them, with no transpose pass.
//
// Every wait is bounded (args.wait_ns): a wait that runs out sets the error
// flag; the TMA warp then waits for its copies in flight and the MMA warp
// for its MMAs before the CTA frees its tensor memory and returns.
#include "tc_gemm.cuh"

#include <cudaTypedefs.h>

#include <atomic>
#include <mutex>

#include "tc.cuh"

namespace sed {
namespace {

constexpr int kGemmStages = 4;
constexpr int kGemmThreads = 192;            // warps 0-3 epilogue, 4 TMA, 5 MMA
constexpr uint32_t kABytes = 128 * 128;      // 128 rows x 64 BF16
constexpr uint32_t kMnBoxBytes = 64 * 128;   // one 64 x 64 box of an M- or N-major operand

template <int BN>
struct GemmShape {
  static constexpr uint32_t b_bytes = BN * 128;
  static constexpr uint32_t stage = kABytes + b_bytes;
  static constexpr size_t smem = (size_t)kGemmStages * stage + 1024;  // + alignment slack
  static constexpr uint32_t tmem_cols = BN < 32 ? 32 : BN;
};

// Lane l ends with the sum over the warp's lanes of v[l]: a butterfly that
// halves the columns each lane keeps at every step (31 shuffles in all).
__device__ __forceinline__ float warp_column_sums(float (&v)[32], int lane) {
#pragma unroll
  for (int off = 16; off >= 1; off >>= 1) {
    bool const upper = (lane & off) != 0;
#pragma unroll
    for (int j = 0; j < off; ++j) {
      float const send = upper ? v[j] : v[j + off];
      float const keep = upper ? v[j + off] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, off);
    }
  }
  return v[0];
}

__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

template <int BN>
__global__ void __launch_bounds__(kGemmThreads, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, TcGemmArgs p) {
  using Sh = GemmShape<BN>;
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[kGemmStages], empty[kGemmStages];
  __shared__ uint64_t acc_full, drain;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  uint8_t* const smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  int const t = threadIdx.x, warp = t >> 5, lane = t & 31;
  int const m0 = blockIdx.y * 128, n0 = blockIdx.x * BN;
  int const kt0 = (int)((int64_t)p.k_tiles * blockIdx.z / p.split);
  int const nk = (int)((int64_t)p.k_tiles * (blockIdx.z + 1) / p.split) - kt0;  // >= 1: split <= k_tiles

  if (t == 0) {
    for (int i = 0; i < kGemmStages; ++i) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&empty[i], 1);
    }
    tc::mbar_init(&acc_full, 1);
    tc::mbar_init(&drain, 1);
    abort_flag = 0;
    tc::fence_mbar_init();
  }
  if (warp == 4 && lane == 0) {
    tc::tma_prefetch_map(&ta);
    tc::tma_prefetch_map(&tb);
  }
  __syncwarp();
  if (warp == 0) tc::tmem_alloc(&tmem_slot, Sh::tmem_cols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  uint32_t const tmem = tmem_slot;
  // everything above is private to the CTA; the operands and outputs belong
  // to the kernels before and after this one
  tc::grid_dependency_wait();
  tc::launch_dependents();

  if (warp == 4) {
    // ---- TMA warp: slab i goes to stage i % S once the MMAs of slab i - S
    // have read it
    if (lane == 0) {
      int issued = 0;
      for (int i = 0; i < nk; ++i) {
        int const st = i % kGemmStages;
        uint32_t const use = (uint32_t)(i / kGemmStages);
        if (use > 0 && !tc::mbar_wait(&empty[st], (use - 1) & 1u, p.wait_ns)) {
          abort_flag = 1;
          break;
        }
        uint8_t* const a_dst = smem + (size_t)st * Sh::stage;
        uint8_t* const b_dst = a_dst + kABytes;
        int const k = (kt0 + i) * 64;
        tc::mbar_expect_tx(&full[st], Sh::stage);
        if (p.a_mn) {
          tc::tma_load_2d(a_dst, &ta, m0, k, &full[st]);
          tc::tma_load_2d(a_dst + kMnBoxBytes, &ta, m0 + 64, k, &full[st]);
        } else {
          tc::tma_load_2d(a_dst, &ta, k, m0, &full[st]);
        }
        if (p.b_mn) {
#pragma unroll
          for (int j = 0; j < BN / 64; ++j) tc::tma_load_2d(b_dst + kMnBoxBytes * j, &tb, n0 + 64 * j, k, &full[st]);
        } else {
          tc::tma_load_2d(b_dst, &tb, k, n0, &full[st]);
        }
        issued = i + 1;
      }
      // never leave with copies in flight
      for (int h = issued > kGemmStages ? issued - kGemmStages : 0; h < issued; ++h)
        if (!tc::mbar_wait(&full[h % kGemmStages], (uint32_t)(h / kGemmStages) & 1u, p.wait_ns)) abort_flag = 1;
    }
    __syncwarp();
  } else if (warp == 5) {
    // ---- MMA warp: lane 0 issues and commits
    uint32_t const idesc = tc::idesc_bf16_f32_major(128, BN, p.a_mn != 0, p.b_mn != 0);
    bool ok = true;
    for (int i = 0; i < nk; ++i) {
      int const st = i % kGemmStages;
      bool const r = tc::mbar_wait(&full[st], (uint32_t)(i / kGemmStages) & 1u, p.wait_ns);
      ok = __all_sync(0xffffffffu, r);
      tc::fence_after_sync();
      if (!ok) break;
      uint32_t const a_s = tc::smem_u32(smem + (size_t)st * Sh::stage), b_s = a_s + kABytes;
      if (lane == 0) {
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          uint64_t const ad = p.a_mn ? tc::desc_sw128_mn(a_s + 2048u * kk, kMnBoxBytes) : tc::desc_sw128(a_s + 32u * kk);
          uint64_t const bd = p.b_mn ? tc::desc_sw128_mn(b_s + 2048u * kk, kMnBoxBytes) : tc::desc_sw128(b_s + 32u * kk);
          tc::mma_bf16(tmem, ad, bd, idesc, (i > 0 || kk > 0) ? 1u : 0u);
        }
        tc::mma_commit(&empty[st]);
      }
      __syncwarp();
    }
    if (lane == 0) {
      if (ok)
        tc::mma_commit(&acc_full);
      else
        abort_flag = 1;
      tc::mma_commit(&drain);  // every MMA issued has completed before the tensor memory is freed
      if (!tc::mbar_wait(&drain, 0, p.wait_ns)) abort_flag = 1;
    }
    __syncwarp();
  } else {
    // ---- epilogue: warp w reads tensor-memory lanes 32 w .. 32 w + 31
    bool const r = tc::mbar_wait(&acc_full, 0, p.wait_ns);
    bool const ok = __all_sync(0xffffffffu, r);
    tc::fence_after_sync();
    if (!ok) {
      if (lane == 0) abort_flag = 1;
    } else {
      int const m = m0 + warp * 32 + lane;
      bool const live = m < p.M;
      uint32_t const taddr = tmem + ((uint32_t)(warp * 32) << 16);
      bool const vec_add = p.ld_f32 % 4 == 0 && (reinterpret_cast<uintptr_t>(p.out_f32) & 15u) == 0;
#pragma unroll 1
      for (int c = 0; c < BN; c += 32) {
        float v[32];
        tc::tmem_ld32(taddr + (uint32_t)c, v);
        int const n = n0 + c;
        if (p.epilogue == kEpiTanh) {
          if (live) {
            uint32_t w[16];
#pragma unroll
            for (int j = 0; j < 16; ++j)
              w[j] = tc::pack_bf16x2(tanhf(v[2 * j] + __ldg(p.bias + n + 2 * j)),
                                     tanhf(v[2 * j + 1] + __ldg(p.bias + n + 2 * j + 1)));
            uint4* const dst = reinterpret_cast<uint4*>(p.out_bf16 + (int64_t)m * p.ld_out + n);
#pragma unroll
            for (int q = 0; q < 4; ++q) dst[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
          }
        } else if (p.epilogue == kEpiBack) {
          if (live) {
            uint4 const* const src = reinterpret_cast<uint4 const*>(p.aux + (int64_t)m * p.ld_aux + n);
            uint32_t w[16];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              uint4 const u = src[q];
              float const h0 = bf16_lo(u.x), h1 = bf16_hi(u.x), h2 = bf16_lo(u.y), h3 = bf16_hi(u.y);
              float const h4 = bf16_lo(u.z), h5 = bf16_hi(u.z), h6 = bf16_lo(u.w), h7 = bf16_hi(u.w);
              v[8 * q + 0] *= 1.0f - h0 * h0;
              v[8 * q + 1] *= 1.0f - h1 * h1;
              v[8 * q + 2] *= 1.0f - h2 * h2;
              v[8 * q + 3] *= 1.0f - h3 * h3;
              v[8 * q + 4] *= 1.0f - h4 * h4;
              v[8 * q + 5] *= 1.0f - h5 * h5;
              v[8 * q + 6] *= 1.0f - h6 * h6;
              v[8 * q + 7] *= 1.0f - h7 * h7;
            }
#pragma unroll
            for (int j = 0; j < 16; ++j) w[j] = tc::pack_bf16x2(v[2 * j], v[2 * j + 1]);
            uint4* const dst = reinterpret_cast<uint4*>(p.out_bf16 + (int64_t)m * p.ld_out + n);
#pragma unroll
            for (int q = 0; q < 4; ++q) dst[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j) v[j] = 0.0f;
          }
          float const s = warp_column_sums(v, lane);
          p.colsum[((int64_t)blockIdx.y * 4 + warp) * p.N + n + lane] = s;  // partial per (m-tile, warp)
        } else if (live) {  // kEpiAdd: this split's slab, reduced in a fixed order afterwards
          float* const dst = p.out_f32 + ((int64_t)blockIdx.z * p.M + m) * p.ld_f32 + n;
          if (vec_add && n + 32 <= p.n_valid) {
#pragma unroll
            for (int q = 0; q < 8; ++q)
              reinterpret_cast<float4*>(dst)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j)
              if (n + j < p.n_valid) dst[j] = v[j];
          }
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, Sh::tmem_cols);
  }
  if (t == 0 && abort_flag) atomicExch(p.error, 1);
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    else
      (void)cudaGetLastError();
  });
  return fn;
}

template <int BN>
int launch(cudaStream_t s, CUtensorMap const& a, CUtensorMap const& b, TcGemmArgs const& args) {
  static std::atomic<uint64_t> configured{0};  // one bit per device
  int dev = 0;
  SED_TRY_CUDA(cudaGetDevice(&dev));
  uint64_t const bit = 1ull << (dev & 63);
  if (!(configured.load() & bit)) {
    SED_TRY_CUDA(cudaFuncSetAttribute(k_tc_gemm<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)GemmShape<BN>::smem));
    configured.fetch_or(bit);
  }
  dim3 const grid((unsigned)(args.N / BN), (unsigned)((args.M + 127) / 128), (unsigned)args.split);
  SED_TRY_CUDA(launch_pdl(k_tc_gemm<BN>, grid, dim3(kGemmThreads), GemmShape<BN>::smem, s, a, b, args));
  note_launches(1);
  return LS_SUCCESS;
}

}  // namespace

int tma_map_bf16(CUtensorMap* out, void const* base, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows) {
  auto fn = encode_fn();
  if (!fn) return fail(LS_CUDA_ERROR, "cuTensorMapEncodeTiled is not available from the driver");
  if (!out || !base || rows == 0 || cols == 0 || cols > ld || ld % 8 || (reinterpret_cast<uintptr_t>(base) & 15u) ||
      box_rows == 0 || box_rows > 256)
    return fail(LS_INVALID_ARGUMENT, "tma_map_bf16: bad tensor shape or alignment");
  cuuint64_t const dims[2] = {cols, rows};
  cuuint64_t const strides[1] = {ld * 2};
  cuuint32_t const box[2] = {64, box_rows};
  cuuint32_t const elem[2] = {1, 1};
  CUresult const r = fn(out, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, elem,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(LS_CUDA_ERROR, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return LS_SUCCESS;
}

int tc_gemm(cudaStream_t s, CUtensorMap const& a, CUtensorMap const& b, TcGemmArgs const& args, int tile_n) {
  if ((tile_n != 64 && tile_n != 128) || args.M <= 0 || args.N <= 0 || args.N % tile_n || args.k_tiles <= 0 ||
      args.split < 1 || args.split > args.k_tiles || args.M > 65535 * 128 || !args.error)
    return fail(LS_INVALID_ARGUMENT, "tc_gemm: bad shape");
  return tile_n == 128 ? launch<128>(s, a, b, args) : launch<64>(s, a, b, args);
}

}  // namespace sed
