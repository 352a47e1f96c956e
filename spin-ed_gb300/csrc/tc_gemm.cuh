// tc_gemm.cuh — a BF16 GEMM on the 5th-generation tensor cores for the
// learned start vector's training step (mlp.cu): D = A B^T with A (M x K) and
// B (N x K) read by TMA from row-major BF16 arrays in either orientation, FP32
// accumulators in tensor memory, and a fused epilogue.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdint>
#include <utility>

#include "sed_internal.hpp"

namespace sed {

// A tensor map over a row-major BF16 array of `rows` rows of `cols` elements
// (row pitch `ld` elements, a multiple of 8), 128-byte swizzle, for boxes of
// 64 columns x `box_rows` rows. Rows past `rows` read as zero.
int tma_map_bf16(CUtensorMap* out, void const* base, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows);

enum TcEpilogue : int {
  kEpiTanh = 0,  // out_bf16[m][n] = bf16(tanh(acc + bias[n]))
  kEpiBack = 1,  // v = acc (1 - aux[m][n]^2); out_bf16[m][n] = bf16(v); column sums of v (see colsum)
  kEpiAdd = 2,   // out_f32[z][m][n] = acc for n < n_valid, z = the K split (one slab of M x ld_f32 per split)
};

struct TcGemmArgs {
  int M = 0, N = 0;   // output rows and columns; N a multiple of the tile width
  int k_tiles = 0;    // K / 64, rounded up (the tensor maps zero-fill past K)
  int split = 1;      // K splits, one CTA row each (gridDim.z)
  int a_mn = 0;       // A stored M-major: element (m, k) at a[k][m] (else a[m][k])
  int b_mn = 0;       // B stored N-major: element (n, k) at b[k][n] (else b[n][k])
  int epilogue = kEpiTanh;
  float const* bias = nullptr;
  __nv_bfloat16* out_bf16 = nullptr;
  int64_t ld_out = 0;
  __nv_bfloat16 const* aux = nullptr;
  int64_t ld_aux = 0;
  float* colsum = nullptr;  // kEpiBack: colsum[(m-tile * 4 + warp) * N + n] = the sum over the warp's 32 rows
  float* out_f32 = nullptr;
  int64_t ld_f32 = 0;
  int n_valid = 0;
  int* error = nullptr;  // set to 1 when a wait on the tensor cores or a copy timed out
  uint64_t wait_ns = 0;
};

// Launches kernel k on stream s with programmatic stream serialisation: it
// may start while the previous kernel of the stream finishes, and must call
// tc::grid_dependency_wait before it touches memory that kernel (or any
// earlier one) writes or reads.
template <class... Params, class... Args>
cudaError_t launch_pdl(void (*k)(Params...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

// Launches the GEMM on `s` (programmatic stream serialisation: the CTAs set
// up their barriers and tensor memory while the previous kernel finishes).
// The map of an operand stored K-major must have boxes of 64 x 128 rows (A)
// or 64 x tile-width rows (B); an M- or N-major operand's map has boxes of
// 64 x 64 rows. tile_n: 64 or 128.
int tc_gemm(cudaStream_t s, CUtensorMap const& a, CUtensorMap const& b, TcGemmArgs const& args, int tile_n);

}  // namespace sed
