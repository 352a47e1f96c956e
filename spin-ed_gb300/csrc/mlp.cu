// mlp.cu — the learned start vector: a small MLP over spin configurations,
// trained and evaluated on the GPU by the kernels in this file.
//
// Network (n inputs -> h -> h -> 2), x_j = +1 / -1 for spin j up / down:
//   h1 = tanh(W1 x + b1), h2 = tanh(W2 h1 + b2), (a, s) = W3 h2 + b3.
// a models log|psi(x)|, s the logit of "sign psi(x) = prior(x)", with the
// sign prior (-1)^popcount(x & sign_mask) (a Marshall-type sublattice rule
// for bipartite lattices; sign_mask = 0 means no prior). Weights are kept as
// an FP32 master copy for Adam and used in BF16 (round to nearest even) by the
// forward and backward passes; products accumulate in FP32.
//
// The symmetric-basis amplitude of representative r relates to the amplitude
// of the configuration itself by psi(r) = c_r * n_r, n_r = ||P r|| =
// sqrt(S_r / |G|) (every orbit member carries |c_r n_r|). Training labels are
// log|c_r n_r| and sign(c_r) for representatives drawn with probability
// |c_r|^2 from ground states the solver computed at neighbouring couplings;
// the start vector is v_r = prior(r) sign(s) exp(a) / n_r.
//
// Two paths. Tensor cores (n_in <= 64, hidden 128, 256 or 512, the default):
// training runs every product of the forward and backward passes through
// the tcgen05 GEMM of tc_gemm.cu with BF16 activations (the weight-gradient
// products read the activations transposed, through M-/N-major operand
// descriptors), and inference runs the whole network in one persistent
// kernel, k_mlp_forward_tc. CUDA cores (any shape, or SED_MLP_PATH_SIMT):
// SIMT GEMM tiles (64 x 64 outputs per 256-thread block, 16-deep K steps
// through shared memory, 4 x 4 outputs per thread) with arbitrary strides
// and FP32 activations.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <type_traits>

#include "sed_internal.hpp"
#include "tc.cuh"
#include "tc_gemm.cuh"
#include "util.cuh"

namespace sed {
namespace {

constexpr int kTile = 64, kTK = 16;

// C[m][n] (=|+=) act(sum_k A(m,k) B(k,n) + bias[n]) with arbitrary strides;
// A is FP32, B is TB (float or bf16). act: 0 none, 1 tanh.
template <class TB>
__global__ void __launch_bounds__(256)
    k_gemm(int M, int N, int K, float const* __restrict__ A, int64_t sam, int64_t sak,
           TB const* __restrict__ B, int64_t sbk, int64_t sbn, float* __restrict__ C, int64_t ldc,
           float const* __restrict__ bias, int act, int accumulate) {
  __shared__ float As[kTK][kTile + 1];
  __shared__ float Bs[kTK][kTile + 1];
  int const tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  int const m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
  // loads run along whichever of (m, k) has unit stride, for coalescing
  bool const a_k_fast = sak == 1, b_n_fast = sbn == 1;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kTK) {
    for (int q = threadIdx.x; q < kTK * kTile; q += 256) {
      int const kk = a_k_fast ? q % kTK : q / kTile, mm = a_k_fast ? q / kTK : q % kTile;
      int const gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? A[gm * sam + gk * sak] : 0.0f;
    }
    for (int q = threadIdx.x; q < kTK * kTile; q += 256) {
      int const kk = b_n_fast ? q / kTile : q % kTK, nn = b_n_fast ? q % kTile : q / kTK;
      int const gn = n0 + nn, gk = k0 + kk;
      float bv = 0.0f;
      if (gn < N && gk < K) {
        if constexpr (std::is_same<TB, float>::value)
          bv = B[gk * sbk + gn * sbn];
        else
          bv = __bfloat162float(B[gk * sbk + gn * sbn]);
      }
      Bs[kk][nn] = bv;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        a[i] = As[kk][ty * 4 + i];
        b[i] = Bs[kk][tx * 4 + i];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int const gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int const gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      float v = acc[i][j];
      if (bias) v += bias[gn];
      if (act == 1) v = tanhf(v);
      float* c = C + (int64_t)gm * ldc + gn;
      *c = accumulate ? *c + v : v;
    }
  }
}

// x[b][j] = +1 / -1 from the bits of states[b].
__global__ void k_spins(uint64_t const* __restrict__ states, int64_t n, int bits, float* __restrict__ x) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n * bits;
       q += (int64_t)gridDim.x * blockDim.x) {
    int64_t const b = q / bits;
    int const j = (int)(q % bits);
    x[q] = ((states[b] >> j) & 1u) ? 1.0f : -1.0f;
  }
}

__device__ __forceinline__ float prior_flip(uint64_t state, uint64_t mask) {
  return (__popcll(state & mask) & 1) ? 1.0f : 0.0f;
}

// Output gradient of L = mean_b [(a_b - t_b)^2 + BCE(s_b, y_b)] with
// y_b = [sign psi_b == prior(state_b)], and the loss partials.
__global__ void k_out_grad(float const* __restrict__ out, uint64_t const* __restrict__ states, uint64_t sign_mask,
                           float const* __restrict__ t_abs, float const* __restrict__ t_sign, int64_t n,
                           float* __restrict__ dout, double* __restrict__ loss_partial) {
  __shared__ double red[32];
  double l = 0.0;
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < n;
       b += (int64_t)gridDim.x * blockDim.x) {
    float const a = out[2 * b], s = out[2 * b + 1];
    float const da = a - t_abs[b];
    float const y = fabsf(t_sign[b] - prior_flip(states[b], sign_mask));
    float const p = 1.0f / (1.0f + expf(-s));
    dout[2 * b] = 2.0f * da / (float)n;
    dout[2 * b + 1] = (p - y) / (float)n;
    // BCE with logits in its stable form: max(s, 0) - s y + log(1 + e^-|s|)
    l += (double)da * da + (double)(fmaxf(s, 0.0f) - s * y + log1pf(expf(-fabsf(s))));
  }
  double const tot = block_sum(l, red);
  if (threadIdx.x == 0) loss_partial[blockIdx.x] = tot;
}

// g *= 1 - h^2 (tanh derivative, in place on the gradient)
__global__ void k_tanh_back(float const* __restrict__ h, float* __restrict__ g, int64_t n) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    g[q] *= 1.0f - h[q] * h[q];
}

// Adam step on the FP32 master copy, refreshing the BF16 copy; with w1p set
// also the tensor-core training's copy of W1 (the first n_w1 = hidden x
// n_in parameters), rows padded to 64 inputs; with zero_g the gradient is
// cleared after use.
__global__ void k_adam(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, __nv_bfloat16* __restrict__ pb, int64_t n, float lr, float c1,
                       float c2, __nv_bfloat16* __restrict__ w1p, int n_in, int64_t n_w1, bool zero_g) {
  tc::grid_dependency_wait();
  tc::launch_dependents();
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    float const gq = g[q];
    if (zero_g) g[q] = 0.0f;  // the next step's gradient accumulates from zero
    float const mq = 0.9f * m[q] + 0.1f * gq;
    float const vq = 0.999f * v[q] + 0.001f * gq * gq;
    m[q] = mq;
    v[q] = vq;
    float const pq = p[q] - lr * (mq * c1) / (sqrtf(vq * c2) + 1e-8f);
    p[q] = pq;
    pb[q] = __float2bfloat16(pq);
    if (w1p && q < n_w1) w1p[(q / n_in) * 64 + q % n_in] = __float2bfloat16(pq);
  }
}

// ------------------------------------------- tensor-core training step ---
// One batch of rows [0, n): X (BF16 spins, 64 columns, zero past n_in) ->
// h1 = bf16(tanh(X W1^T + b1)) -> h2 = bf16(tanh(h1 W2^T + b2)) on the
// tensor cores (tc_gemm); k_head evaluates (a, s) = W3 h2 + b3, the loss and
// g2 = bf16((dout W3) (1 - h2^2)); the tensor cores then give
// g1 = bf16((g2 W2) (1 - h1^2)) with db1 in its epilogue, dW2 = g2^T h1 and
// dW1 = g1^T X (K = the batch, read M-/N-major). The column sums db2, db1
// add the unrounded values. Batches are drawn in the order of a keyed
// permutation of the samples, made on the device once per epoch.

// W1 (FP32, hidden x n_in) -> BF16 rows of 64, zero padded
__global__ void k_w1_pad(float const* __restrict__ w1, int n_in, int hidden, __nv_bfloat16* __restrict__ w1p) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < hidden * 64; q += gridDim.x * blockDim.x) {
    int const r = q / 64, c = q % 64;
    w1p[q] = __float2bfloat16(c < n_in ? w1[r * n_in + c] : 0.0f);
  }
}

__device__ __forceinline__ uint32_t mix32(uint32_t x) {  // the "lowbias32" integer hash (C. Wellons)
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// perm[j] = pi(j) for j < n: a four-round Feistel network on 2 half bits
// (the smallest even width covering n), keyed by key0..3, walked along its
// cycles until the value falls below n; a bijection of [0, n).
__global__ void k_perm(uint32_t n, int half, uint4 key, uint32_t* __restrict__ perm) {
  uint32_t const mask = (1u << half) - 1u;
  uint32_t const keys[4] = {key.x, key.y, key.z, key.w};
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    uint32_t x = j;
    do {
      uint32_t l = x >> half, r = x & mask;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        uint32_t const nr = l ^ (mix32(r ^ keys[k]) & mask);
        l = r;
        r = nr;
      }
      x = (l << half) | r;
    } while (x >= n);
    perm[j] = x;
  }
}

// Batch rows r < rows from samples perm[b0 + r] (b0 + r without perm): the
// X row (64 BF16 spins, zero past n_in; eight threads per row, 16 bytes
// each) and the row's state and targets.
__global__ void k_batch(uint64_t const* __restrict__ states, float const* __restrict__ t_abs,
                        float const* __restrict__ t_sign, uint32_t const* __restrict__ perm, uint64_t b0,
                        int64_t rows, int n_in, __nv_bfloat16* __restrict__ X, uint64_t* __restrict__ bst,
                        float* __restrict__ bta, float* __restrict__ bts) {
  tc::grid_dependency_wait();  // the previous step still reads X and the batch arrays
  tc::launch_dependents();
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < rows * 8; q += (int64_t)gridDim.x * blockDim.x) {
    int64_t const r = q >> 3;
    int const c = (int)(q & 7);
    uint64_t const idx = perm ? perm[b0 + r] : b0 + r;
    uint64_t const s = states[idx];
    uint32_t w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      int const j = 8 * c + 2 * k;
      uint32_t const lo = j < n_in ? (((s >> j) & 1u) ? 0x3F80u : 0xBF80u) : 0u;
      uint32_t const hi = j + 1 < n_in ? (((s >> (j + 1)) & 1u) ? 0x3F80u : 0xBF80u) : 0u;
      w[k] = lo | (hi << 16);
    }
    reinterpret_cast<uint4*>(X + r * 64)[c] = make_uint4(w[0], w[1], w[2], w[3]);
    if (c == 0) {
      bst[r] = s;
      bta[r] = t_abs[idx];
      bts[r] = t_sign[idx];
    }
  }
}

constexpr int kHeadChunks = 2;  // 8-column chunks per lane: hidden <= 512
constexpr int kHeadRows = 4;    // rows whose loads a warp issues together

// This block's sums of (db2, dW3 row 0, dW3 row 1, db3) into
// part[blockIdx.x][3H + 2]: each warp puts its lanes' columns (and lane 0's
// db3 terms) in shared memory, then the warps' values are added in warp
// order, so the result does not depend on timing (no atomics).
__device__ __forceinline__ void head_block_partial(float const (&ab)[kHeadChunks][8], float const (&a0)[kHeadChunks][8],
                                                   float const (&a1)[kHeadChunks][8], float sd0, float sd1, int H,
                                                   float* smem, float* __restrict__ part) {
  int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31, chunks = H / 8, W = 3 * H + 2;
  int const nw = blockDim.x >> 5;
  float* const mine = smem + warp * W;
#pragma unroll
  for (int q = 0; q < kHeadChunks; ++q) {
    int const ch = lane + 32 * q;
    if (ch >= chunks) continue;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      mine[8 * ch + j] = ab[q][j];
      mine[H + 8 * ch + j] = a0[q][j];
      mine[2 * H + 8 * ch + j] = a1[q][j];
    }
  }
  if (lane == 0) {
    mine[3 * H] = sd0;
    mine[3 * H + 1] = sd1;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < W; c += blockDim.x) {
    float t = 0.0f;
    for (int w = 0; w < nw; ++w) t += smem[w * W + c];
    part[(int64_t)blockIdx.x * W + c] = t;
  }
}

// The step's gradient from its partial sums, each added in a fixed order:
// W1 and W2 from the K-split slabs of their GEMMs (s1, s2 slabs), b2, W3 and
// b3 from the output-layer blocks' rows (nhb rows of 3H + 2); b1 is left to
// k_column_sums.
__global__ void k_grad_rest(float* __restrict__ g, int n_in, int H, float const* __restrict__ w1part, int s1,
                            float const* __restrict__ w2part, int s2, float const* __restrict__ hpart, int nhb) {
  tc::grid_dependency_wait();
  tc::launch_dependents();
  int64_t const nW1 = (int64_t)H * n_in, ob1 = nW1, oW2 = ob1 + H, ob2 = oW2 + (int64_t)H * H, oW3 = ob2 + H,
                ob3 = oW3 + 2 * H, n = ob3 + 2;
  int const W = 3 * H + 2;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    if (q >= ob1 && q < oW2) continue;  // b1: k_column_sums
    float t = 0.0f;
    if (q < nW1) {
      for (int z = 0; z < s1; ++z) t += w1part[(int64_t)z * nW1 + q];
    } else if (q < ob2) {
      int64_t const e = q - oW2;
      for (int z = 0; z < s2; ++z) t += w2part[(int64_t)z * H * H + e];
    } else {
      int const c = q < oW3 ? (int)(q - ob2) : q < ob3 ? H + (int)(q - oW3) : 3 * H + (int)(q - ob3);
      for (int b = 0; b < nhb; ++b) t += hpart[(int64_t)b * W + c];
    }
    g[q] = t;
  }
}

// out[i] = sum over p < np of a[p][i] (a: np rows of `ld`, one block per
// column i): strided partial sums added in a fixed tree order, so the result
// does not depend on timing. Used for b1 from the g1 GEMM's partial column
// sums and for the CUDA-core path's bias gradients.
__global__ void __launch_bounds__(256) k_column_sums(float* __restrict__ out, float const* __restrict__ a, int64_t np,
                                                     int ld) {
  __shared__ float red[8];
  tc::grid_dependency_wait();
  tc::launch_dependents();
  int const i = blockIdx.x;
  float t = 0.0f;
  for (int64_t p = threadIdx.x; p < np; p += blockDim.x) t += a[p * ld + i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    float u = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) u += red[w];
    out[i] = u;
  }
}

// Shared memory of the output-layer kernels: one row of partial sums per warp.
size_t head_smem_bytes(int H) { return (size_t)8 * (3 * H + 2) * 4; }

// Patch network (sed_mlp_create_patch): X row b N + i holds the P spins of
// site i's patch (patch[i][0..P)) of sample b, zero past P; eight threads
// per row, 16 bytes each; thread (row b N, chunk 0) also copies sample b's
// state and targets (t_abs / t_sign may be null: inference).
__global__ void k_batch_patch(uint64_t const* __restrict__ states, float const* __restrict__ t_abs,
                              float const* __restrict__ t_sign, uint32_t const* __restrict__ perm, uint64_t b0,
                              int64_t samples, int n_sites, int P, uint16_t const* __restrict__ patch,
                              __nv_bfloat16* __restrict__ X, uint64_t* __restrict__ bst, float* __restrict__ bta,
                              float* __restrict__ bts) {
  tc::grid_dependency_wait();
  tc::launch_dependents();
  int64_t const rows = samples * n_sites;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < rows * 8; q += (int64_t)gridDim.x * blockDim.x) {
    int64_t const r = q >> 3;
    int const c = (int)(q & 7);
    int64_t const b = r / n_sites;
    int const site = (int)(r - b * n_sites);
    uint64_t const idx = perm ? perm[b0 + b] : b0 + b;
    uint64_t const s = states[idx];
    uint16_t const* const ps = patch + (int64_t)site * P;
    uint32_t w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      int const j = 8 * c + 2 * k;
      uint32_t const lo = j < P ? (((s >> ps[j]) & 1u) ? 0x3F80u : 0xBF80u) : 0u;
      uint32_t const hi = j + 1 < P ? (((s >> ps[j + 1]) & 1u) ? 0x3F80u : 0xBF80u) : 0u;
      w[k] = lo | (hi << 16);
    }
    reinterpret_cast<uint4*>(X + r * 64)[c] = make_uint4(w[0], w[1], w[2], w[3]);
    if (site == 0 && c == 0) {
      bst[b] = s;
      if (t_abs) bta[b] = t_abs[idx];
      if (t_sign) bts[b] = t_sign[idx];
    }
  }
}

// Patch network output layer for samples [0, n), one warp per sample over
// its n_sites rows of h2 (rows b N .. b N + N - 1; lane l holds the 8-column
// chunks l and l + 32): hs = sum over the sites of h2, (a, s) = W3 hs + b3.
// With `out` set only (a, s) are written (inference). Otherwise the output
// gradient as in k_head, g2 = (dout W3) (1 - h2^2) for every site row (BF16),
// the block's partial sums of db2 (unrounded g2), dW3 = dout^T hs and db3
// (head_block_partial) and its loss partial.
__global__ void __launch_bounds__(256)
    k_head_patch(__nv_bfloat16 const* __restrict__ h2, int H, int n_sites, int64_t n,
                 __nv_bfloat16 const* __restrict__ W3, float const* __restrict__ b3,
                 uint64_t const* __restrict__ bst, float const* __restrict__ bta, float const* __restrict__ bts,
                 uint64_t sign_mask, __nv_bfloat16* __restrict__ g2, float* __restrict__ part,
                 double* __restrict__ loss_partial, float* __restrict__ out) {
  extern __shared__ float sacc[];  // [warps][3H + 2] (training only)
  __shared__ double red[32];
  bool const train = out == nullptr;
  tc::grid_dependency_wait();
  tc::launch_dependents();
  int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31, chunks = H / 8;
  float w0[kHeadChunks][8], w1[kHeadChunks][8], ab[kHeadChunks][8], a0[kHeadChunks][8], a1[kHeadChunks][8];
#pragma unroll
  for (int q = 0; q < kHeadChunks; ++q) {
    int const ch = lane + 32 * q;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      w0[q][j] = ch < chunks ? __bfloat162float(W3[8 * ch + j]) : 0.0f;
      w1[q][j] = ch < chunks ? __bfloat162float(W3[H + 8 * ch + j]) : 0.0f;
      ab[q][j] = a0[q][j] = a1[q][j] = 0.0f;
    }
  }
  float const b30 = b3[0], b31 = b3[1], inv_n = 1.0f / (float)n;
  float sd0 = 0.0f, sd1 = 0.0f;
  double l = 0.0;
  auto load_row = [&](int64_t row, float (&h)[kHeadChunks][8]) {
#pragma unroll
    for (int q = 0; q < kHeadChunks; ++q) {
      int const ch = lane + 32 * q;
      uint4 const u = ch < chunks ? reinterpret_cast<uint4 const*>(h2 + row * H)[ch] : make_uint4(0, 0, 0, 0);
      uint32_t const wv[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        h[q][2 * k] = __uint_as_float(wv[k] << 16);
        h[q][2 * k + 1] = __uint_as_float(wv[k] & 0xFFFF0000u);
      }
    }
  };
  int64_t const nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t b = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp; b < n; b += nw) {
    float hs[kHeadChunks][8] = {};
    int64_t const r0 = b * n_sites;
    for (int i = 0; i < n_sites; ++i) {
      float h[kHeadChunks][8];
      load_row(r0 + i, h);
#pragma unroll
      for (int q = 0; q < kHeadChunks; ++q)
#pragma unroll
        for (int j = 0; j < 8; ++j) hs[q][j] += h[q][j];
    }
    float pa = 0.0f, ps = 0.0f;
#pragma unroll
    for (int q = 0; q < kHeadChunks; ++q)
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        pa = fmaf(w0[q][j], hs[q][j], pa);
        ps = fmaf(w1[q][j], hs[q][j], ps);
      }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      pa += __shfl_xor_sync(0xffffffffu, pa, o);
      ps += __shfl_xor_sync(0xffffffffu, ps, o);
    }
    float const a = pa + b30, s = ps + b31;
    if (!train) {
      if (lane == 0) {
        out[2 * b] = a;
        out[2 * b + 1] = s;
      }
      continue;
    }
    float const da = a - bta[b];
    float const y = fabsf(bts[b] - prior_flip(bst[b], sign_mask));
    float const pr = 1.0f / (1.0f + expf(-s));
    float const d0 = 2.0f * da * inv_n, d1 = (pr - y) * inv_n;
    if (lane == 0) {
      l += (double)da * da + (double)(fmaxf(s, 0.0f) - s * y + log1pf(expf(-fabsf(s))));
      sd0 += d0;
      sd1 += d1;
    }
#pragma unroll
    for (int q = 0; q < kHeadChunks; ++q)
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        a0[q][j] = fmaf(d0, hs[q][j], a0[q][j]);
        a1[q][j] = fmaf(d1, hs[q][j], a1[q][j]);
      }
    for (int i = 0; i < n_sites; ++i) {
      float h[kHeadChunks][8];
      load_row(r0 + i, h);
#pragma unroll
      for (int q = 0; q < kHeadChunks; ++q) {
        int const ch = lane + 32 * q;
        if (ch >= chunks) continue;
        uint32_t pk[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          float g[2];
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            int const j = 2 * k + e;
            g[e] = (d0 * w0[q][j] + d1 * w1[q][j]) * (1.0f - h[q][j] * h[q][j]);
            ab[q][j] += g[e];
          }
          pk[k] = tc::pack_bf16x2(g[0], g[1]);
        }
        reinterpret_cast<uint4*>(g2 + (r0 + i) * H)[ch] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
  }
  if (!train) return;
  double const tot = block_sum(l, red);
  if (threadIdx.x == 0) loss_partial[blockIdx.x] = tot;
  head_block_partial(ab, a0, a1, sd0, sd1, H, sacc, part);
}

// Output layer, loss and first backward step for rows [0, n): one warp per
// row, lane l holding the 8-column chunks l and l + 32 of h2. Per row
// (a, s) = W3 h2 + b3 (warp sums), the output gradient as in k_out_grad,
// g2 = (dout W3) (1 - h2^2) written as BF16; the block's partial sums of g2
// (db2), of dout_c h2 (dW3) and of dout (db3) into part (head_block_partial);
// the loss partial of the block into loss_partial.
__global__ void __launch_bounds__(256)
    k_head(__nv_bfloat16 const* __restrict__ h2, int H, int64_t n, __nv_bfloat16 const* __restrict__ W3,
           float const* __restrict__ b3, uint64_t const* __restrict__ bst, float const* __restrict__ bta,
           float const* __restrict__ bts, uint64_t sign_mask, __nv_bfloat16* __restrict__ g2,
           float* __restrict__ part, double* __restrict__ loss_partial) {
  extern __shared__ float sacc[];  // [warps][3H + 2]
  __shared__ double red[32];
  tc::grid_dependency_wait();
  tc::launch_dependents();
  int const warp = threadIdx.x >> 5, lane = threadIdx.x & 31, chunks = H / 8;
  float w0[kHeadChunks][8], w1[kHeadChunks][8], ab[kHeadChunks][8], a0[kHeadChunks][8], a1[kHeadChunks][8];
#pragma unroll
  for (int q = 0; q < kHeadChunks; ++q) {
    int const ch = lane + 32 * q;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      w0[q][j] = ch < chunks ? __bfloat162float(W3[8 * ch + j]) : 0.0f;
      w1[q][j] = ch < chunks ? __bfloat162float(W3[H + 8 * ch + j]) : 0.0f;
      ab[q][j] = a0[q][j] = a1[q][j] = 0.0f;
    }
  }
  float const b30 = b3[0], b31 = b3[1], inv_n = 1.0f / (float)n;
  float sd0 = 0.0f, sd1 = 0.0f;
  double l = 0.0;
  // warp w takes groups of kHeadRows consecutive rows; each group's loads are
  // all issued before its arithmetic
  int64_t const nw = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r0 = ((int64_t)blockIdx.x * (blockDim.x >> 5) + warp) * kHeadRows; r0 < n; r0 += nw * kHeadRows) {
    uint4 u[kHeadRows][kHeadChunks];
    float ta[kHeadRows], ts[kHeadRows];
    uint64_t sv[kHeadRows];
#pragma unroll
    for (int i = 0; i < kHeadRows; ++i) {
      int64_t const r = r0 + i;
      bool const row_ok = r < n;
#pragma unroll
      for (int q = 0; q < kHeadChunks; ++q) {
        int const ch = lane + 32 * q;
        u[i][q] = (row_ok && ch < chunks) ? reinterpret_cast<uint4 const*>(h2 + r * H)[ch] : make_uint4(0, 0, 0, 0);
      }
      ta[i] = row_ok ? bta[r] : 0.0f;
      ts[i] = row_ok ? bts[r] : 0.0f;
      sv[i] = row_ok ? bst[r] : 0;
    }
#pragma unroll
    for (int i = 0; i < kHeadRows; ++i) {
      int64_t const r = r0 + i;
      if (r >= n) break;  // warp-uniform
      float h[kHeadChunks][8];
      float pa = 0.0f, ps = 0.0f;
#pragma unroll
      for (int q = 0; q < kHeadChunks; ++q) {
        uint32_t const wv[4] = {u[i][q].x, u[i][q].y, u[i][q].z, u[i][q].w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          h[q][2 * k] = __uint_as_float(wv[k] << 16);
          h[q][2 * k + 1] = __uint_as_float(wv[k] & 0xFFFF0000u);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          pa = fmaf(w0[q][j], h[q][j], pa);
          ps = fmaf(w1[q][j], h[q][j], ps);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        pa += __shfl_xor_sync(0xffffffffu, pa, o);
        ps += __shfl_xor_sync(0xffffffffu, ps, o);
      }
      float const a = pa + b30, s = ps + b31;
      float const da = a - ta[i];
      float const y = fabsf(ts[i] - prior_flip(sv[i], sign_mask));
      float const pr = 1.0f / (1.0f + expf(-s));
      float const d0 = 2.0f * da * inv_n, d1 = (pr - y) * inv_n;
      if (lane == 0) {
        l += (double)da * da + (double)(fmaxf(s, 0.0f) - s * y + log1pf(expf(-fabsf(s))));
        sd0 += d0;
        sd1 += d1;
      }
#pragma unroll
      for (int q = 0; q < kHeadChunks; ++q) {
        int const ch = lane + 32 * q;
        if (ch >= chunks) continue;
        uint32_t pk[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          float g[2];
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            int const j = 2 * k + e;
            g[e] = (d0 * w0[q][j] + d1 * w1[q][j]) * (1.0f - h[q][j] * h[q][j]);
            ab[q][j] += g[e];
            a0[q][j] = fmaf(d0, h[q][j], a0[q][j]);
            a1[q][j] = fmaf(d1, h[q][j], a1[q][j]);
          }
          pk[k] = tc::pack_bf16x2(g[0], g[1]);
        }
        reinterpret_cast<uint4*>(g2 + r * H)[ch] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
  }
  double const tot = block_sum(l, red);  // contains a __syncthreads
  if (threadIdx.x == 0) loss_partial[blockIdx.x] = tot;
  head_block_partial(ab, a0, a1, sd0, sd1, H, sacc, part);
}

__global__ void k_to_bf16(float const* __restrict__ p, __nv_bfloat16* __restrict__ pb, int64_t n) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    pb[q] = __float2bfloat16(p[q]);
}

// v_r = prior(r) sign(s) exp(a - a_max) / n_r, n_r = sqrt(S_r / |G|)
__global__ void k_start_from_net(float const* __restrict__ out, uint64_t const* __restrict__ reps,
                                 uint32_t const* __restrict__ weights, int64_t n, uint64_t sign_mask,
                                 float a_max, double group_order, double* __restrict__ v) {
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < n; b += (int64_t)gridDim.x * blockDim.x) {
    float const a = out[2 * b], s = out[2 * b + 1];
    double const amp = exp((double)(a - a_max)) * sqrt(group_order / (double)weights[b]);
    bool const neg = (s < 0.0f) != (prior_flip(reps[b], sign_mask) != 0.0f);
    v[b] = neg ? -amp : amp;
  }
}

__global__ void k_max_first(float const* __restrict__ out, int64_t n, float* __restrict__ part) {
  __shared__ float red[256];
  float m = -3.0e38f;
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < n; b += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, out[2 * b]);
  red[threadIdx.x] = m;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// ------------------------------------------------------------- sampling ---
constexpr int kChunk = 4096;  // elements per block of the prefix sum (256 threads x 16)

// Per chunk: sum of psi^2 and of prior(r) psi_r |psi_r| (the weight with which
// psi agrees with the sign prior, used to fix psi's global sign).
__global__ void k_chunk_sums(double const* __restrict__ psi, uint64_t const* __restrict__ reps, uint64_t D,
                             uint64_t sign_mask, double* __restrict__ sums) {
  __shared__ double red[32];
  uint64_t const base = (uint64_t)blockIdx.x * kChunk;
  double s = 0.0, a = 0.0;
  for (int q = threadIdx.x; q < kChunk; q += blockDim.x) {
    uint64_t const i = base + q;
    if (i < D) {
      double const w = psi[i] * psi[i];
      s += w;
      bool const neg = (psi[i] < 0.0) != (prior_flip(reps[i], sign_mask) != 0.0f);
      a += neg ? -w : w;
    }
  }
  double const t = block_sum(s, red);
  double const u = block_sum(a, red);
  if (threadIdx.x == 0) {
    sums[blockIdx.x] = t;
    sums[gridDim.x + blockIdx.x] = u;
  }
}

// prefix[i] = offset[chunk] + sum_{j <= i in chunk} psi_j^2
__global__ void __launch_bounds__(256) k_chunk_prefix(double const* __restrict__ psi, uint64_t D,
                                                       double const* __restrict__ offset,
                                                       double* __restrict__ prefix) {
  __shared__ double part[256];
  uint64_t const base = (uint64_t)blockIdx.x * kChunk + threadIdx.x * 16;
  double v[16];
  double run = 0.0;
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    uint64_t const i = base + q;
    double const p = i < D ? psi[i] : 0.0;
    run += p * p;
    v[q] = run;
  }
  part[threadIdx.x] = run;
  __syncthreads();
  for (int o = 1; o < 256; o <<= 1) {  // Hillis-Steele inclusive scan of the thread totals
    double const t = (int)threadIdx.x >= o ? part[threadIdx.x - o] : 0.0;
    __syncthreads();
    part[threadIdx.x] += t;
    __syncthreads();
  }
  double const before = offset[blockIdx.x] + (threadIdx.x ? part[threadIdx.x - 1] : 0.0);
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    uint64_t const i = base + q;
    if (i < D) prefix[i] = before + v[q];
  }
}

// Sample q: u = total * U[0,1) from Philox block (q, seed); its index is the
// smallest i with prefix[i] > u.
__global__ void k_draw(double const* __restrict__ prefix, uint64_t D, double total, uint64_t n, uint64_t seed,
                       double sign, double const* __restrict__ psi, uint64_t const* __restrict__ reps,
                       uint32_t const* __restrict__ weights, double group_order, uint64_t* __restrict__ states,
                       float* __restrict__ t_abs, float* __restrict__ t_sign) {
  for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t c[4] = {(uint32_t)q, (uint32_t)(q >> 32), 0x5EEDu, 0u};
    philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    double const u = u01_53(c[0], c[1]) * total;
    uint64_t lo = 0, hi = D - 1;
    while (lo < hi) {
      uint64_t const mid = lo + (hi - lo) / 2;
      if (prefix[mid] > u)
        hi = mid;
      else
        lo = mid + 1;
    }
    double const p = sign * psi[lo];
    states[q] = reps[lo];
    t_abs[q] = (float)(log(fabs(p)) + 0.5 * log((double)weights[lo] / group_order));
    t_sign[q] = p > 0.0 ? 1.0f : 0.0f;
  }
}

unsigned blocks_for(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

// ------------------------------------------------ tensor-core inference ---
// The whole network for tiles of 128 states on the 5th-generation tensor
// cores, for n <= 64 inputs and hidden H = 128, 256 or 512:
//   X [128 x 64] (spins built in shared memory from the state bits, zero
//   padded), h1 = tanh(X W1^T + b1) -> TMEM (FP32) -> BF16 back into TMEM,
//   h2 = tanh(h1 W2^T + b2) -> TMEM, (a, s) = W3 h2 + b3 in registers.
// Persistent: one CTA per SM walks the tiles blockIdx.x, + gridDim.x, ...
// TMEM (512 columns): two accumulator slots of 128 columns (0-127, 128-255)
// and h1 as the A operand of layer 2 (columns 256 .. 256 + H/2, two BF16 per
// column). Both layers produce their output 128 columns at a time, cycling
// through the two slots, so the epilogue of one block overlaps the MMAs of
// the next. Keeping h1 out of shared memory leaves room for a deep ring of
// weight stages: the weights (pre-swizzled images in global memory, a few
// hundred KB, L2-resident) are re-read for every tile, and the copies in
// flight must cover the L2 latency.
constexpr int kTcRows = 128;
constexpr int kTcEpiWarps = 16;                    // 4 per TMEM lane quarter
constexpr int kTcThreads = (kTcEpiWarps + 2) * 32;  // + one copy warp + one MMA warp
constexpr int kTcTileBytes = 128 * 128;             // one weight K tile: 128 rows x 64 BF16, swizzled
constexpr int kTcJobTiles = 4;                      // K tiles per layer-2 job (one ring stage)
constexpr int kTcMaxStages = 8;                     // ring of weight stages of kTcJobTiles K tiles each
constexpr int kTcMaxBlocks = 4;                     // H / 128
constexpr uint32_t kTcCols = 512;                   // TMEM columns per CTA
constexpr uint32_t kTcH1Col = 256;                  // first TMEM column of h1
constexpr uint64_t kTcWaitNs = 1000000000ull;       // default: 1 s per wait, far beyond any MMA or copy
constexpr size_t kTcSmemLimit = 232448 - 1024;      // opt-in shared memory per CTA, less the static part

struct MlpTcArgs {
  uint64_t const* states;
  int64_t n;
  int n_in, hidden, stages;
  uint8_t const* w1img;  // hidden rows x 128 B (K = 64, zero padded), swizzled
  uint8_t const* w2img;  // hidden/64 tiles of hidden rows x 128 B, swizzled
  float const* b1;
  float const* b2;
  __nv_bfloat16 const* W3;  // [2][hidden]
  float const* b3;
  float* out;  // [n][2]; for a patch network [n / n_sites][2], zeroed before the launch
  int* error;
  uint64_t wait_ns;  // bound on every mbarrier wait
  // patch network: n = samples x n_sites rows, row b n_sites + i is site i's
  // patch of states[b] (patch[i * n_in + j] = the site of input j), and the
  // rows' outputs add into out[b] (b3 once, with site 0)
  uint16_t const* patch = nullptr;
  int n_sites = 0;
};

// dynamic shared memory: the X tile, b1, b2, W3 (FP32), two buffers of
// per-warp partial sums, then the weight ring with as many stages as fit
size_t tc_fixed_bytes(int hidden) {
  return (size_t)kTcRows * 128 + 4 * (size_t)hidden * 4 + 2 * (size_t)4 * kTcRows * 2 * 4 + 1024;
}
int tc_job_tiles(int hidden) { return std::min(kTcJobTiles, hidden / 64); }
int tc_stages(int hidden) {
  return (int)std::min<size_t>(kTcMaxStages, (kTcSmemLimit - tc_fixed_bytes(hidden)) /
                                                  ((size_t)tc_job_tiles(hidden) * kTcTileBytes));
}
size_t tc_smem_bytes(int hidden) {
  return tc_fixed_bytes(hidden) + (size_t)tc_stages(hidden) * tc_job_tiles(hidden) * kTcTileBytes;
}

__device__ __forceinline__ void epi_sync() {  // the 512 epilogue threads only
  asm volatile("bar.sync 1, %0;" ::"r"(kTcEpiWarps * 32) : "memory");
}

// Input word of row t % 128 of `tile` (0 past n), read by epilogue thread
// t: the state itself, or for a patch network the row's patch gathered into
// bits 0 .. n_in - 1.
__device__ __forceinline__ uint64_t tc_state(MlpTcArgs const& p, int64_t tile, int t) {
  int64_t const xrow = tile * kTcRows + (t & 127);
  if (xrow >= p.n) return 0;
  if (!p.n_sites) return p.states[xrow];
  int64_t const b = xrow / p.n_sites;
  int const site = (int)(xrow - b * p.n_sites);
  uint64_t const s = p.states[b];
  uint16_t const* const ps = p.patch + (int64_t)site * p.n_in;
  uint64_t x = 0;
  for (int j = 0; j < p.n_in; ++j) x |= ((s >> __ldg(ps + j)) & 1ull) << j;
  return x;
}

// X tile row t % 128 from its state s: input j -> BF16 +1 / -1, zero for
// j >= n_in; four threads per row, two 16-byte chunks each. Called by the
// 512 epilogue threads.
__device__ __forceinline__ void tc_build_x(MlpTcArgs const& p, uint64_t s, uint8_t* X, int t) {
  int const xr = t & 127, part = t >> 7;
#pragma unroll
  for (int cc = 0; cc < 2; ++cc) {
    int const c = 2 * part + cc;
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int const j = 8 * c + 2 * q;
      uint32_t const lo = j < p.n_in ? (((s >> j) & 1) ? 0x3F80u : 0xBF80u) : 0u;
      uint32_t const hi = j + 1 < p.n_in ? (((s >> (j + 1)) & 1) ? 0x3F80u : 0xBF80u) : 0u;
      w[q] = lo | (hi << 16);
    }
    *reinterpret_cast<uint4*>(X + xr * 128 + ((c ^ (xr & 7)) << 4)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// Warp-specialised: warp 16 streams the weights through the ring (waiting
// only for a stage's previous MMAs to finish), warp 17 issues the MMAs,
// warps 0-15 run the epilogues and build the X tiles. Per tile the weight
// stream is H/128 jobs of W1 (row block q, K = 64) followed by the W2 jobs
// (row block q, K tile kb) in q-major order; global job g lives in stage
// g % stages. Accumulator uses are numbered u = 0, 1, ... over the layer-1
// and layer-2 blocks of all tiles in order; use u takes slot u % 2.
// Barriers: acc_full (MMAs of a use done; committed by the MMA warp),
// acc_empty (the epilogue has read the slot), h1_ready (block q of h1 is in
// TMEM), x_ready (the X tile is in shared memory); the last three get one
// arrival per epilogue warp.
__global__ void __launch_bounds__(kTcThreads, 1) k_mlp_forward_tc(MlpTcArgs p) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[kTcMaxStages], empty[kTcMaxStages];
  __shared__ uint64_t acc_full[2], acc_empty[2], h1_ready[kTcMaxBlocks];
  __shared__ uint64_t x_ready, drain;
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  uint8_t* const smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  int const H = p.hidden, NM = 128, blocks = H / NM, ktiles = H / 64, S = p.stages;
  int const JT = min(kTcJobTiles, ktiles), kjobs = ktiles / JT;  // K tiles per layer-2 job, jobs per block
  uint32_t const stage_bytes = (uint32_t)(JT * kTcTileBytes);
  uint8_t* const X = smem;  // 128 rows x 128 B
  uint8_t* const B0 = X + (size_t)kTcRows * 128;
  float* const sb1 = reinterpret_cast<float*>(B0 + (size_t)S * stage_bytes);
  float* const sb2 = sb1 + H;
  float* const sw3 = sb2 + H;        // [2][H]
  float* const spart = sw3 + 2 * H;  // [2 buffers][4 column slices][128 rows][2]
  int const t = threadIdx.x, warp = t >> 5, lane = t & 31;
  int64_t const n_tiles = (p.n + kTcRows - 1) / kTcRows;
  int const my_tiles = blockIdx.x < n_tiles ? (int)((n_tiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  int const jobs_per_tile = blocks + kjobs * blocks;

  if (t == 0) {
    for (int i = 0; i < S; ++i) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&acc_full[i], 1);
      tc::mbar_init(&acc_empty[i], kTcEpiWarps);
    }
    for (int q = 0; q < kTcMaxBlocks; ++q) tc::mbar_init(&h1_ready[q], kTcEpiWarps);
    tc::mbar_init(&x_ready, kTcEpiWarps);
    tc::mbar_init(&drain, 1);
    abort_flag = 0;
    tc::fence_mbar_init();
  }
  __syncwarp();
  if (warp == 0) tc::tmem_alloc(&tmem_slot, kTcCols);
  for (int c = t; c < H; c += kTcThreads) {
    sb1[c] = __ldg(p.b1 + c);
    sb2[c] = __ldg(p.b2 + c);
    sw3[c] = __bfloat162float(p.W3[c]);
    sw3[H + c] = __bfloat162float(p.W3[H + c]);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  uint32_t const tmem = tmem_slot;

  if (warp == kTcEpiWarps) {
    // ---- copy warp: keep the ring full (stage st, its use count `use`)
    if (lane == 0) {
      int64_t const total = (int64_t)my_tiles * jobs_per_tile;
      int64_t g = 0;
      int st = 0, u = 0;
      uint32_t use = 0;
      for (; g < total; ++g) {
        if (use > 0 && !tc::mbar_wait(&empty[st], (use - 1) & 1, p.wait_ns)) {
          abort_flag = 1;
          break;
        }
        uint8_t* const dst = B0 + (size_t)st * stage_bytes;
        if (u < blocks) {  // W1 row block u (K = 64)
          tc::mbar_expect_tx(&full[st], kTcTileBytes);
          tc::bulk_g2s(dst, p.w1img + (size_t)u * kTcTileBytes, kTcTileBytes, &full[st]);
        } else {  // W2 row block q, K tiles kg JT .. kg JT + JT - 1
          int const v = u - blocks, q = v / kjobs, kg = v % kjobs;
          tc::mbar_expect_tx(&full[st], stage_bytes);
          for (int i = 0; i < JT; ++i)
            tc::bulk_g2s(dst + (size_t)i * kTcTileBytes, p.w2img + ((size_t)(kg * JT + i) * H + (size_t)q * NM) * 128,
                         kTcTileBytes, &full[st]);
        }
        if (++u == jobs_per_tile) u = 0;
        if (++st == S) {
          st = 0;
          ++use;
        }
      }
      // never leave with copies in flight: wait for the last stages to land
      for (int64_t h = g > S ? g - S : 0; h < g; ++h)
        if (!tc::mbar_wait(&full[h % S], (uint32_t)(h / S) & 1, p.wait_ns)) abort_flag = 1;
    }
    __syncwarp();
  } else if (warp == kTcEpiWarps + 1) {
    // ---- MMA warp: the whole warp runs the loop, so that stage addresses
    // and descriptors are warp-uniform; one elected lane issues the MMAs
    // and commits.
    uint32_t const idesc = tc::idesc_bf16_f32(128, (uint32_t)NM);
    bool ok = true;
    int st = 0;          // ring stage of the next job
    uint32_t sph = 0;    // parity of that stage's current use
    int64_t u = 0;       // accumulator use
    auto take = [&]() {  // wait for the next job's stage to land
      bool const r = tc::mbar_wait(&full[st], sph, p.wait_ns);
      tc::fence_after_sync();
      return __all_sync(0xffffffffu, r);
    };
    auto release = [&](bool leader) {  // the stage is free once the MMAs issued so far have read it
      if (leader) tc::mma_commit(&empty[st]);
      if (++st == S) {
        st = 0;
        sph ^= 1u;
      }
    };
    auto slot_free = [&](int64_t uu) {  // the epilogue has drained use uu - 2 of the slot
      bool const r = uu < 2 || tc::mbar_wait(&acc_empty[uu & 1], (uint32_t)((uu >> 1) - 1) & 1, p.wait_ns);
      tc::fence_after_sync();
      return __all_sync(0xffffffffu, r);
    };
    for (int it = 0; it < my_tiles && ok; ++it) {
      uint32_t const par = (uint32_t)it & 1;
      ok = __all_sync(0xffffffffu, tc::mbar_wait(&x_ready, par, p.wait_ns) && !abort_flag);
      tc::fence_after_sync();
      // layer 1: block q of X W1^T
      for (int q = 0; q < blocks && ok; ++q, ++u) {
        ok = slot_free(u) && take();
        if (!ok) break;
        uint32_t const d = tmem + (uint32_t)((u & 1) * NM);
        uint32_t const at = tc::smem_u32(X), b0 = tc::smem_u32(B0 + (size_t)st * stage_bytes);
        bool const leader = tc::elect_one();
        if (leader) {
#pragma unroll
          for (int k = 0; k < 4; ++k)
            tc::mma_bf16(d, tc::desc_sw128(at + 32 * k), tc::desc_sw128(b0 + 32 * k), idesc, k > 0 ? 1u : 0u);
        }
        release(leader);
        if (leader) tc::mma_commit(&acc_full[u & 1]);
        __syncwarp();
      }
      // layer 2: block q of h1 W2^T over all K tiles, h1 read from TMEM
      for (int q = 0; q < blocks && ok; ++q, ++u) {
        ok = slot_free(u);
        uint32_t const d = tmem + (uint32_t)((u & 1) * NM);
        for (int kg = 0; kg < kjobs && ok; ++kg) {
          // K tiles kb = kg JT .. + JT - 1; h1 block b holds K tiles 2 b, 2 b + 1
          for (int b = (kg * JT) >> 1; q == 0 && ok && b <= (kg * JT + JT - 1) >> 1; ++b) {
            ok = __all_sync(0xffffffffu, tc::mbar_wait(&h1_ready[b], par, p.wait_ns) && !abort_flag);
            tc::fence_after_sync();
          }
          if (ok) ok = take();
          if (!ok) break;
          uint32_t const b0 = tc::smem_u32(B0 + (size_t)st * stage_bytes);
          bool const leader = tc::elect_one();
          if (leader) {
            for (int i = 0; i < JT; ++i) {
              int const kb = kg * JT + i;
#pragma unroll
              for (int k = 0; k < 4; ++k)
                tc::mma_bf16_ts(d, tmem + kTcH1Col + (uint32_t)(kb * 32 + k * 8),
                                tc::desc_sw128(b0 + (uint32_t)(i * kTcTileBytes) + 32 * k), idesc,
                                (kb > 0 || k > 0) ? 1u : 0u);
            }
          }
          release(leader);
          __syncwarp();
        }
        if (ok && tc::elect_one()) tc::mma_commit(&acc_full[u & 1]);
        __syncwarp();
      }
    }
    // every MMA issued has completed before TMEM is released
    if (tc::elect_one()) {
      if (!ok) abort_flag = 1;
      tc::mma_commit(&drain);
      if (!tc::mbar_wait(&drain, 0, p.wait_ns)) abort_flag = 1;
    }
    __syncwarp();
  } else {
    // ---- epilogue warps: warp w reads TMEM lanes 32 (w % 4) .. + 31 (its
    // rows) and columns 32 (w / 4) .. + 31 of each 128-column block
    int const quarter = warp & 3, cq = warp >> 2;
    int const r = quarter * 32 + lane;
    uint32_t const lane_addr = tmem + ((uint32_t)(quarter * 32) << 16);
    bool ok = true;
    int64_t u = 0;
    if (my_tiles > 0) {
      tc_build_x(p, tc_state(p, blockIdx.x, t), X, t);
      tc::fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&x_ready);
    }
    float const b3a = __ldg(p.b3), b3s = __ldg(p.b3 + 1);
    // wait for accumulator use uu and load this warp's 32 columns of it;
    // the slot is handed back as soon as the load has completed
    auto load_acc = [&](int64_t uu, float (&v)[32]) {
      if (ok) ok = tc::mbar_wait(&acc_full[uu & 1], (uint32_t)(uu >> 1) & 1, p.wait_ns) && !abort_flag;
      tc::fence_after_sync();
      __syncwarp();
      if (!ok) return false;
      tc::tmem_ld32(lane_addr + (uint32_t)((uu & 1) * NM + cq * 32), v);
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&acc_empty[uu & 1]);
      return true;
    };
    // (a, s) of a finished tile: the four column slices' partials plus b3;
    // run by threads 0-127 one tile later, off the epilogue's critical path
    auto write_out = [&](int64_t tile, float const* sp) {
      if (t < kTcRows) {
        int64_t const row = tile * kTcRows + t;
        int64_t const b = p.n_sites ? row / p.n_sites : row;
        bool const first = !p.n_sites || row == b * p.n_sites;  // the row that carries b3
        float sa = first ? b3a : 0.0f, ss = first ? b3s : 0.0f;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          sa += sp[(i * kTcRows + t) * 2];
          ss += sp[(i * kTcRows + t) * 2 + 1];
        }
        if (ok && row < p.n) {
          if (p.n_sites) {
            atomicAdd(p.out + 2 * b, sa);
            atomicAdd(p.out + 2 * b + 1, ss);
          } else {
            reinterpret_cast<float2*>(p.out)[row] = make_float2(sa, ss);
          }
        }
      }
    };
    // After a failed wait a warp skips the remaining work but still passes
    // every epi_sync, so that the named barrier never waits for it.
    for (int it = 0; it < my_tiles; ++it) {
      int64_t const tile = (int64_t)blockIdx.x + (int64_t)it * gridDim.x;
      uint32_t const par = (uint32_t)it & 1;
      // the next tile's states, loaded early: X is built after epilogue 1
      uint64_t const s_next = it + 1 < my_tiles ? tc_state(p, tile + gridDim.x, t) : 0;
      // epilogue 1: h1 = tanh(acc + b1) -> BF16 pairs -> TMEM, block by block
      for (int q = 0; q < blocks; ++q, ++u) {
        float v[32];
        if (!load_acc(u, v)) break;
        int const c0 = q * NM + cq * 32;
        uint32_t pk[16];
#pragma unroll
        for (int i = 0; i < 8; ++i) {  // 16-byte broadcast loads of the biases
          float4 const b = *reinterpret_cast<float4 const*>(sb1 + c0 + 4 * i);
          pk[2 * i] = tc::pack_bf16x2(tc::tanh_fast(v[4 * i] + b.x), tc::tanh_fast(v[4 * i + 1] + b.y));
          pk[2 * i + 1] = tc::pack_bf16x2(tc::tanh_fast(v[4 * i + 2] + b.z), tc::tanh_fast(v[4 * i + 3] + b.w));
        }
        tc::tmem_st16(lane_addr + kTcH1Col + (uint32_t)(c0 >> 1), pk);
        tc::fence_before_sync();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&h1_ready[q]);
      }
      // the next tile's X (layer 1 of this tile has finished reading X)
      if (ok && it + 1 < my_tiles) {
        tc_build_x(p, s_next, X, t);
        tc::fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&x_ready);
      }
      // the previous tile's output (its partials are complete since its epi_sync)
      if (it > 0) write_out(tile - gridDim.x, spart + (size_t)(par ^ 1u) * (4 * kTcRows * 2));
      // epilogue 2: h2 = tanh(acc + b2); partial (a, s) over this warp's columns
      float a = 0.0f, sg = 0.0f;
      for (int q = 0; q < blocks; ++q, ++u) {
        float v[32];
        if (!load_acc(u, v)) break;
        int const c0 = q * NM + cq * 32;
#pragma unroll
        for (int i = 0; i < 8; ++i) {  // 16-byte broadcast loads of b2 and W3
          float4 const b = *reinterpret_cast<float4 const*>(sb2 + c0 + 4 * i);
          float4 const wa = *reinterpret_cast<float4 const*>(sw3 + c0 + 4 * i);
          float4 const ws = *reinterpret_cast<float4 const*>(sw3 + H + c0 + 4 * i);
          float const h0 = tc::tanh_fast(v[4 * i] + b.x), h1 = tc::tanh_fast(v[4 * i + 1] + b.y);
          float const h2 = tc::tanh_fast(v[4 * i + 2] + b.z), h3 = tc::tanh_fast(v[4 * i + 3] + b.w);
          a = fmaf(wa.x, h0, fmaf(wa.y, h1, fmaf(wa.z, h2, fmaf(wa.w, h3, a))));
          sg = fmaf(ws.x, h0, fmaf(ws.y, h1, fmaf(ws.z, h2, fmaf(ws.w, h3, sg))));
        }
      }
      // two buffers of partials: a buffer is rewritten two tiles later, after
      // its reader (write_out in the next tile) has passed the next epi_sync
      float* const sp = spart + (size_t)par * (4 * kTcRows * 2);
      sp[(cq * kTcRows + r) * 2] = a;
      sp[(cq * kTcRows + r) * 2 + 1] = sg;
      epi_sync();
    }
    if (my_tiles > 0)
      write_out((int64_t)blockIdx.x + (int64_t)(my_tiles - 1) * gridDim.x,
                spart + (size_t)((my_tiles - 1) & 1) * (4 * kTcRows * 2));
    if (!ok) abort_flag = 1;
  }
  tc::fence_before_sync();
  __syncthreads();
  if (abort_flag && t == 0) atomicExch(p.error, 1);
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kTcCols);
  }
}

// Weight images for k_mlp_forward_tc from the BF16 parameters: W1 [H][n_in]
// (zero padded to 64 columns) and W2 [H][H], swizzled as the MMA reads them.
__global__ void k_mlp_images(__nv_bfloat16 const* __restrict__ W1, __nv_bfloat16 const* __restrict__ W2, int n_in,
                             int H, uint8_t* __restrict__ w1img, uint8_t* __restrict__ w2img) {
  int64_t const n1 = (int64_t)H * 8, n2 = (int64_t)(H / 64) * H * 8;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n1 + n2; q += (int64_t)gridDim.x * blockDim.x) {
    uint16_t e[8];
    uint8_t* dst;
    if (q < n1) {
      int const R = (int)(q >> 3), c = (int)(q & 7);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        int const j = 8 * c + i;
        e[i] = j < n_in ? __bfloat16_as_ushort(W1[(int64_t)R * n_in + j]) : (uint16_t)0;
      }
      dst = w1img + (int64_t)R * 128 + ((c ^ (R & 7)) << 4);
    } else {
      int64_t const u = q - n1;
      int const c = (int)(u & 7);
      int64_t const rr = u >> 3;
      int const R = (int)(rr % H), kb = (int)(rr / H);
#pragma unroll
      for (int i = 0; i < 8; ++i) e[i] = __bfloat16_as_ushort(W2[(int64_t)R * H + kb * 64 + 8 * c + i]);
      dst = w2img + ((int64_t)kb * H + R) * 128 + ((c ^ (R & 7)) << 4);
    }
    uint4 v;
    v.x = e[0] | ((uint32_t)e[1] << 16);
    v.y = e[2] | ((uint32_t)e[3] << 16);
    v.z = e[4] | ((uint32_t)e[5] << 16);
    v.w = e[6] | ((uint32_t)e[7] << 16);
    *reinterpret_cast<uint4*>(dst) = v;
  }
}

}  // namespace

struct MlpData {
  int device = -1;
  unsigned n_in = 0, hidden = 0;
  uint64_t sign_mask = 0;
  uint64_t n_params = 0;
  uint64_t oW1 = 0, ob1 = 0, oW2 = 0, ob2 = 0, oW3 = 0, ob3 = 0;  // offsets into the parameter blob
  DeviceBuffer p, pb, g, m, v;  // FP32 master, BF16 copy, gradient, Adam moments
  uint64_t step = 0;
  cudaStream_t stream = nullptr;
  DeviceBuffer x, h1, h2, out, d2, d1, dout, loss_part;  // activations of one batch
  uint64_t cap = 0, cap_train = 0;
  // tensor-core inference: swizzled weight images (rebuilt when the BF16
  // weights change) and a device error flag
  DeviceBuffer wimg, tc_error;
  bool img_valid = false;
  int path = 0;  // SED_MLP_PATH_*
  int n_sm = 0;  // multiprocessors of the device (grid of the persistent kernel)
  // tensor-core training: one batch's BF16 activations (row-major), its
  // states and targets, the padded BF16 copy of W1, an error flag, and the
  // tensor maps over them (K-major "k" and M-/N-major "m" boxes)
  DeviceBuffer tX, tH1, tH2, tG2, tG1, tW1p, tState, tAbs, tSign, t_error;
  // partial sums of the gradient, reduced in a fixed order (k_grad_rest,
  // k_column_sums): the K-split slabs of dW1 and dW2, the column sums of g1 per
  // (128-row tile, warp), the output-layer blocks' rows
  DeviceBuffer pW1, pW2, pB1, pHead;
  uint64_t t_cap = 0, t_cap_samples = 0, t_rows = 0;
  bool t_wmaps = false;
  // patch network (n_sites > 0): the n_in = P sites of each site's patch,
  // [n_sites][P] on the device; one activation row per (sample, site)
  unsigned n_sites = 0;
  DeviceBuffer patch_dev;
  CUtensorMap mXk{}, mXm{}, mW1k{}, mH1k{}, mH1m{}, mW2k{}, mW2m{}, mG2k{}, mG2m{}, mG1m{};
  ~MlpData() {
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

template <class TB>
void gemm(cudaStream_t s, int M, int N, int K, float const* A, int64_t sam, int64_t sak, TB const* B, int64_t sbk,
          int64_t sbn, float* C, int64_t ldc, float const* bias, int act, int accumulate) {
  dim3 grid((N + kTile - 1) / kTile, (M + kTile - 1) / kTile);
  { k_gemm<TB><<<grid, 256, 0, s>>>(M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, bias, act, accumulate); note_launches(1); }
}

int ensure_batch(MlpData& d, uint64_t n, bool train) {
  uint64_t const h = d.hidden;
  if (n > d.cap) {
    d.cap = 0;
    if (int st = d.x.allocate(n * d.n_in * 4)) return st;
    if (int st = d.h1.allocate(n * h * 4)) return st;
    if (int st = d.h2.allocate(n * h * 4)) return st;
    if (int st = d.out.allocate(n * 2 * 4)) return st;
    if (int st = d.loss_part.allocate(152 * 16 * 8)) return st;
    d.cap = n;
  }
  if (train && n > d.cap_train) {
    d.cap_train = 0;
    if (int st = d.d2.allocate(n * h * 4)) return st;
    if (int st = d.d1.allocate(n * h * 4)) return st;
    if (int st = d.dout.allocate(n * 2 * 4)) return st;
    d.cap_train = n;
  }
  return LS_SUCCESS;
}

// forward pass for states[0..n) (device pointer); activations stay in d.x/h1/h2/out
int forward(MlpData& d, uint64_t const* states, uint64_t n, bool train) {
  if (int st = ensure_batch(d, n, train)) return st;
  cudaStream_t s = d.stream;
  int const N = (int)n, H = (int)d.hidden, I = (int)d.n_in;
  __nv_bfloat16 const* W = d.pb.as<__nv_bfloat16>();
  float const* P = d.p.as<float>();
  { k_spins<<<blocks_for((int64_t)n * I), 256, 0, s>>>(states, (int64_t)n, I, d.x.as<float>()); note_launches(1); }
  // h1 [N x H] = tanh(x W1^T + b1): B(k, n) = W1[n][k]
  gemm<__nv_bfloat16>(s, N, H, I, d.x.as<float>(), I, 1, W + d.oW1, 1, I, d.h1.as<float>(), H, P + d.ob1, 1, 0);
  gemm<__nv_bfloat16>(s, N, H, H, d.h1.as<float>(), H, 1, W + d.oW2, 1, H, d.h2.as<float>(), H, P + d.ob2, 1, 0);
  gemm<__nv_bfloat16>(s, N, 2, H, d.h2.as<float>(), H, 1, W + d.oW3, 1, H, d.out.as<float>(), 2, P + d.ob3, 0, 0);
  SED_TRY_CUDA(cudaGetLastError());
  return LS_SUCCESS;
}

// loss and gradient (into d.g) of one batch after forward(..., train = true)
int backward(MlpData& d, uint64_t const* states, uint64_t n, float const* t_abs, float const* t_sign,
             double* loss) {
  cudaStream_t s = d.stream;
  int const N = (int)n, H = (int)d.hidden, I = (int)d.n_in;
  __nv_bfloat16 const* W = d.pb.as<__nv_bfloat16>();
  float* G = d.g.as<float>();
  unsigned const lb = blocks_for((int64_t)n);
  SED_TRY_CUDA(cudaMemsetAsync(d.g.ptr, 0, d.n_params * 4, s));
  { k_out_grad<<<lb, 256, 0, s>>>(d.out.as<float>(), states, d.sign_mask, t_abs, t_sign, (int64_t)n, d.dout.as<float>(), d.loss_part.as<double>()); note_launches(1); }
  // dW3 [2 x H] = dout^T h2 ; db3 = colsum(dout)
  gemm<float>(s, 2, H, N, d.dout.as<float>(), 1, 2, d.h2.as<float>(), H, 1, G + d.oW3, H, nullptr, 0, 0);
  { k_column_sums<<<2, 256, 0, s>>>(G + d.ob3, d.dout.as<float>(), (int64_t)n, 2); note_launches(1); }
  // dh2 [N x H] = dout W3, times tanh'
  gemm<__nv_bfloat16>(s, N, H, 2, d.dout.as<float>(), 2, 1, W + d.oW3, H, 1, d.d2.as<float>(), H, nullptr, 0, 0);
  { k_tanh_back<<<blocks_for((int64_t)n * H), 256, 0, s>>>(d.h2.as<float>(), d.d2.as<float>(), (int64_t)n * H); note_launches(1); }
  // dW2 [H x H] = dh2^T h1 ; db2
  gemm<float>(s, H, H, N, d.d2.as<float>(), 1, H, d.h1.as<float>(), H, 1, G + d.oW2, H, nullptr, 0, 0);
  { k_column_sums<<<H, 256, 0, s>>>(G + d.ob2, d.d2.as<float>(), (int64_t)n, H); note_launches(1); }
  // dh1 [N x H] = dh2 W2, times tanh'
  gemm<__nv_bfloat16>(s, N, H, H, d.d2.as<float>(), H, 1, W + d.oW2, H, 1, d.d1.as<float>(), H, nullptr, 0, 0);
  { k_tanh_back<<<blocks_for((int64_t)n * H), 256, 0, s>>>(d.h1.as<float>(), d.d1.as<float>(), (int64_t)n * H); note_launches(1); }
  // dW1 [H x I] = dh1^T x ; db1
  gemm<float>(s, H, I, N, d.d1.as<float>(), 1, H, d.x.as<float>(), I, 1, G + d.oW1, I, nullptr, 0, 0);
  { k_column_sums<<<H, 256, 0, s>>>(G + d.ob1, d.d1.as<float>(), (int64_t)n, H); note_launches(1); }
  SED_TRY_CUDA(cudaGetLastError());
  if (loss) {
    std::vector<double> lp(lb);
    SED_TRY_CUDA(cudaMemcpyAsync(lp.data(), d.loss_part.ptr, lb * 8, cudaMemcpyDeviceToHost, s));
    SED_TRY_CUDA(cudaStreamSynchronize(s));
    double t = 0.0;
    for (double q : lp) t += q;
    *loss = t / (double)n;
  }
  return LS_SUCCESS;
}

// The fused inference kernel's shapes.
bool fused_shape(MlpData const& d) {
  return d.n_in <= 64 && (d.hidden == 128 || d.hidden == 256 || d.hidden == 512);
}

bool tc_eligible(MlpData const& d) {
  if (d.n_sites) return true;  // patch networks run on the tensor cores only (checked at creation)
  return d.path != SED_MLP_PATH_SIMT && d.n_in <= 64 && (d.hidden == 128 || d.hidden == 256 || d.hidden == 512);
}

// (a, s) for states[0..n) (device pointer) into out[2 n] (device), on the
// tensor cores.
int forward_tc(MlpData& d, uint64_t const* states, uint64_t n, float* out) {
  cudaStream_t s = d.stream;
  int const H = (int)d.hidden;
  size_t const img1 = (size_t)H * 128, img2 = (size_t)H * H * 2;
  if (!d.img_valid) {
    if (int st = d.wimg.allocate(img1 + img2)) return st;
    if (!d.tc_error.ptr)
      if (int st = d.tc_error.allocate(16)) return st;
    __nv_bfloat16 const* W = d.pb.as<__nv_bfloat16>();
    { k_mlp_images<<<blocks_for((int64_t)(H * 8 + H * H / 8)), 256, 0, s>>>(W + d.oW1, W + d.oW2, (int)d.n_in, H, d.wimg.as<uint8_t>(), d.wimg.as<uint8_t>() + img1); note_launches(1); }
    SED_TRY_CUDA(cudaGetLastError());
    d.img_valid = true;
  }
  if (n == 0) return LS_SUCCESS;
  size_t const smem = tc_smem_bytes(H);
  SED_TRY_CUDA(cudaFuncSetAttribute(k_mlp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  SED_TRY_CUDA(cudaMemsetAsync(d.tc_error.ptr, 0, 4, s));
  uint64_t const rows = d.n_sites ? n * d.n_sites : n;
  if (d.n_sites) SED_TRY_CUDA(cudaMemsetAsync(out, 0, n * 8, s));  // the site rows add into it
  MlpTcArgs a;
  a.states = states;
  a.n = (int64_t)rows;
  a.patch = d.n_sites ? d.patch_dev.as<uint16_t>() : nullptr;
  a.n_sites = (int)d.n_sites;
  a.n_in = (int)d.n_in;
  a.hidden = H;
  a.stages = tc_stages(H);
  a.w1img = d.wimg.as<uint8_t>();
  a.w2img = d.wimg.as<uint8_t>() + img1;
  a.b1 = d.p.as<float>() + d.ob1;
  a.b2 = d.p.as<float>() + d.ob2;
  a.W3 = d.pb.as<__nv_bfloat16>() + d.oW3;
  a.b3 = d.p.as<float>() + d.ob3;
  a.out = out;
  a.error = d.tc_error.as<int>();
  a.wait_ns = device_wait_ns(kTcWaitNs);
  if (d.n_sm == 0) SED_TRY_CUDA(cudaDeviceGetAttribute(&d.n_sm, cudaDevAttrMultiProcessorCount, d.device));
  uint64_t const tiles = (rows + kTcRows - 1) / kTcRows;
  unsigned const grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)d.n_sm);  // persistent: one CTA per SM
  { k_mlp_forward_tc<<<grid, kTcThreads, smem, s>>>(a); note_launches(1); }
  SED_TRY_CUDA(cudaGetLastError());
  int err = 0;
  SED_TRY_CUDA(cudaMemcpyAsync(&err, d.tc_error.ptr, 4, cudaMemcpyDeviceToHost, s));
  SED_TRY_CUDA(cudaStreamSynchronize(s));
  if (err) return fail(LS_DEVICE_TIMEOUT, "MLP tensor-core forward: a wait on the tensor cores timed out");
  return LS_SUCCESS;
}

int refresh_bf16(MlpData& d) {
  d.img_valid = false;
  { k_to_bf16<<<blocks_for((int64_t)d.n_params), 256, 0, d.stream>>>(d.p.as<float>(), d.pb.as<__nv_bfloat16>(), (int64_t)d.n_params); note_launches(1); }
  SED_TRY_CUDA(cudaGetLastError());
  return LS_SUCCESS;
}

// device copy of a host-or-device array
int stage(DeviceBuffer& buf, void const* src, size_t bytes, cudaStream_t s) {
  if (int st = buf.allocate(std::max<size_t>(bytes, 16))) return st;
  SED_TRY_CUDA(cudaMemcpyAsync(buf.ptr, src, bytes, cudaMemcpyDefault, s));
  return LS_SUCCESS;
}

// Activation rows of one tensor-core pass at most (the GEMM grid's rows of
// 128-row tiles).
constexpr uint64_t kTcMaxRows = 65535ull * 128;

// Activation rows of a batch: one per sample, or one per (sample, site) for
// a patch network.
uint64_t tc_rows(MlpData const& d, uint64_t samples) { return samples * (d.n_sites ? d.n_sites : 1u); }
// Output tile width of the hidden-layer GEMMs.
int tc_tile(MlpData const& d) { return d.hidden >= 128 ? 128 : 64; }

// K splits of a weight gradient: as many CTAs as fit on the multiprocessors
// in one wave (one 128-column CTA per multiprocessor)
int tc_split(MlpData const& d, int tiles, int k_tiles) {
  return std::max(1, std::min(k_tiles, d.n_sm / tiles));
}

// Launch geometry of one training step on n samples (n_sm must be known).
struct TcShape {
  int rows, k_tiles, s2, s1, m_tiles, hb;
};
TcShape tc_shape(MlpData const& d, uint64_t n) {
  TcShape t;
  int const H = (int)d.hidden, tn = tc_tile(d), mh = (H + 127) / 128;
  t.rows = (int)tc_rows(d, n);
  t.k_tiles = (t.rows + 63) / 64;
  t.s2 = tc_split(d, mh * (H / tn), t.k_tiles);
  t.s1 = tc_split(d, mh, t.k_tiles);
  t.m_tiles = (t.rows + 127) / 128;
  uint64_t const per_block = d.n_sites ? 8 : 64;  // samples per output-layer block
  t.hb = (int)std::max<uint64_t>(1, std::min<uint64_t>((n + per_block - 1) / per_block, 152 * 16));
  return t;
}

// Tensor-core training: buffers for batches of up to `samples` samples,
// tensor maps for batches of exactly `samples` (rows past them read as
// zero); with `reset` also the padded W1 copy refreshed from the FP32 master
// and the error flag cleared.
int tc_train_prepare(MlpData& d, uint64_t samples, bool reset = true) {
  uint64_t const H = d.hidden, rows = tc_rows(d, samples);
  uint32_t const tn = (uint32_t)tc_tile(d);
  if (rows > d.t_cap) {
    d.t_cap = d.t_rows = 0;
    for (DeviceBuffer* b : {&d.tH1, &d.tH2, &d.tG2, &d.tG1})
      if (int st = b->allocate(rows * H * 2)) return st;
    if (int st = d.tX.allocate(rows * 64 * 2)) return st;
    d.t_cap = rows;
  }
  if (samples > d.t_cap_samples) {
    d.t_cap_samples = 0;
    if (int st = d.tState.allocate(samples * 8)) return st;
    if (int st = d.tAbs.allocate(samples * 4)) return st;
    if (int st = d.tSign.allocate(samples * 4)) return st;
    d.t_cap_samples = samples;
  }
  if (!d.loss_part.ptr)
    if (int st = d.loss_part.allocate(152 * 16 * 8)) return st;
  if (!d.t_wmaps) {
    if (int st = d.tW1p.allocate(H * 64 * 2)) return st;
    if (int st = d.t_error.allocate(16)) return st;
    __nv_bfloat16 const* W2 = d.pb.as<__nv_bfloat16>() + d.oW2;
    if (int st = tma_map_bf16(&d.mW1k, d.tW1p.ptr, H, 64, 64, tn)) return st;
    if (int st = tma_map_bf16(&d.mW2k, W2, H, H, H, tn)) return st;
    if (int st = tma_map_bf16(&d.mW2m, W2, H, H, H, 64)) return st;
    d.t_wmaps = true;
  }
  if (rows != d.t_rows) {
    d.t_rows = 0;
    if (int st = tma_map_bf16(&d.mXk, d.tX.ptr, rows, 64, 64, 128)) return st;
    if (int st = tma_map_bf16(&d.mXm, d.tX.ptr, rows, 64, 64, 64)) return st;
    if (int st = tma_map_bf16(&d.mH1k, d.tH1.ptr, rows, H, H, 128)) return st;
    if (int st = tma_map_bf16(&d.mH1m, d.tH1.ptr, rows, H, H, 64)) return st;
    if (int st = tma_map_bf16(&d.mG2k, d.tG2.ptr, rows, H, H, 128)) return st;
    if (int st = tma_map_bf16(&d.mG2m, d.tG2.ptr, rows, H, H, 64)) return st;
    if (int st = tma_map_bf16(&d.mG1m, d.tG1.ptr, rows, H, H, 64)) return st;
    d.t_rows = rows;
  }
  if (d.n_sm == 0) SED_TRY_CUDA(cudaDeviceGetAttribute(&d.n_sm, cudaDevAttrMultiProcessorCount, d.device));
  {  // partial-sum buffers of a step on this many samples
    TcShape const sh = tc_shape(d, samples);
    auto need = [](DeviceBuffer& b, size_t bytes) { return b.bytes >= bytes ? LS_SUCCESS : b.allocate(bytes); };
    if (int st = need(d.pW1, (size_t)sh.s1 * H * d.n_in * 4)) return st;
    if (int st = need(d.pW2, (size_t)sh.s2 * H * H * 4)) return st;
    if (int st = need(d.pB1, (size_t)sh.m_tiles * 4 * H * 4)) return st;
    if (int st = need(d.pHead, (size_t)sh.hb * (3 * H + 2) * 4)) return st;
    SED_TRY_CUDA(cudaFuncSetAttribute(k_head, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)head_smem_bytes((int)H)));
    SED_TRY_CUDA(cudaFuncSetAttribute(k_head_patch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)head_smem_bytes((int)H)));
  }
  if (reset) {
    { k_w1_pad<<<blocks_for((int64_t)H * 64), 256, 0, d.stream>>>(d.p.as<float>() + d.oW1, (int)d.n_in, (int)H, d.tW1p.as<__nv_bfloat16>()); note_launches(1); }
    SED_TRY_CUDA(cudaMemsetAsync(d.t_error.ptr, 0, 4, d.stream));
    SED_TRY_CUDA(cudaGetLastError());
  }
  return LS_SUCCESS;
}

// Forward and backward pass of batch rows [0, n) (staged by k_batch): the
// gradient into d.g, the loss (if requested) into *loss. Every kernel of the
// step is launched with programmatic stream serialisation. The gradient's
// sums go through partial-sum buffers reduced in a fixed order, so a step
// gives the same bits every time.
int tc_train_step(MlpData& d, uint64_t n, double* loss) {
  cudaStream_t s = d.stream;
  TcShape const sh = tc_shape(d, n);
  int const H = (int)d.hidden, N = sh.rows, tn = tc_tile(d);
  float* const G = d.g.as<float>();
  float const* const P = d.p.as<float>();
  TcGemmArgs base;
  base.error = d.t_error.as<int>();
  base.wait_ns = device_wait_ns(kTcWaitNs);
  // h1 = bf16(tanh(X W1^T + b1)), h2 = bf16(tanh(h1 W2^T + b2))
  TcGemmArgs f = base;
  f.M = N;
  f.N = H;
  f.k_tiles = 1;
  f.epilogue = kEpiTanh;
  f.bias = P + d.ob1;
  f.out_bf16 = d.tH1.as<__nv_bfloat16>();
  f.ld_out = H;
  if (int st = tc_gemm(s, d.mXk, d.mW1k, f, tn)) return st;
  f.k_tiles = H / 64;
  f.bias = P + d.ob2;
  f.out_bf16 = d.tH2.as<__nv_bfloat16>();
  if (int st = tc_gemm(s, d.mH1k, d.mW2k, f, tn)) return st;
  // output layer, loss, g2, db2, dW3, db3
  unsigned const hb = (unsigned)sh.hb;
  size_t const hsm = head_smem_bytes(H);
  if (d.n_sites) {  // one warp per sample
    SED_TRY_CUDA(launch_pdl(k_head_patch, dim3(hb), dim3(256), hsm, s, (__nv_bfloat16 const*)d.tH2.as<__nv_bfloat16>(), H, (int)d.n_sites, (int64_t)n, (__nv_bfloat16 const*)(d.pb.as<__nv_bfloat16>() + d.oW3), P + d.ob3, (uint64_t const*)d.tState.as<uint64_t>(), (float const*)d.tAbs.as<float>(), (float const*)d.tSign.as<float>(), d.sign_mask, d.tG2.as<__nv_bfloat16>(), d.pHead.as<float>(), d.loss_part.as<double>(), (float*)nullptr));
  } else {  // <= 8 rows a warp
    SED_TRY_CUDA(launch_pdl(k_head, dim3(hb), dim3(256), hsm, s, (__nv_bfloat16 const*)d.tH2.as<__nv_bfloat16>(), H, (int64_t)n, (__nv_bfloat16 const*)(d.pb.as<__nv_bfloat16>() + d.oW3), P + d.ob3, (uint64_t const*)d.tState.as<uint64_t>(), (float const*)d.tAbs.as<float>(), (float const*)d.tSign.as<float>(), d.sign_mask, d.tG2.as<__nv_bfloat16>(), d.pHead.as<float>(), d.loss_part.as<double>()));
  }
  note_launches(1);
  // g1 = bf16((g2 W2) (1 - h1^2)) and db1; W2 read N-major (element (i, o) at W2[o][i])
  TcGemmArgs b = base;
  b.M = N;
  b.N = H;
  b.k_tiles = H / 64;
  b.b_mn = 1;
  b.epilogue = kEpiBack;
  b.aux = d.tH1.as<__nv_bfloat16>();
  b.ld_aux = H;
  b.colsum = d.pB1.as<float>();
  b.out_bf16 = d.tG1.as<__nv_bfloat16>();
  b.ld_out = H;
  if (int st = tc_gemm(s, d.mG2k, d.mW2m, b, tn)) return st;
  // dW2 = g2^T h1 and dW1 = g1^T X: K = the batch, both operands read M-/N-major
  TcGemmArgs w = base;
  w.M = H;
  w.N = H;
  w.k_tiles = (N + 63) / 64;
  w.a_mn = w.b_mn = 1;
  w.epilogue = kEpiAdd;
  w.out_f32 = d.pW2.as<float>();
  w.ld_f32 = H;
  w.n_valid = H;
  w.split = sh.s2;
  if (int st = tc_gemm(s, d.mG2m, d.mH1m, w, tn)) return st;
  w.N = 64;
  w.out_f32 = d.pW1.as<float>();
  w.ld_f32 = d.n_in;
  w.n_valid = (int)d.n_in;
  w.split = sh.s1;
  if (int st = tc_gemm(s, d.mG1m, d.mXm, w, 64)) return st;
  // the gradient, each entry added in a fixed order
  SED_TRY_CUDA(launch_pdl(k_column_sums, dim3(H), dim3(256), 0, s, G + d.ob1, (float const*)d.pB1.as<float>(), (int64_t)sh.m_tiles * 4, H));
  SED_TRY_CUDA(launch_pdl(k_grad_rest, dim3(blocks_for((int64_t)d.n_params)), dim3(256), 0, s, G, (int)d.n_in, H, (float const*)d.pW1.as<float>(), sh.s1, (float const*)d.pW2.as<float>(), sh.s2, (float const*)d.pHead.as<float>(), (int)hb));
  note_launches(2);
  if (loss) {
    std::vector<double> lp(hb);
    SED_TRY_CUDA(cudaMemcpyAsync(lp.data(), d.loss_part.ptr, hb * 8, cudaMemcpyDeviceToHost, s));
    SED_TRY_CUDA(cudaStreamSynchronize(s));
    double t = 0.0;
    for (double q : lp) t += q;
    *loss = t / (double)n;
  }
  return LS_SUCCESS;
}

int tc_check_error(MlpData& d) {
  int err = 0;
  SED_TRY_CUDA(cudaMemcpyAsync(&err, d.t_error.ptr, 4, cudaMemcpyDeviceToHost, d.stream));
  SED_TRY_CUDA(cudaStreamSynchronize(d.stream));
  if (err) return fail(LS_DEVICE_TIMEOUT, "MLP tensor-core training: a wait on the tensor cores or a copy timed out");
  return LS_SUCCESS;
}

// Patch network inference for hidden sizes the fused kernel does not take
// (64): (a, s) for states[0..n) (device) into out[2 n] (device), in chunks
// of about 2^21 activation rows through the training step's forward GEMMs
// and k_head_patch. Larger networks run in k_mlp_forward_tc.
int forward_patch(MlpData& d, uint64_t const* states, uint64_t n, float* out) {
  if (n == 0) return LS_SUCCESS;
  cudaStream_t s = d.stream;
  int const H = (int)d.hidden, tn = tc_tile(d);
  uint64_t const chunk = std::max<uint64_t>(1, ((uint64_t)1 << 21) / d.n_sites);
  for (uint64_t b0 = 0; b0 < n; b0 += chunk) {
    uint64_t const nb = std::min(chunk, n - b0);
    if (int st = tc_train_prepare(d, nb, b0 == 0)) return st;
    int64_t const rows = (int64_t)tc_rows(d, nb);
    SED_TRY_CUDA(launch_pdl(k_batch_patch, dim3(blocks_for(rows * 8)), dim3(256), 0, s, states, (float const*)nullptr, (float const*)nullptr, (uint32_t const*)nullptr, b0, (int64_t)nb, (int)d.n_sites, (int)d.n_in, (uint16_t const*)d.patch_dev.as<uint16_t>(), d.tX.as<__nv_bfloat16>(), d.tState.as<uint64_t>(), d.tAbs.as<float>(), d.tSign.as<float>()));
    note_launches(1);
    TcGemmArgs f;
    f.error = d.t_error.as<int>();
    f.wait_ns = device_wait_ns(kTcWaitNs);
    f.M = (int)rows;
    f.N = H;
    f.k_tiles = 1;
    f.epilogue = kEpiTanh;
    f.bias = d.p.as<float>() + d.ob1;
    f.out_bf16 = d.tH1.as<__nv_bfloat16>();
    f.ld_out = H;
    if (int st = tc_gemm(s, d.mXk, d.mW1k, f, tn)) return st;
    f.k_tiles = H / 64;
    f.bias = d.p.as<float>() + d.ob2;
    f.out_bf16 = d.tH2.as<__nv_bfloat16>();
    if (int st = tc_gemm(s, d.mH1k, d.mW2k, f, tn)) return st;
    unsigned const hb = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((nb + 7) / 8, 152 * 16));
    SED_TRY_CUDA(launch_pdl(k_head_patch, dim3(hb), dim3(256), 0, s, (__nv_bfloat16 const*)d.tH2.as<__nv_bfloat16>(), H, (int)d.n_sites, (int64_t)nb, (__nv_bfloat16 const*)(d.pb.as<__nv_bfloat16>() + d.oW3), (float const*)(d.p.as<float>() + d.ob3), (uint64_t const*)nullptr, (float const*)nullptr, (float const*)nullptr, d.sign_mask, (__nv_bfloat16*)nullptr, (float*)nullptr, (double*)nullptr, out + 2 * b0));
    note_launches(1);
  }
  return tc_check_error(d);
}

}  // namespace
}  // namespace sed

struct sed_mlp {
  sed::MlpData d;
};

using namespace sed;

extern "C" {

int sed_mlp_create(sed_mlp** out, unsigned n_inputs, unsigned hidden, uint64_t sign_mask, uint64_t seed) {
  if (!out) return fail(LS_INVALID_ARGUMENT, "sed_mlp_create: NULL argument");
  *out = nullptr;
  if (n_inputs == 0 || n_inputs > 64 || hidden == 0 || hidden > 4096)
    return fail(LS_INVALID_ARGUMENT, "sed_mlp_create: n_inputs must be 1..64 and hidden 1..4096");
  if (n_inputs < 64 && (sign_mask >> n_inputs) != 0)
    return fail(LS_INVALID_ARGUMENT, "sed_mlp_create: sign_mask has bits beyond n_inputs");
  auto* m = new (std::nothrow) sed_mlp;
  if (!m) return fail(LS_OUT_OF_MEMORY, "sed_mlp_create");
  MlpData& d = m->d;
  if (int st = current_device(&d.device)) {
    delete m;
    return st;
  }
  d.n_in = n_inputs;
  d.hidden = hidden;
  d.sign_mask = sign_mask;
  uint64_t const I = n_inputs, H = hidden;
  d.oW1 = 0;
  d.ob1 = d.oW1 + H * I;
  d.oW2 = d.ob1 + H;
  d.ob2 = d.oW2 + H * H;
  d.oW3 = d.ob2 + H;
  d.ob3 = d.oW3 + 2 * H;
  d.n_params = d.ob3 + 2;
  // Gaussian init with variance 1/fan_in, biases zero (host mt19937_64, so a
  // seed gives the same network on every machine)
  std::vector<float> host(d.n_params, 0.0f);
  std::mt19937_64 rng(seed);
  auto init = [&](uint64_t off, uint64_t count, uint64_t fan_in) {
    std::normal_distribution<double> nd(0.0, 1.0 / std::sqrt((double)fan_in));
    for (uint64_t q = 0; q < count; ++q) host[off + q] = (float)nd(rng);
  };
  init(d.oW1, H * I, I);
  init(d.oW2, H * H, H);
  init(d.oW3, 2 * H, H);
  int st = LS_SUCCESS;
  if (cudaStreamCreateWithFlags(&d.stream, cudaStreamNonBlocking) != cudaSuccess) {
    d.stream = nullptr;
    st = fail(LS_CUDA_ERROR, "sed_mlp_create: cudaStreamCreate");
  }
  if (!st) st = d.p.allocate(d.n_params * 4);
  if (!st) st = d.pb.allocate(d.n_params * 2);
  if (!st) st = d.g.allocate(d.n_params * 4);
  if (!st) st = d.m.allocate(d.n_params * 4);
  if (!st) st = d.v.allocate(d.n_params * 4);
  if (!st && cudaMemcpy(d.p.ptr, host.data(), d.n_params * 4, cudaMemcpyHostToDevice) != cudaSuccess)
    st = fail(LS_CUDA_ERROR, "sed_mlp_create: upload");
  if (!st && (cudaMemset(d.m.ptr, 0, d.n_params * 4) != cudaSuccess ||
              cudaMemset(d.v.ptr, 0, d.n_params * 4) != cudaSuccess))
    st = fail(LS_CUDA_ERROR, "sed_mlp_create: cudaMemset");
  if (!st) st = refresh_bf16(d);
  if (!st && cudaStreamSynchronize(d.stream) != cudaSuccess)
    st = fail(LS_CUDA_ERROR, "sed_mlp_create: initialisation");
  if (st) {
    delete m;
    return st;
  }
  *out = m;
  return LS_SUCCESS;
}

int sed_mlp_set_patch_sites(sed_mlp* m, unsigned n_sites, uint16_t const* patch_sites, uint64_t sign_mask) {
  if (!m || !patch_sites || n_sites == 0) return fail(LS_INVALID_ARGUMENT, "sed_mlp_set_patch_sites: bad argument");
  MlpData& d = m->d;
  if (!d.n_sites) return fail(LS_INVALID_ARGUMENT, "sed_mlp_set_patch_sites: not a patch network");
  if (n_sites > 64) return fail(LS_INVALID_ARGUMENT, "sed_mlp_set_patch_sites: at most 64 sites");
  if (n_sites < 64 && (sign_mask >> n_sites) != 0)
    return fail(LS_INVALID_ARGUMENT, "sed_mlp_set_patch_sites: sign_mask has bits beyond n_sites");
  for (uint64_t q = 0; q < (uint64_t)n_sites * d.n_in; ++q)
    if (patch_sites[q] >= n_sites) return fail(LS_INVALID_ARGUMENT, "sed_mlp_set_patch_sites: site out of range");
  ScopedDevice dev(d.device);
  DeviceBuffer buf;
  if (int st = buf.allocate((size_t)n_sites * d.n_in * 2)) return st;
  SED_TRY_CUDA(cudaMemcpy(buf.ptr, patch_sites, (size_t)n_sites * d.n_in * 2, cudaMemcpyHostToDevice));
  SED_TRY_CUDA(cudaStreamSynchronize(d.stream));  // no pass of the old geometry is in flight
  d.patch_dev = std::move(buf);
  d.n_sites = n_sites;
  d.sign_mask = sign_mask;
  d.t_rows = 0;  // activation rows per sample changed: new tensor maps
  return LS_SUCCESS;
}

int sed_mlp_create_patch(sed_mlp** out, unsigned n_sites, unsigned patch, uint16_t const* patch_sites,
                         unsigned hidden, uint64_t sign_mask, uint64_t seed) {
  if (!out) return fail(LS_INVALID_ARGUMENT, "sed_mlp_create_patch: NULL argument");
  *out = nullptr;
  if (patch == 0 || patch > 64 || (hidden != 64 && hidden != 128 && hidden != 256))
    return fail(LS_INVALID_ARGUMENT, "sed_mlp_create_patch: patch must be 1..64 and hidden 64, 128 or 256");
  if (n_sites == 0 || n_sites > 64 || !patch_sites)
    return fail(LS_INVALID_ARGUMENT, "sed_mlp_create_patch: n_sites must be 1..64 with a patch table");
  sed_mlp* m = nullptr;
  if (int st = sed_mlp_create(&m, patch, hidden, 0, seed)) return st;
  m->d.n_sites = 1;  // marks the patch network for the check below
  if (int st = sed_mlp_set_patch_sites(m, n_sites, patch_sites, sign_mask)) {
    sed_mlp_destroy(m);
    return st;
  }
  *out = m;
  return LS_SUCCESS;
}

void sed_mlp_destroy(sed_mlp* m) {
  if (!m) return;
  ScopedDevice dev(m->d.device);
  delete m;
}

uint64_t sed_mlp_num_params(sed_mlp const* m) { return m ? m->d.n_params : 0; }

int sed_mlp_set_path(sed_mlp* m, int path) {
  if (!m) return fail(LS_INVALID_ARGUMENT, "sed_mlp_set_path: NULL argument");
  if (path != SED_MLP_PATH_AUTO && path != SED_MLP_PATH_SIMT)
    return fail(LS_INVALID_ARGUMENT, "sed_mlp_set_path: unknown path");
  if (m->d.n_sites && path == SED_MLP_PATH_SIMT)
    return fail(LS_INVALID_ARGUMENT, "sed_mlp_set_path: a patch network runs on the tensor cores only");
  m->d.path = path;
  return LS_SUCCESS;
}

int sed_mlp_uses_tensor_cores(sed_mlp const* m) { return m && tc_eligible(m->d) ? 1 : 0; }

int sed_mlp_get_params(sed_mlp const* m, float* out) {
  if (!m || !out) return fail(LS_INVALID_ARGUMENT, "sed_mlp_get_params: NULL argument");
  ScopedDevice dev(m->d.device);
  if (int st = wait_for_caller({out})) return st;
  SED_TRY_CUDA(cudaMemcpy(out, m->d.p.ptr, m->d.n_params * 4, cudaMemcpyDefault));
  return LS_SUCCESS;
}

int sed_mlp_set_params(sed_mlp* m, float const* in) {
  if (!m || !in) return fail(LS_INVALID_ARGUMENT, "sed_mlp_set_params: NULL argument");
  MlpData& d = m->d;
  ScopedDevice dev(d.device);
  if (int st = wait_for_caller({in})) return st;
  SED_TRY_CUDA(cudaMemcpy(d.p.ptr, in, d.n_params * 4, cudaMemcpyDefault));
  if (int st = refresh_bf16(d)) return st;
  SED_TRY_CUDA(cudaStreamSynchronize(d.stream));
  return LS_SUCCESS;
}

int sed_mlp_forward(sed_mlp* m, uint64_t const* states, uint64_t n, float* out) {
  if (!m || (n && (!states || !out))) return fail(LS_INVALID_ARGUMENT, "sed_mlp_forward: NULL argument");
  MlpData& d = m->d;
  ScopedDevice dev(d.device);
  if (int st = wait_for_caller({states, out})) return st;
  uint64_t const chunk = 1u << 18;
  DeviceBuffer sbuf;
  if (n)
    if (int st = sbuf.allocate(std::min(chunk, n) * 8)) return st;
  bool const tc_path = tc_eligible(d);
  for (uint64_t b0 = 0; b0 < n; b0 += chunk) {
    uint64_t const nb = std::min(chunk, n - b0);
    SED_TRY_CUDA(cudaMemcpyAsync(sbuf.ptr, states + b0, nb * 8, cudaMemcpyDefault, d.stream));
    if (d.n_sites && !fused_shape(d)) {
      if (int st = ensure_batch(d, nb, false)) return st;
      if (int st = forward_patch(d, sbuf.as<uint64_t>(), nb, d.out.as<float>())) return st;
    } else if (tc_path) {
      if (int st = ensure_batch(d, nb, false)) return st;
      if (int st = forward_tc(d, sbuf.as<uint64_t>(), nb, d.out.as<float>())) return st;
    } else if (int st = forward(d, sbuf.as<uint64_t>(), nb, false)) {
      return st;
    }
    SED_TRY_CUDA(cudaMemcpyAsync(out + 2 * b0, d.out.ptr, nb * 8, cudaMemcpyDefault, d.stream));
  }
  SED_TRY_CUDA(cudaStreamSynchronize(d.stream));
  return LS_SUCCESS;
}

int sed_mlp_loss_grad(sed_mlp* m, uint64_t const* states, float const* t_abs, float const* t_sign, uint64_t n,
                      double* loss, float* grads) {
  if (!m || !n || !states || !t_abs || !t_sign) return fail(LS_INVALID_ARGUMENT, "sed_mlp_loss_grad: bad argument");
  if (n > (1u << 20)) return fail(LS_INVALID_ARGUMENT, "sed_mlp_loss_grad: at most 2^20 samples per call");
  MlpData& d = m->d;
  ScopedDevice dev(d.device);
  if (int st = wait_for_caller({states, t_abs, t_sign, grads})) return st;
  DeviceBuffer sb, ta, ts;
  if (int st = stage(sb, states, n * 8, d.stream)) return st;
  if (int st = stage(ta, t_abs, n * 4, d.stream)) return st;
  if (int st = stage(ts, t_sign, n * 4, d.stream)) return st;
  if (tc_eligible(d)) {
    if (tc_rows(d, n) > kTcMaxRows)
      return fail(LS_INVALID_ARGUMENT, "sed_mlp_loss_grad: a patch network takes at most " +
                                           std::to_string(kTcMaxRows / d.n_sites) + " samples per call");
    if (int st = tc_train_prepare(d, n)) return st;
    if (d.n_sites) {
      { k_batch_patch<<<blocks_for((int64_t)tc_rows(d, n) * 8), 256, 0, d.stream>>>(sb.as<uint64_t>(), ta.as<float>(), ts.as<float>(), nullptr, 0, (int64_t)n, (int)d.n_sites, (int)d.n_in, d.patch_dev.as<uint16_t>(), d.tX.as<__nv_bfloat16>(), d.tState.as<uint64_t>(), d.tAbs.as<float>(), d.tSign.as<float>()); note_launches(1); }
    } else {
      { k_batch<<<blocks_for((int64_t)n * 8), 256, 0, d.stream>>>(sb.as<uint64_t>(), ta.as<float>(), ts.as<float>(), nullptr, 0, (int64_t)n, (int)d.n_in, d.tX.as<__nv_bfloat16>(), d.tState.as<uint64_t>(), d.tAbs.as<float>(), d.tSign.as<float>()); note_launches(1); }
    }
    if (int st = tc_train_step(d, n, loss)) return st;
    if (int st = tc_check_error(d)) return st;
  } else {
    if (int st = forward(d, sb.as<uint64_t>(), n, true)) return st;
    if (int st = backward(d, sb.as<uint64_t>(), n, ta.as<float>(), ts.as<float>(), loss)) return st;
  }
  if (grads) SED_TRY_CUDA(cudaMemcpyAsync(grads, d.g.ptr, d.n_params * 4, cudaMemcpyDefault, d.stream));
  SED_TRY_CUDA(cudaStreamSynchronize(d.stream));
  return LS_SUCCESS;
}

int sed_mlp_train(sed_mlp* m, uint64_t const* states, float const* t_abs, float const* t_sign, uint64_t n,
                  unsigned epochs, unsigned batch, float lr, uint64_t seed, double* final_loss) {
  if (!m || !n || !states || !t_abs || !t_sign || !batch || !(lr > 0.0f))
    return fail(LS_INVALID_ARGUMENT, "sed_mlp_train: bad argument");
  if (batch > (1u << 20)) return fail(LS_INVALID_ARGUMENT, "sed_mlp_train: batch must be <= 2^20");
  MlpData& d = m->d;
  ScopedDevice dev(d.device);
  if (int st = wait_for_caller({states, t_abs, t_sign})) return st;
  uint64_t const bsz = std::min<uint64_t>(batch, n);
  uint64_t const nb = n / bsz;
  double loss = 0.0;
  auto adam = [&](__nv_bfloat16* w1p) -> int {
    ++d.step;
    float const c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)d.step)));
    float const c2 = (float)(1.0 / (1.0 - std::pow(0.999, (double)d.step)));
    dim3 const grid(blocks_for((int64_t)d.n_params));
    if (w1p) {  // tensor-core step (it rewrites the whole gradient)
      SED_TRY_CUDA(launch_pdl(k_adam, grid, dim3(256), 0, d.stream, d.p.as<float>(), d.g.as<float>(), d.m.as<float>(), d.v.as<float>(), d.pb.as<__nv_bfloat16>(), (int64_t)d.n_params, lr, c1, c2, w1p, (int)d.n_in, (int64_t)d.hidden * d.n_in, false));
    } else {
      k_adam<<<grid, 256, 0, d.stream>>>(d.p.as<float>(), d.g.as<float>(), d.m.as<float>(), d.v.as<float>(), d.pb.as<__nv_bfloat16>(), (int64_t)d.n_params, lr, c1, c2, nullptr, (int)d.n_in, (int64_t)0, false);
    }
    note_launches(1);
    return LS_SUCCESS;
  };
  if (d.n_sites && n >= (1ull << 31))
    return fail(LS_INVALID_ARGUMENT, "sed_mlp_train: a patch network trains on at most 2^31 - 1 samples");
  if (d.n_sites && tc_rows(d, std::min<uint64_t>(batch, n)) > kTcMaxRows)
    return fail(LS_INVALID_ARGUMENT, "sed_mlp_train: batch x sites exceeds " + std::to_string(kTcMaxRows) + " rows");
  if (tc_eligible(d) && n < (1ull << 31)) {
    // tensor cores: the samples stay on the device; each epoch draws its
    // batches in the order of a keyed permutation (k_perm, keys from
    // mt19937_64(seed)) made on the device
    DeviceBuffer sb, ta, ts, perm;
    if (int st = stage(sb, states, n * 8, d.stream)) return st;
    if (int st = stage(ta, t_abs, n * 4, d.stream)) return st;
    if (int st = stage(ts, t_sign, n * 4, d.stream)) return st;
    if (int st = perm.allocate(n * 4)) return st;
    if (int st = tc_train_prepare(d, bsz)) return st;
    int half = 1;
    while ((1ull << (2 * half)) < n) ++half;
    std::mt19937_64 rng(seed);
    for (unsigned ep = 0; ep < epochs; ++ep) {
      uint64_t const k01 = rng(), k23 = rng();
      uint4 const key = make_uint4((uint32_t)k01, (uint32_t)(k01 >> 32), (uint32_t)k23, (uint32_t)(k23 >> 32));
      { k_perm<<<blocks_for((int64_t)n), 256, 0, d.stream>>>((uint32_t)n, half, key, perm.as<uint32_t>()); note_launches(1); }
      for (uint64_t bi = 0; bi < nb; ++bi) {
        if (d.n_sites)
          SED_TRY_CUDA(launch_pdl(k_batch_patch, dim3(blocks_for((int64_t)tc_rows(d, bsz) * 8)), dim3(256), 0, d.stream, (uint64_t const*)sb.as<uint64_t>(), (float const*)ta.as<float>(), (float const*)ts.as<float>(), (uint32_t const*)perm.as<uint32_t>(), bi * bsz, (int64_t)bsz, (int)d.n_sites, (int)d.n_in, (uint16_t const*)d.patch_dev.as<uint16_t>(), d.tX.as<__nv_bfloat16>(), d.tState.as<uint64_t>(), d.tAbs.as<float>(), d.tSign.as<float>()));
        else
          SED_TRY_CUDA(launch_pdl(k_batch, dim3(blocks_for((int64_t)bsz * 8)), dim3(256), 0, d.stream, (uint64_t const*)sb.as<uint64_t>(), (float const*)ta.as<float>(), (float const*)ts.as<float>(), (uint32_t const*)perm.as<uint32_t>(), bi * bsz, (int64_t)bsz, (int)d.n_in, d.tX.as<__nv_bfloat16>(), d.tState.as<uint64_t>(), d.tAbs.as<float>(), d.tSign.as<float>()));
        note_launches(1);
        bool const last = ep + 1 == epochs && bi + 1 == nb;
        if (int st = tc_train_step(d, bsz, last ? &loss : nullptr)) return st;
        if (int st = adam(d.tW1p.as<__nv_bfloat16>())) return st;
      }
      SED_TRY_CUDA(cudaGetLastError());
    }
    d.img_valid = false;
    if (int st = tc_check_error(d)) return st;
    if (final_loss) *final_loss = loss;
    return LS_SUCCESS;
  }
  // CUDA cores: the data set is shuffled on the host once per epoch (an index
  // permutation from mt19937_64(seed)) and uploaded; batches are contiguous
  // slices of it
  std::vector<uint64_t> hs(n);
  std::vector<float> ha(n), hg(n);
  SED_TRY_CUDA(cudaMemcpy(hs.data(), states, n * 8, cudaMemcpyDefault));
  SED_TRY_CUDA(cudaMemcpy(ha.data(), t_abs, n * 4, cudaMemcpyDefault));
  SED_TRY_CUDA(cudaMemcpy(hg.data(), t_sign, n * 4, cudaMemcpyDefault));
  DeviceBuffer sb, ta, ts;
  if (int st = sb.allocate(n * 8)) return st;
  if (int st = ta.allocate(n * 4)) return st;
  if (int st = ts.allocate(n * 4)) return st;
  std::vector<uint64_t> order(n);
  for (uint64_t q = 0; q < n; ++q) order[q] = q;
  std::mt19937_64 rng(seed);
  std::vector<uint64_t> bs(n);
  std::vector<float> ba(n), bg(n);
  for (unsigned ep = 0; ep < epochs; ++ep) {
    std::shuffle(order.begin(), order.end(), rng);
    for (uint64_t q = 0; q < n; ++q) {
      bs[q] = hs[order[q]];
      ba[q] = ha[order[q]];
      bg[q] = hg[order[q]];
    }
    SED_TRY_CUDA(cudaMemcpyAsync(sb.ptr, bs.data(), n * 8, cudaMemcpyHostToDevice, d.stream));
    SED_TRY_CUDA(cudaMemcpyAsync(ta.ptr, ba.data(), n * 4, cudaMemcpyHostToDevice, d.stream));
    SED_TRY_CUDA(cudaMemcpyAsync(ts.ptr, bg.data(), n * 4, cudaMemcpyHostToDevice, d.stream));
    for (uint64_t bi = 0; bi < nb; ++bi) {
      uint64_t const b0 = bi * bsz;
      if (int st = forward(d, sb.as<uint64_t>() + b0, bsz, true)) return st;
      bool const last = ep + 1 == epochs && bi + 1 == nb;
      if (int st = backward(d, sb.as<uint64_t>() + b0, bsz, ta.as<float>() + b0, ts.as<float>() + b0,
                            last ? &loss : nullptr))
        return st;
      if (int st = adam(nullptr)) return st;
    }
    d.img_valid = false;
    SED_TRY_CUDA(cudaGetLastError());
    // the host staging buffers are rewritten next epoch: wait for the uploads
    SED_TRY_CUDA(cudaStreamSynchronize(d.stream));
  }
  if (final_loss) *final_loss = loss;
  return LS_SUCCESS;
}

int sed_mlp_sample(ls_spin_basis const* basis, double const* psi, uint64_t n, uint64_t seed, uint64_t sign_mask,
                   uint64_t* states, float* t_abs, float* t_sign) {
  if (!basis || !psi || (n && (!states || !t_abs || !t_sign)))
    return fail(LS_INVALID_ARGUMENT, "sed_mlp_sample: NULL argument");
  BasisData& b = *basis->d;
  if (!b.built) return fail(LS_CACHE_NOT_BUILT, "basis has not been built (call ls_build)");
  if (b.D == 0) return fail(LS_INVALID_ARGUMENT, "sed_mlp_sample: empty basis");
  if (n == 0) return LS_SUCCESS;
  ScopedDevice dev(b.device);
  if (int st = wait_for_caller({psi, states, t_abs, t_sign})) return st;
  cudaStream_t s = nullptr;
  SED_TRY_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } guard{s};
  uint64_t const D = b.D, chunks = (D + kChunk - 1) / kChunk;
  DeviceBuffer dpsi, sums, offs, prefix, os, oa, og;
  if (int st = stage(dpsi, psi, D * 8, s)) return st;
  if (int st = sums.allocate(2 * chunks * 8)) return st;
  if (int st = offs.allocate(chunks * 8)) return st;
  if (int st = prefix.allocate(D * 8)) return st;
  if (int st = os.allocate(n * 8)) return st;
  if (int st = oa.allocate(n * 4)) return st;
  if (int st = og.allocate(n * 4)) return st;
  { k_chunk_sums<<<(unsigned)chunks, 256, 0, s>>>(dpsi.as<double>(), b.reps.as<uint64_t>(), D, sign_mask, sums.as<double>()); note_launches(1); }
  std::vector<double> hs(2 * chunks);
  SED_TRY_CUDA(cudaMemcpyAsync(hs.data(), sums.ptr, 2 * chunks * 8, cudaMemcpyDeviceToHost, s));
  SED_TRY_CUDA(cudaStreamSynchronize(s));
  double total = 0.0, agree = 0.0;
  for (uint64_t c = 0; c < chunks; ++c) {
    double const t = hs[c];
    hs[c] = total;
    total += t;
    agree += hs[chunks + c];
  }
  hs.resize(chunks);
  double const sign = agree < 0.0 ? -1.0 : 1.0;
  if (!(total > 0.0) || !std::isfinite(total))
    return fail(LS_INVALID_ARGUMENT, "sed_mlp_sample: psi has no finite nonzero weight");
  SED_TRY_CUDA(cudaMemcpyAsync(offs.ptr, hs.data(), chunks * 8, cudaMemcpyHostToDevice, s));
  { k_chunk_prefix<<<(unsigned)chunks, 256, 0, s>>>(dpsi.as<double>(), D, offs.as<double>(), prefix.as<double>()); note_launches(1); }
  // draw below the last prefix value, which may differ from total by rounding
  double last = 0.0;
  SED_TRY_CUDA(cudaMemcpyAsync(&last, prefix.as<double>() + (D - 1), 8, cudaMemcpyDeviceToHost, s));
  SED_TRY_CUDA(cudaStreamSynchronize(s));
  { k_draw<<<blocks_for((int64_t)n), 256, 0, s>>>(prefix.as<double>(), D, last, n, seed, sign, dpsi.as<double>(), b.reps.as<uint64_t>(), b.weights.as<uint32_t>(), (double)b.plan.group_order, os.as<uint64_t>(), oa.as<float>(), og.as<float>()); note_launches(1); }
  SED_TRY_CUDA(cudaGetLastError());
  SED_TRY_CUDA(cudaMemcpyAsync(states, os.ptr, n * 8, cudaMemcpyDefault, s));
  SED_TRY_CUDA(cudaMemcpyAsync(t_abs, oa.ptr, n * 4, cudaMemcpyDefault, s));
  SED_TRY_CUDA(cudaMemcpyAsync(t_sign, og.ptr, n * 4, cudaMemcpyDefault, s));
  SED_TRY_CUDA(cudaStreamSynchronize(s));
  return LS_SUCCESS;
}

int sed_mlp_start_vector(sed_mlp* m, ls_spin_basis const* basis, double* out) {
  if (!m || !basis || !out) return fail(LS_INVALID_ARGUMENT, "sed_mlp_start_vector: NULL argument");
  MlpData& d = m->d;
  BasisData& b = *basis->d;
  if (!b.built) return fail(LS_CACHE_NOT_BUILT, "basis has not been built (call ls_build)");
  if (d.n_sites ? b.n != d.n_sites : b.n != d.n_in)
    return fail(LS_DIMENSION_MISMATCH, d.n_sites ? "sed_mlp_start_vector: patch table sites != number of spins"
                                                 : "sed_mlp_start_vector: network inputs != number of spins");
  if (b.D == 0) return LS_SUCCESS;
  ScopedDevice dev(d.device);
  if (int st = wait_for_caller({out})) return st;
  uint64_t const D = b.D, chunk = 1u << 18;
  DeviceBuffer amp, part, vout;
  if (int st = amp.allocate(D * 8)) return st;  // (a, s) pairs
  if (int st = part.allocate(152 * 16 * 4)) return st;
  if (d.n_sites && !fused_shape(d)) {
    if (int st = forward_patch(d, b.reps.as<uint64_t>(), D, amp.as<float>())) return st;
  } else if (tc_eligible(d)) {
    if (int st = forward_tc(d, b.reps.as<uint64_t>(), D, amp.as<float>())) return st;
  } else {
    for (uint64_t b0 = 0; b0 < D; b0 += chunk) {
      uint64_t const nb = std::min(chunk, D - b0);
      if (int st = forward(d, b.reps.as<uint64_t>() + b0, nb, false)) return st;
      SED_TRY_CUDA(cudaMemcpyAsync(amp.as<float>() + 2 * b0, d.out.ptr, nb * 8, cudaMemcpyDeviceToDevice, d.stream));
    }
  }
  unsigned const lb = blocks_for((int64_t)D);
  { k_max_first<<<lb, 256, 0, d.stream>>>(amp.as<float>(), (int64_t)D, part.as<float>()); note_launches(1); }
  std::vector<float> hp(lb);
  SED_TRY_CUDA(cudaMemcpyAsync(hp.data(), part.ptr, lb * 4, cudaMemcpyDeviceToHost, d.stream));
  SED_TRY_CUDA(cudaStreamSynchronize(d.stream));
  float amax = -3.0e38f;
  for (float q : hp) amax = std::max(amax, q);
  cudaPointerAttributes attr{};
  bool const dev_out = cudaPointerGetAttributes(&attr, out) == cudaSuccess &&
                       (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged);
  (void)cudaGetLastError();
  double* dst = out;
  if (!dev_out) {
    if (int st = vout.allocate(D * 8)) return st;
    dst = vout.as<double>();
  }
  { k_start_from_net<<<lb, 256, 0, d.stream>>>(amp.as<float>(), b.reps.as<uint64_t>(), b.weights.as<uint32_t>(), (int64_t)D, d.sign_mask, amax, (double)b.plan.group_order, dst); note_launches(1); }
  SED_TRY_CUDA(cudaGetLastError());
  if (!dev_out) SED_TRY_CUDA(cudaMemcpyAsync(out, dst, D * 8, cudaMemcpyDeviceToHost, d.stream));
  SED_TRY_CUDA(cudaStreamSynchronize(d.stream));
  return LS_SUCCESS;
}

}  // extern "C"
