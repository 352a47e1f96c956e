// batch.cu — many Hamiltonians of uneven size solved in one persistent launch
// (sed_eigh_batched): the lowest nev <= 4 eigenpairs of every operator by
// block Lanczos with block size 4. Vectors are stored in FP64; the products
// of the block SpMV, the Gram-Schmidt passes, CholQR2 and the Ritz vectors
// run in double-float arithmetic on the FP32 pipe (df.cuh); norms, the
// Rayleigh-Ritz solve and the true residuals are FP64.
//
// One cooperative kernel runs the whole solve for all problems. Its CTAs are
// split into groups (batch_layout: large problems get several CTAs, small
// ones share one-CTA groups and are solved one after another), and a group
// synchronises through a bounded barrier in global memory. Within a group
// the rows of the problem are split by SELL-32 slices.
//
// Per problem, with Krylov blocks V_j stored row-interleaved ([D][4], so the
// SpMV gathers one 32-byte sector per element for all four columns):
//   V_0 = QR(start block)                                  (CholQR2)
//   W = H V_j ; C_i = V_i^T W, W -= V_i C_i for i <= j      (CGS2, two passes)
//   W = V_{j+1} B_j                                          (CholQR2)
//   T: diagonal blocks A_j = sym(C_j), sub-diagonal blocks B_j
// Every `rr_every` steps (and at the end of a cycle) the group's first CTA
// diagonalises T (cyclic Jacobi with parallel round-robin rotations in shared
// memory) and estimates the Ritz residuals ||B_j y_last||; the cycle ends when
// all nev estimates are below tol / 2 or the basis is full. Ritz vectors
// Psi = V Y are then formed, their true residuals ||H psi - theta psi|| are
// computed, and the problem is done when all are below tol; otherwise block
// Lanczos restarts from Psi.
//
// Cross-CTA data (partial sums, T, decisions, the gathered x of the SpMV) is
// read with ld.global.cg so that no stale L1 line is used after a barrier.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <mutex>
#include <numeric>
#include <tuple>
#include <vector>

#include "operator_impl.cuh"
#include "df.cuh"
#include "tc.cuh"

namespace sed {
namespace {

constexpr int kB = 4;               // block size
constexpr int kMaxBlocks = 16;      // stored Krylov blocks per cycle (n <= 64)
constexpr int kMaxN = kB * kMaxBlocks;
constexpr int kPart = 16 * (kMaxBlocks + 1);  // partial sums per CTA and slot
constexpr int kGsStages = 4;                   // shared-memory stages of the Gram-Schmidt row streams
constexpr uint64_t kGsWaitNs = 1000000000ull;  // default bound on a wait for one stage's copies (1 s)
constexpr uint64_t kBarrierNs = 20000000000ull;  // default: 20 s per barrier, far beyond any phase
// Part of a block step that more CTAs do not shorten, in rows of the mean
// work per row (the group layout's model). Fitted on 128 J1-J2 chains
// (N = 16..28, problems alone in their groups): a block step took 0.25 ms
// plus 0.18 us per row of the CTA's share, i.e. about 1400 rows.
constexpr double kLayoutFixedRows = 1400.0;
constexpr size_t kStatsOff = 12 * 8;                // per-problem output record: out[12], stats[4], flag[4], prof[8]
constexpr size_t kProfOff = kStatsOff + 32;
constexpr size_t kOutBytes = kProfOff + 64;

struct ChainDesc {
  StreamView S;       // real operator, FP64 stream form
  uint64_t D, n_slices;
  double* V;          // (m_blocks + 1) blocks of [D][4]
  float* Vs;          // V split into double-float rows (Row4s), for the Gram-Schmidt products
  float* Xs;          // [D] Row4s: the block under Gram-Schmidt, in double-float
  float2* table_s;    // [n_codes]: the matrix-element table split into double-float (k_split_tables)
  double* W;          // [D][4]
  double* part;       // [2][ncta][kPart]
  double* W2;         // [D][4] second scratch block (thick restart)
  double* Tc;         // [kMaxBlocks][kMaxN * 4]: step j's projections C_i = V_i^T H V_j, i <= j
  double* Bblk;       // [kMaxBlocks][16] sub-diagonal blocks (upper triangular)
  double* Y;          // [kMaxN][8] Ritz vectors of T (row q, column i)
  double* out;        // theta[8], residual[4]
  uint32_t* stats;    // block steps, restarts, matvecs, status (0 running, 1 done, 2 not converged, 3 breakdown)
  uint32_t* flag;     // [4]: decision words written by the leader CTA
  uint64_t* prof;     // [8] nanoseconds per phase on the leader CTA: spmv, cgs2, qr, rayleigh-ritz, ritz+restart, residual
  uint32_t m_blocks;
  uint32_t nev;
  uint32_t packed;    // stream entries hold col | code << col_bits
  uint64_t seed;
};

struct GroupDesc {
  uint32_t cta0, ncta, first, count;  // CTAs [cta0, cta0 + ncta); chains order[first .. first + count)
  uint32_t* bar;                      // [2]: arrivals, generation
};

struct BatchArgs {
  ChainDesc const* chains;
  GroupDesc const* groups;
  uint32_t const* cta_group;
  uint32_t const* order;
  double tol;
  uint32_t max_steps;     // block steps per problem in total
  uint32_t rr_every;
  int* error;
  uint64_t wait_ns;        // bound on every barrier wait
  uint64_t copy_wait_ns;   // bound on every wait for a row-stream stage's copies
  uint32_t extra_arrivals; // arrivals a barrier waits for beyond its CTAs (0; see sed_debug_barrier_extra_arrivals)
};

// One row of a [D][4] block (32 bytes, one sector).
struct alignas(32) Row4 {
  double x, y, z, w;
};
__device__ __forceinline__ Row4 mk4(double a, double b, double c, double d) { return Row4{a, b, c, d}; }

__device__ __forceinline__ double ldcg(double const* p) { return __ldcg(p); }
__device__ __forceinline__ uint32_t ldcg(uint32_t const* p) { return __ldcg(p); }
__device__ __forceinline__ Row4 ldcg4(double const* p) {
  double2 const a = __ldcg(reinterpret_cast<double2 const*>(p));
  double2 const b = __ldcg(reinterpret_cast<double2 const*>(p) + 1);
  return mk4(a.x, a.y, b.x, b.y);
}

// Rows of split blocks for the double-float Gram-Schmidt products (df.cuh).
struct alignas(32) Row4s {
  float4 h, l;  // a [D][4] row: hi parts, then lo parts
};

__device__ __forceinline__ Row4s split_row(Row4 const& r) {
  Row4s o;
  df_split(r.x, o.h.x, o.l.x);
  df_split(r.y, o.h.y, o.l.y);
  df_split(r.z, o.h.z, o.l.z);
  df_split(r.w, o.h.w, o.l.w);
  return o;
}

// (S, E)[s][t] += a_s w_t over one row of a split block a and of X.
__device__ __forceinline__ void df_dots(Row4s const& a, Row4s const& w, float (&S)[16], float (&E)[16]) {
  float const ah[4] = {a.h.x, a.h.y, a.h.z, a.h.w}, al[4] = {a.l.x, a.l.y, a.l.z, a.l.w};
  float const wh[4] = {w.h.x, w.h.y, w.h.z, w.h.w}, wl[4] = {w.l.x, w.l.y, w.l.z, w.l.w};
#pragma unroll
  for (int s = 0; s < 4; ++s)
#pragma unroll
    for (int t = 0; t < 4; ++t) df_mac(ah[s], al[s], wh[t], wl[t], S[s * 4 + t], E[s * 4 + t]);
}

// (S, E)[t] += sum_s a_s c[s][t] for one split row a and 4 x 4 split
// coefficients (c4h, c4l: row s as one float4 each).
__device__ __forceinline__ void df_axpy(Row4s const& a, float4 const* c4h, float4 const* c4l, float (&S)[4],
                                        float (&E)[4]) {
  float const ah[4] = {a.h.x, a.h.y, a.h.z, a.h.w}, al[4] = {a.l.x, a.l.y, a.l.z, a.l.w};
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    float4 const h = c4h[s], l = c4l[s];
    df_mac(ah[s], al[s], h.x, l.x, S[0], E[0]);
    df_mac(ah[s], al[s], h.y, l.y, S[1], E[1]);
    df_mac(ah[s], al[s], h.z, l.z, S[2], E[2]);
    df_mac(ah[s], al[s], h.w, l.w, S[3], E[3]);
  }
}

// row -= (S + E), column by column.
__device__ __forceinline__ void df_sub_row(Row4s& row, float const (&S)[4], float const (&E)[4]) {
  Row4s w = row;
  df_sub(w.h.x, w.l.x, S[0], E[0]);
  df_sub(w.h.y, w.l.y, S[1], E[1]);
  df_sub(w.h.z, w.l.z, S[2], E[2]);
  df_sub(w.h.w, w.l.w, S[3], E[3]);
  row = w;
}

// Bounded barrier of the `n` CTAs of a group; false if it timed out (then
// *error = 2) or another CTA has already reported an error, which ends the
// wait early. Every thread of the CTA must call it.
__device__ bool group_barrier(uint32_t* bar, uint32_t n, BatchArgs const& a) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    uint32_t const need = n + a.extra_arrivals;
    if (need > 1) {
      volatile uint32_t* gen = bar + 1;
      uint32_t const g = *gen;
      __threadfence();
      if (atomicAdd(bar, 1u) == need - 1) {
        atomicExch(bar, 0u);
        __threadfence();
        atomicAdd(bar + 1, 1u);
      } else {
        uint64_t const t0 = tc::global_ns();
        while (*gen == g) {
          if (*(volatile int*)a.error) {
            ok = 0;
            break;
          }
          if (tc::global_ns() - t0 > a.wait_ns) {
            ok = 0;
            atomicExch(a.error, 2);
            break;
          }
          __nanosleep(64);
        }
      }
      __threadfence();
    }
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// Sums K per-thread values over the CTA; thread k < K of the CTA gets total k
// in out[k] (shared). red: [warps][K] shared scratch.
template <int K>
__device__ __forceinline__ void cta_sum(double (&v)[K], double* red, double* out) {
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp * K + k] = x;
  }
  __syncthreads();
  if ((int)threadIdx.x < K) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += red[w * K + threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

struct Ctx {
  ChainDesc const& c;
  uint32_t rank, ncta;
  uint32_t* bar;
  BatchArgs const* args;
  uint64_t r0, r1;      // own rows
  uint64_t s0, s1;      // own slices
  uint32_t slot;        // partial-sum double buffer
  double* red;          // shared [warps][16]
  double* tmp;          // shared [kPart]
  double* dyn;          // the dynamic shared area (row-stream stages outside the Jacobi solve)
  uint64_t* gs_bar;     // shared [kGsStages] mbarriers of the row streams
  uint32_t* gs_phase;   // parity bit per mbarrier (same value in every thread)
};

// Publishes this CTA's K partial sums (in shared `local`), waits for the group
// and leaves the group totals in shared `total` (same order on every CTA).
__device__ bool group_sum(Ctx& x, double const* local, int K, double* total) {
  double* mine = x.c.part + ((size_t)x.slot * x.ncta + x.rank) * kPart;
  for (int k = threadIdx.x; k < K; k += blockDim.x) mine[k] = local[k];
  __threadfence();
  if (!group_barrier(x.bar, x.ncta, *x.args)) return false;
  double const* all = x.c.part + (size_t)x.slot * x.ncta * kPart;
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    double s = 0.0;
    for (uint32_t r = 0; r < x.ncta; ++r) s += ldcg(all + (size_t)r * kPart + k);
    total[k] = s;
  }
  x.slot ^= 1u;
  __syncthreads();
  return true;
}

// Cholesky of the 4x4 Gram matrix G (row-major) -> upper R with G = R^T R.
// Returns false on a pivot below eps * trace (rank deficiency).
__device__ bool chol4(double const* G, double* R) {
  double const tr = G[0] + G[5] + G[10] + G[15];
  for (int i = 0; i < 16; ++i) R[i] = 0.0;
  for (int j = 0; j < 4; ++j) {
    double d = G[j * 4 + j];
    for (int k = 0; k < j; ++k) d -= R[k * 4 + j] * R[k * 4 + j];
    if (!(d > 1e-24 * tr) || !(tr > 0.0)) return false;
    double const rjj = sqrt(d);
    R[j * 4 + j] = rjj;
    for (int i = j + 1; i < 4; ++i) {
      double s = G[j * 4 + i];
      for (int k = 0; k < j; ++k) s -= R[k * 4 + j] * R[k * 4 + i];
      R[j * 4 + i] = s / rjj;
    }
  }
  return true;
}

// In place X <- X R^{-1} on own rows (X = [D][4]); y R = x by forward
// substitution, dividing by the diagonal through its reciprocals (four FP64
// divisions per CTA instead of four per row: a division is a long sequence
// on GB300's narrow FP64 pipe).
__device__ void apply_rinv(Ctx& x, double* X, double const* R) {
  double const inv[4] = {1.0 / R[0], 1.0 / R[5], 1.0 / R[10], 1.0 / R[15]};
  for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += blockDim.x) {
    Row4 const v = *reinterpret_cast<Row4 const*>(X + r * 4);
    double const a[4] = {v.x, v.y, v.z, v.w};
    double y[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      double s = a[j];
#pragma unroll
      for (int k = 0; k < j; ++k) s -= y[k] * R[k * 4 + j];
      y[j] = s * inv[j];
    }
    *reinterpret_cast<Row4*>(X + r * 4) = mk4(y[0], y[1], y[2], y[3]);
  }
}

// CholQR2 of the block X in place; Rtot (shared, 16) = R2 R1. false on
// breakdown or barrier failure (ok distinguishes them).
__device__ bool block_qr(Ctx& x, double* X, double* Rtot, bool& ok) {
  __shared__ double G[16], R[16], P[16];
  ok = true;
  for (int pass = 0; pass < 2; ++pass) {
    double g[10] = {};
    for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += blockDim.x) {
      Row4 const v = *reinterpret_cast<Row4 const*>(X + r * 4);
      double const a[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = i; j < 4; ++j) {
          int const q = i * 4 - i * (i - 1) / 2 + (j - i);  // packed upper triangle
          g[q] = fma(a[i], a[j], g[q]);
        }
    }
    cta_sum<10>(g, x.red, x.tmp);
    if (!group_sum(x, x.tmp, 10, x.tmp + 16)) {
      ok = false;
      return false;
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < 4; ++i)
        for (int j = i; j < 4; ++j) {
          int const q = i * 4 - i * (i - 1) / 2 + (j - i);
          G[i * 4 + j] = G[j * 4 + i] = x.tmp[16 + q];
        }
    }
    __syncthreads();
    __shared__ int good;
    if (threadIdx.x == 0) good = chol4(G, R) ? 1 : 0;
    __syncthreads();
    if (!good) return false;
    apply_rinv(x, X, R);
    if (threadIdx.x == 0) {
      if (pass == 0) {
        for (int i = 0; i < 16; ++i) Rtot[i] = R[i];
      } else {  // Rtot = R2 * R1
        for (int i = 0; i < 4; ++i)
          for (int j = 0; j < 4; ++j) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += R[i * 4 + k] * Rtot[k * 4 + j];
            P[i * 4 + j] = s;
          }
        for (int i = 0; i < 16; ++i) Rtot[i] = P[i];
      }
    }
    __syncthreads();
  }
  return true;
}

// CholQR2 of the block X in double-float: on entry Xs holds X split (as
// cgs2 leaves it); the Gram matrices and X R^{-1} run on the split rows, and
// on exit X (FP64) and the split copy Vs_out (may be null) hold the factor Q.
// Rtot (shared, 16) = R2 R1; false on breakdown or barrier failure (ok
// distinguishes them).
__device__ bool block_qr_df(Ctx& x, double* X, Row4s* Vs_out, double* Rtot, bool& ok) {
  __shared__ double G[16], R[16], P[16];
  __shared__ float Rh[16], Rl[16];
  Row4s* Xs = reinterpret_cast<Row4s*>(x.c.Xs);
  ok = true;
  for (int pass = 0; pass < 2; ++pass) {
    float S[10] = {}, E[10] = {};
    for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += blockDim.x) {
      Row4s const v = Xs[r];
      float const ah[4] = {v.h.x, v.h.y, v.h.z, v.h.w}, al[4] = {v.l.x, v.l.y, v.l.z, v.l.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = i; j < 4; ++j) {
          int const q = i * 4 - i * (i - 1) / 2 + (j - i);  // packed upper triangle
          df_mac(ah[i], al[i], ah[j], al[j], S[q], E[q]);
        }
    }
    double g[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) g[q] = (double)S[q] + (double)E[q];
    cta_sum<10>(g, x.red, x.tmp);
    if (!group_sum(x, x.tmp, 10, x.tmp + 16)) {
      ok = false;
      return false;
    }
    if (threadIdx.x == 0) {
      for (int i = 0; i < 4; ++i)
        for (int j = i; j < 4; ++j) {
          int const q = i * 4 - i * (i - 1) / 2 + (j - i);
          G[i * 4 + j] = G[j * 4 + i] = x.tmp[16 + q];
        }
    }
    __syncthreads();
    __shared__ int good;
    if (threadIdx.x == 0) {
      good = chol4(G, R) ? 1 : 0;
      if (good) {
        // R's off-diagonal entries and the reciprocals of its diagonal, split
        for (int i = 0; i < 16; ++i) {
          double const v = (i % 5 == 0) ? 1.0 / R[i] : R[i];
          df_split(v, Rh[i], Rl[i]);
        }
      }
    }
    __syncthreads();
    if (!good) return false;
    // X <- X R^{-1}: y_j = (x_j - sum_{k<j} y_k R_kj) / R_jj
    for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += blockDim.x) {
      Row4s const v = Xs[r];
      float yh[4] = {v.h.x, v.h.y, v.h.z, v.h.w}, yl[4] = {v.l.x, v.l.y, v.l.z, v.l.w};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
#pragma unroll
        for (int k = 0; k < j; ++k) {
          float ph, pl;
          df_mul(yh[k], yl[k], Rh[k * 4 + j], Rl[k * 4 + j], ph, pl);
          df_sub(yh[j], yl[j], ph, pl);
        }
        df_mul(yh[j], yl[j], Rh[j * 5], Rl[j * 5], yh[j], yl[j]);
      }
      Row4s o;
      o.h = make_float4(yh[0], yh[1], yh[2], yh[3]);
      o.l = make_float4(yl[0], yl[1], yl[2], yl[3]);
      Xs[r] = o;
    }
    if (threadIdx.x == 0) {
      if (pass == 0) {
        for (int i = 0; i < 16; ++i) Rtot[i] = R[i];
      } else {  // Rtot = R2 * R1
        for (int i = 0; i < 4; ++i)
          for (int j = 0; j < 4; ++j) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += R[i * 4 + k] * Rtot[k * 4 + j];
            P[i * 4 + j] = s;
          }
        for (int i = 0; i < 16; ++i) Rtot[i] = P[i];
      }
    }
    __syncthreads();
  }
  for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += blockDim.x) {
    Row4s const w = Xs[r];
    *reinterpret_cast<Row4*>(X + r * 4) = mk4((double)w.h.x + (double)w.l.x, (double)w.h.y + (double)w.l.y,
                                              (double)w.h.z + (double)w.l.z, (double)w.h.w + (double)w.l.w);
    if (Vs_out) Vs_out[r] = w;
  }
  tc::fence_proxy_async_global();  // Vs_out is read by the row streams
  __syncthreads();
  return true;
}

constexpr int kBlockSpmvU = 4;  // slots whose gathers a lane issues together

// W = H X on own rows (X, W: [D][4]); gathers of X go through L2.
__device__ void block_spmv(Ctx& x, double const* X, double* W) {
  StreamView const& S = x.c.S;
  uint32_t const lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t const col_mask = S.col_bits < 32 ? ((1u << S.col_bits) - 1u) : 0xFFFFFFFFu;
  bool const packed = x.c.packed != 0;
  double const* table = static_cast<double const*>(S.table);
  for (uint64_t s = x.s0 + warp; s < x.s1; s += nw) {
    uint64_t const base = S.slice_ptr[s];
    uint32_t const width = (uint32_t)((S.slice_ptr[s + 1] - base) >> 5);
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    uint32_t const* ent = S.entries + base + lane;
    // kBlockSpmvU slots per step: their entry loads (issued one step ahead),
    // then their gathers, then the FMAs in slot order (the same order as one
    // slot at a time), so several gathers are in flight per lane
    uint32_t v[kBlockSpmvU];
#pragma unroll
    for (int u = 0; u < kBlockSpmvU; ++u) v[u] = (uint32_t)u < width ? __ldcs(ent + (uint64_t)u * 32) : kNull;
    for (uint32_t e0 = 0; e0 < width; e0 += kBlockSpmvU) {
      uint32_t vn[kBlockSpmvU];
#pragma unroll
      for (int u = 0; u < kBlockSpmvU; ++u)
        vn[u] = e0 + kBlockSpmvU + u < width ? __ldcs(ent + (uint64_t)(e0 + kBlockSpmvU + u) * 32) : kNull;
      double t[kBlockSpmvU];
      Row4 xv[kBlockSpmvU];
#pragma unroll
      for (int u = 0; u < kBlockSpmvU; ++u) {
        if (v[u] != kNull) {
          uint32_t const col = v[u] & col_mask;
          uint32_t const code =
              packed ? (v[u] >> S.col_bits) : (uint32_t)__ldcs(S.codes + base + lane + (uint64_t)(e0 + u) * 32);
          t[u] = __ldg(table + code);
          xv[u] = ldcg4(X + (uint64_t)col * 4);
        } else {
          t[u] = 0.0;
          xv[u] = mk4(0.0, 0.0, 0.0, 0.0);
        }
      }
#pragma unroll
      for (int u = 0; u < kBlockSpmvU; ++u) {
        if (v[u] == kNull) continue;
        a0 = fma(t[u], xv[u].x, a0);
        a1 = fma(t[u], xv[u].y, a1);
        a2 = fma(t[u], xv[u].z, a2);
        a3 = fma(t[u], xv[u].w, a3);
      }
#pragma unroll
      for (int u = 0; u < kBlockSpmvU; ++u) v[u] = vn[u];
    }
    uint64_t const i = s * 32 + lane;
    if (i < x.c.D) {
      double const f = S.inv_sqrt_s[S.row_class[i]];
      double const dg = static_cast<double const*>(S.diag)[i];
      Row4 const xi = ldcg4(X + i * 4);
      *reinterpret_cast<Row4*>(W + i * 4) =
          mk4(fma(f, a0, dg * xi.x), fma(f, a1, dg * xi.y), fma(f, a2, dg * xi.z), fma(f, a3, dg * xi.w));
    }
  }
}

// ------------------------------------------- Gram-Schmidt row streams ---
// The Gram-Schmidt products read the CTA's own rows of split blocks (Vs, Xs)
// in tiles of 2 blockDim rows, copied into the dynamic shared area by bulk
// asynchronous copies (one thread issues them; mbarriers count their bytes)
// a few tiles ahead of the arithmetic, so the loads' latency is hidden
// behind the products instead of stalling each warp once per row. Waits are
// bounded (copy_wait_ns): a copy that does not arrive sets the launch's error
// flag; thread 0 then waits (bounded) for the CTA's copies still in flight
// and the solve returns.

// Waits for stage barrier q (every thread) and flips its parity.
__device__ bool gs_wait(Ctx& x, uint32_t q) {
  bool const ok = tc::mbar_wait(&x.gs_bar[q], (*x.gs_phase >> q) & 1u, x.args->copy_wait_ns);
  *x.gs_phase ^= 1u << q;
  return ok;
}

// After a failed wait on barrier `failed` (its parity already flipped):
// records the error; thread 0 waits (bounded) for the copies still in
// flight on it and on the barriers in `pending` (bit mask, not yet waited).
__device__ bool gs_abort(Ctx& x, uint32_t failed, uint32_t pending) {
  if (threadIdx.x == 0) {
    atomicExch(x.args->error, 3);
    tc::mbar_wait(&x.gs_bar[failed], ((*x.gs_phase >> failed) & 1u) ^ 1u, x.args->copy_wait_ns);
    for (uint32_t q = 0; q < (uint32_t)kGsStages; ++q)
      if (pending & (1u << q)) tc::mbar_wait(&x.gs_bar[q], (*x.gs_phase >> q) & 1u, x.args->copy_wait_ns);
  }
  for (uint32_t q = 0; q < (uint32_t)kGsStages; ++q)
    if (pending & (1u << q)) *x.gs_phase ^= 1u << q;
  return false;
}

// (S, E) += V_i^T X over own rows (both split): two stages, each a V tile
// and an X tile.
__device__ bool gs_dots(Ctx& x, Row4s const* Vi, Row4s const* Xs, float (&S)[16], float (&E)[16]) {
  uint32_t const TR = 2 * blockDim.x;
  uint64_t const r0 = x.r0, r1 = x.r1;
  uint32_t const ntiles = (uint32_t)((r1 - r0 + TR - 1) / TR);
  Row4s* st = reinterpret_cast<Row4s*>(x.dyn);
  auto rows_of = [&](uint32_t k) { return (uint32_t)min((uint64_t)TR, r1 - (r0 + (uint64_t)k * TR)); };
  auto issue = [&](uint32_t k) {
    uint32_t const q = k & 1u, n = rows_of(k);
    uint64_t const row = r0 + (uint64_t)k * TR;
    tc::mbar_expect_tx(&x.gs_bar[q], 2 * n * (uint32_t)sizeof(Row4s));
    tc::bulk_g2s(st + q * 2 * TR, Vi + row, n * (uint32_t)sizeof(Row4s), &x.gs_bar[q]);
    tc::bulk_g2s(st + q * 2 * TR + TR, Xs + row, n * (uint32_t)sizeof(Row4s), &x.gs_bar[q]);
  };
  tc::fence_proxy_async_smem();  // this thread's shared-memory accesses before the copies' writes
  __syncthreads();               // the stages' previous readers are done
  if (threadIdx.x == 0)
    for (uint32_t k = 0; k < 2 && k < ntiles; ++k) issue(k);
  for (uint32_t k = 0; k < ntiles; ++k) {
    uint32_t const q = k & 1u, n = rows_of(k);
    bool const ok = gs_wait(x, q);
    if (ok) {
      Row4s const* sv = st + q * 2 * TR;
      for (uint32_t r = threadIdx.x; r < n; r += blockDim.x) df_dots(sv[r], sv[TR + r], S, E);
    }
    tc::fence_proxy_async_smem();
    if (__syncthreads_or(!ok)) return gs_abort(x, q, (k + 1 < ntiles ? 1u << ((k + 1) & 1u) : 0u));
    if (threadIdx.x == 0 && k + 2 < ntiles) issue(k + 2);
  }
  return true;
}

// Xs -= sum_{i0 <= i < nb} V_i C_i over own rows, C_i in double-float in
// shared memory (ch, cl: 16 per block); the V tiles stream through
// kGsStages stages, every block of one row tile before the next tile.
__device__ bool gs_update(Ctx& x, Row4s const* Vs, Row4s* Xs, uint32_t i0, uint32_t nb, float const* ch,
                          float const* cl) {
  uint32_t const TR = 2 * blockDim.x;
  uint64_t const r0 = x.r0, r1 = x.r1, D = x.c.D;
  uint32_t const ntiles = (uint32_t)((r1 - r0 + TR - 1) / TR);
  uint32_t const nbb = nb - i0, items = ntiles * nbb;
  Row4s* st = reinterpret_cast<Row4s*>(x.dyn);
  auto rows_of = [&](uint32_t k) { return (uint32_t)min((uint64_t)TR, r1 - (r0 + (uint64_t)k * TR)); };
  auto issue = [&](uint32_t m) {
    uint32_t const k = m / nbb, i = i0 + m % nbb, q = m % kGsStages, n = rows_of(k);
    tc::mbar_expect_tx(&x.gs_bar[q], n * (uint32_t)sizeof(Row4s));
    tc::bulk_g2s(st + q * TR, Vs + (uint64_t)i * D + r0 + (uint64_t)k * TR, n * (uint32_t)sizeof(Row4s),
                 &x.gs_bar[q]);
  };
  tc::fence_proxy_async_smem();
  __syncthreads();
  if (threadIdx.x == 0)
    for (uint32_t m = 0; m < (uint32_t)kGsStages && m < items; ++m) issue(m);
  for (uint32_t k = 0; k < ntiles; ++k) {
    uint32_t const n = rows_of(k);
    uint32_t const ra = threadIdx.x, rb = threadIdx.x + blockDim.x;  // the thread's rows of the tile
    float S0[4] = {}, E0[4] = {}, S1[4] = {}, E1[4] = {};
    for (uint32_t ii = 0; ii < nbb; ++ii) {
      uint32_t const m = k * nbb + ii, q = m % kGsStages;
      bool const ok = gs_wait(x, q);
      if (ok) {
        Row4s const* sv = st + q * TR;
        float4 const* c4h = reinterpret_cast<float4 const*>(ch + 16 * (i0 + ii));
        float4 const* c4l = reinterpret_cast<float4 const*>(cl + 16 * (i0 + ii));
        if (ra < n) df_axpy(sv[ra], c4h, c4l, S0, E0);
        if (rb < n) df_axpy(sv[rb], c4h, c4l, S1, E1);
      }
      tc::fence_proxy_async_smem();
      if (__syncthreads_or(!ok)) {
        uint32_t pending = 0;
        for (uint32_t p = m + 1; p < items && p < m + kGsStages; ++p) pending |= 1u << (p % kGsStages);
        return gs_abort(x, q, pending);
      }
      if (threadIdx.x == 0 && m + kGsStages < items) issue(m + kGsStages);
    }
    uint64_t const row = r0 + (uint64_t)k * TR;
    if (ra < n) df_sub_row(Xs[row + ra], S0, E0);
    if (rb < n) df_sub_row(Xs[row + rb], S1, E1);
  }
  tc::fence_proxy_async_global();  // the next pass's streams read Xs
  __syncthreads();
  return true;
}

// W = H V_j on own rows from the split copy of V_j (Vs block j, complete on
// every CTA): each element's product t x_c is formed and summed in
// double-float (df.cuh) with the split table, so the FP64 pipe only runs the
// row epilogue y = d x + a / sqrt(S_i). Same gathers (one 32-byte row per
// element) and slot scheme as block_spmv.
__device__ void block_spmv_df(Ctx& x, uint32_t j, double* W) {
  StreamView const& S = x.c.S;
  uint32_t const lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t const col_mask = S.col_bits < 32 ? ((1u << S.col_bits) - 1u) : 0xFFFFFFFFu;
  bool const packed = x.c.packed != 0;
  float2 const* table = x.c.table_s;
  Row4s const* Xs = reinterpret_cast<Row4s const*>(x.c.Vs) + (uint64_t)j * x.c.D;
  double const* X = x.c.V + (uint64_t)j * x.c.D * 4;
  for (uint64_t s = x.s0 + warp; s < x.s1; s += nw) {
    uint64_t const base = S.slice_ptr[s];
    uint32_t const width = (uint32_t)((S.slice_ptr[s + 1] - base) >> 5);
    float Sa[4] = {}, Ea[4] = {};
    uint32_t const* ent = S.entries + base + lane;
    // the next step's entries are loaded while this step's gathers are in
    // flight (with 16 warps per SM, the entry load and the gather would
    // otherwise be two exposed latencies per step; two steps ahead measured
    // the same)
    uint32_t v[kBlockSpmvU];
#pragma unroll
    for (int u = 0; u < kBlockSpmvU; ++u) v[u] = (uint32_t)u < width ? __ldcs(ent + (uint64_t)u * 32) : kNull;
    for (uint32_t e0 = 0; e0 < width; e0 += kBlockSpmvU) {
      uint32_t vn[kBlockSpmvU];
#pragma unroll
      for (int u = 0; u < kBlockSpmvU; ++u)
        vn[u] = e0 + kBlockSpmvU + u < width ? __ldcs(ent + (uint64_t)(e0 + kBlockSpmvU + u) * 32) : kNull;
      float2 t[kBlockSpmvU];
      float4 gh[kBlockSpmvU], gl[kBlockSpmvU];
#pragma unroll
      for (int u = 0; u < kBlockSpmvU; ++u) {
        if (v[u] != kNull) {
          uint32_t const col = v[u] & col_mask;
          uint32_t const code =
              packed ? (v[u] >> S.col_bits) : (uint32_t)__ldcs(S.codes + base + lane + (uint64_t)(e0 + u) * 32);
          t[u] = __ldg(table + code);
          float4 const* row = reinterpret_cast<float4 const*>(Xs + col);
          gh[u] = __ldcg(row);
          gl[u] = __ldcg(row + 1);
        } else {
          t[u] = make_float2(0.0f, 0.0f);
          gh[u] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          gl[u] = gh[u];
        }
      }
#pragma unroll
      for (int u = 0; u < kBlockSpmvU; ++u) {
        df_mac(t[u].x, t[u].y, gh[u].x, gl[u].x, Sa[0], Ea[0]);
        df_mac(t[u].x, t[u].y, gh[u].y, gl[u].y, Sa[1], Ea[1]);
        df_mac(t[u].x, t[u].y, gh[u].z, gl[u].z, Sa[2], Ea[2]);
        df_mac(t[u].x, t[u].y, gh[u].w, gl[u].w, Sa[3], Ea[3]);
      }
#pragma unroll
      for (int u = 0; u < kBlockSpmvU; ++u) v[u] = vn[u];
    }
    uint64_t const i = s * 32 + lane;
    if (i < x.c.D) {
      double const f = S.inv_sqrt_s[S.row_class[i]];
      double const dg = static_cast<double const*>(S.diag)[i];
      Row4 const xi = ldcg4(X + i * 4);
      *reinterpret_cast<Row4*>(W + i * 4) = mk4(fma(f, (double)Sa[0] + (double)Ea[0], dg * xi.x),
                                                fma(f, (double)Sa[1] + (double)Ea[1], dg * xi.y),
                                                fma(f, (double)Sa[2] + (double)Ea[2], dg * xi.z),
                                                fma(f, (double)Sa[3] + (double)Ea[3], dg * xi.w));
    }
  }
}

// X -= sum_{i<nb} V_i C_i (two passes of classical Gram-Schmidt). C (shared,
// nb * 16, row-major a*4+c per block, may be null) receives the summed
// coefficients; norms2 (shared, may be null) the squared column norms of X
// before the projection. The first pass runs against blocks first .. nb-1
// only (first > 0 where X = H V_{nb-1} is, in exact arithmetic, orthogonal
// to the older blocks); the second pass always runs against all nb blocks.
__device__ bool cgs2(Ctx& x, double* X, uint32_t nb, double* C, double* norms2, uint32_t first = 0) {
  Row4s const* Vs = reinterpret_cast<Row4s const*>(x.c.Vs);
  Row4s* Xs = reinterpret_cast<Row4s*>(x.c.Xs);
  uint64_t const D = x.c.D;
  int const K = (int)nb * 16;
  if (C)
    for (int k = threadIdx.x; k < K; k += blockDim.x) C[k] = 0.0;
  for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += blockDim.x)
    Xs[r] = split_row(*reinterpret_cast<Row4 const*>(X + r * 4));
  tc::fence_proxy_async_global();  // the row streams read Xs through the async proxy
  __syncthreads();
  for (int pass = 0; pass < 2; ++pass) {
    uint32_t const i0 = pass == 0 ? first : 0u;
    for (uint32_t i = i0; i < nb; ++i) {
      float S[16] = {}, E[16] = {};
      if (!gs_dots(x, Vs + (uint64_t)i * D, Xs, S, E)) return false;
      double p[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) p[k] = (double)S[k] + (double)E[k];
      cta_sum<16>(p, x.red, x.tmp + 16 * i);
    }
    int Kp = K;
    if (pass == 0 && norms2) {
      double q[4] = {};
      for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += blockDim.x) {
        Row4 const w = *reinterpret_cast<Row4 const*>(X + r * 4);
        q[0] = fma(w.x, w.x, q[0]);
        q[1] = fma(w.y, w.y, q[1]);
        q[2] = fma(w.z, w.z, q[2]);
        q[3] = fma(w.w, w.w, q[3]);
      }
      cta_sum<4>(q, x.red, x.tmp + K);
      Kp = K + 4;
    }
    double* tot = x.tmp + kPart;
    int const k0 = 16 * (int)i0;
    if (!group_sum(x, x.tmp + k0, Kp - k0, tot + k0)) return false;
    if (C)
      for (int k = k0 + threadIdx.x; k < K; k += blockDim.x) C[k] += tot[k];
    if (Kp > K && threadIdx.x < 4) norms2[threadIdx.x] = tot[K + threadIdx.x];
    // the coefficients in double-float, over this CTA's partial sums (no
    // longer needed once group_sum has returned)
    float* ch = reinterpret_cast<float*>(x.tmp);
    float* cl = ch + K;
    for (int k = k0 + threadIdx.x; k < K; k += blockDim.x) df_split(tot[k], ch[k], cl[k]);
    __syncthreads();
    // X -= sum_i V_i tot_i
    if (!gs_update(x, Vs, Xs, i0, nb, ch, cl)) return false;
  }
  for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += blockDim.x) {
    Row4s const w = Xs[r];
    *reinterpret_cast<Row4*>(X + r * 4) = mk4((double)w.h.x + (double)w.l.x, (double)w.h.y + (double)w.l.y,
                                              (double)w.h.z + (double)w.l.z, (double)w.h.w + (double)w.l.w);
  }
  __syncthreads();
  return true;
}

// Double-float copies (Vs) of basis blocks b0 .. b1, own rows.
__device__ void split_blocks(Ctx& x, uint32_t b0, uint32_t b1) {
  Row4s* Vs = reinterpret_cast<Row4s*>(x.c.Vs);
  for (uint32_t b = b0; b <= b1; ++b)
    for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += blockDim.x)
      Vs[(uint64_t)b * x.c.D + r] = split_row(*reinterpret_cast<Row4 const*>(x.c.V + ((uint64_t)b * x.c.D + r) * 4));
  tc::fence_proxy_async_global();
  __syncthreads();
}

// QR of the new Krylov block X (already projected against V_0 .. V_{nb-1})
// with deflation: a column whose norm fell below 1e-10 of its norm before the
// projection (norms2), or that is numerically dependent on the others, means
// the block Krylov space lost a direction there (typically a converged Ritz
// vector of the restart block). Such columns are replaced by random vectors,
// projected against the basis, and the block is factored by CholQR2. Rb gets
// R with the replaced columns zeroed (their coupling to H V_j is below the
// threshold). Returns false on barrier failure or if the replacement fails.
__device__ bool lanczos_qr(Ctx& x, double* X, uint32_t nb, double* norms2, double* Rb, uint32_t step,
                           bool& replaced) {
  __shared__ double R[16];
  __shared__ int mask_s, total_mask_s;
  if (threadIdx.x == 0) total_mask_s = 0;
  __syncthreads();
  for (int attempt = 0; attempt < 3; ++attempt) {
    double g[4] = {};
    for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += blockDim.x) {
      Row4 const v = *reinterpret_cast<Row4 const*>(X + r * 4);
      g[0] = fma(v.x, v.x, g[0]);
      g[1] = fma(v.y, v.y, g[1]);
      g[2] = fma(v.z, v.z, g[2]);
      g[3] = fma(v.w, v.w, g[3]);
    }
    cta_sum<4>(g, x.red, x.tmp);
    if (!group_sum(x, x.tmp, 4, x.tmp + 16)) return false;
    if (threadIdx.x == 0) {
      int m = 0;
      for (int c = 0; c < 4; ++c)
        if (!(x.tmp[16 + c] > 1e-20 * norms2[c])) m |= 1 << c;
      mask_s = m;
      total_mask_s |= m;
    }
    __syncthreads();
    int const m = mask_s;
    if (m == 0) break;
    if (attempt == 2) return false;
    for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += blockDim.x) {
      uint32_t cnt[4] = {(uint32_t)r, (uint32_t)(r >> 32), 0xDEF1u + step, (uint32_t)attempt};
      philox(cnt, (uint32_t)x.c.seed, (uint32_t)(x.c.seed >> 32));
      double* row = X + r * 4;
      for (int c = 0; c < 4; ++c)
        if (m & (1 << c)) row[c] = 2.0 * ((double)cnt[c] * (1.0 / 4294967296.0)) - 1.0;
    }
    __syncthreads();
    if (threadIdx.x < 4 && (m & (1 << threadIdx.x))) norms2[threadIdx.x] = (double)x.c.D;
    __syncthreads();
    if (!cgs2(x, X, nb, nullptr, nullptr)) return false;
  }
  bool ok;
  // dependent columns that are not small: a breakdown
  if (!block_qr_df(x, X, reinterpret_cast<Row4s*>(x.c.Vs) + (uint64_t)nb * x.c.D, R, ok)) return false;
  if (threadIdx.x < 16) {
    int const col = threadIdx.x & 3;
    Rb[threadIdx.x] = (total_mask_s & (1 << col)) ? 0.0 : R[threadIdx.x];
  }
  __syncthreads();
  replaced = total_mask_s != 0;
  return true;
}

// Cyclic Jacobi on the symmetric n x n matrix A (shared, row-major, n even)
// with parallel round-robin rotations and a threshold: a rotation whose
// off-diagonal entry is at most 1e-16 of ||A||_F (invariant under the
// rotations) is skipped, and the sweeps end when one performs none (the
// eigenvalues then carry errors of order 1e-32 ||A||^2 / gap). Q (shared)
// receives the eigenvectors as columns. Eigenvalues end on the diagonal of A.
__device__ void jacobi(double* A, double* Q, int n) {
  __shared__ double cs[kMaxN / 2][2];
  __shared__ int pp[kMaxN / 2][2];
  __shared__ double wsum[8];
  __shared__ double thr;
  __shared__ int rotated;
  double f = 0.0;
  for (int k = threadIdx.x; k < n * n; k += blockDim.x) {
    Q[k] = (k / n == k % n) ? 1.0 : 0.0;
    f = fma(A[k], A[k], f);
  }
  for (int o = 16; o > 0; o >>= 1) f += __shfl_xor_sync(0xffffffffu, f, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = f;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += wsum[w];
    thr = 1e-16 * sqrt(t);
    rotated = 0;
  }
  __syncthreads();
  int const half = n / 2;
  for (int sweep = 0; sweep < 40; ++sweep) {
    for (int round = 0; round < n - 1; ++round) {
      // round-robin pairing: player 0 fixed, the others rotate
      if ((int)threadIdx.x < half) {
        int const k = threadIdx.x;
        auto pos = [&](int q) { return q == 0 ? 0 : 1 + ((q - 1 + round) % (n - 1)); };
        int p = pos(k), q = pos(n - 1 - k);
        if (p > q) {
          int const t = p;
          p = q;
          q = t;
        }
        double const apq = A[p * n + q];
        double c = 1.0, s = 0.0;
        if (fabs(apq) > thr) {
          // tan of the angle: the smaller root of t^2 + 2 tau t - 1 = 0
          double const tau = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
          double const t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(fma(tau, tau, 1.0)));
          c = rsqrt(fma(t, t, 1.0));
          s = t * c;
          if (s != 0.0) rotated = 1;
        }
        cs[k][0] = c;
        cs[k][1] = s;
        pp[k][0] = p;
        pp[k][1] = q;
      }
      __syncthreads();
      // rows: A <- J^T A
      for (int e = threadIdx.x; e < half * n; e += blockDim.x) {
        int const k = e / n, col = e % n;
        double const s = cs[k][1];
        if (s == 0.0) continue;
        int const p = pp[k][0], q = pp[k][1];
        double const c = cs[k][0];
        double const ap = A[p * n + col], aq = A[q * n + col];
        A[p * n + col] = c * ap - s * aq;
        A[q * n + col] = s * ap + c * aq;
      }
      __syncthreads();
      // columns: A <- A J, Q <- Q J
      for (int e = threadIdx.x; e < half * n; e += blockDim.x) {
        int const k = e / n, row = e % n;
        double const s = cs[k][1];
        if (s == 0.0) continue;
        int const p = pp[k][0], q = pp[k][1];
        double const c = cs[k][0];
        double const ap = A[row * n + p], aq = A[row * n + q];
        A[row * n + p] = c * ap - s * aq;
        A[row * n + q] = s * ap + c * aq;
        double const qp = Q[row * n + p], qq = Q[row * n + q];
        Q[row * n + p] = c * qp - s * qq;
        Q[row * n + q] = s * qp + c * qq;
      }
      __syncthreads();
    }
    int const any = rotated;
    __syncthreads();  // every thread has read the flag
    if (!any) break;
    if (threadIdx.x == 0) rotated = 0;
    __syncthreads();
  }
}

// Rayleigh-Ritz of T (n = 4 (j + 1)) by the leader CTA. T is assembled from
// the projections of every step (T[block p][block q] = C_p of step q for
// p <= q), which also covers the arrowhead couplings after a thick restart.
// The lowest min(8, n) Ritz values go to c.out[0..8), their vectors to c.Y,
// the residual estimates ||B_j y_last|| of the lowest four to c.out[8..12).
// Returns the largest estimate over the nev wanted pairs.
__device__ double rayleigh_ritz(ChainDesc const& c, uint32_t j, bool have_B, double* A, double* Q) {
  int const n = 4 * (int)(j + 1);
  constexpr int kStride = kMaxN * 4;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    int const r = e / n, q = e % n;
    int const br = r / 4, bq = q / 4, a = r % 4, b = q % 4;
    double v;
    if (br == bq)
      v = 0.5 * (ldcg(c.Tc + bq * kStride + br * 16 + a * 4 + b) + ldcg(c.Tc + bq * kStride + br * 16 + b * 4 + a));
    else if (br < bq)
      v = ldcg(c.Tc + bq * kStride + br * 16 + a * 4 + b);
    else
      v = ldcg(c.Tc + br * kStride + bq * 16 + b * 4 + a);
    A[e] = v;
  }
  __syncthreads();
  jacobi(A, Q, n);
  __shared__ int idx[8];
  __shared__ double worst;
  int const nk = n < 8 ? n : 8;
  if (threadIdx.x == 0) {
    // selection of the nk smallest diagonal entries, ascending
    bool used[kMaxN] = {};
    for (int i = 0; i < nk; ++i) {
      int best = -1;
      for (int q = 0; q < n; ++q)
        if (!used[q] && (best < 0 || A[q * n + q] < A[best * n + best])) best = q;
      used[best] = true;
      idx[i] = best;
      c.out[i] = A[best * n + best];
    }
    worst = 0.0;
    for (int i = 0; i < kB; ++i) {
      double r2 = 0.0;
      if (have_B) {
        for (int a = 0; a < 4; ++a) {
          double s = 0.0;
          for (int b = 0; b < 4; ++b) s += ldcg(c.Bblk + j * 16 + a * 4 + b) * Q[(4 * (int)j + b) * n + idx[i]];
          r2 += s * s;
        }
      }
      c.out[8 + i] = sqrt(r2);
      if (i < (int)c.nev) worst = fmax(worst, sqrt(r2));
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < n * 8; e += blockDim.x) {
    int const q = e / 8, i = e % 8;
    c.Y[q * 8 + i] = i < nk ? Q[q * n + idx[i]] : 0.0;
  }
  __syncthreads();
  return worst;
}

// Ritz vectors Psi = V Y over the basis blocks 0..j (own rows): the lowest
// four into W, the next four into W2 when `both`. The products run in
// double-float arithmetic on the split blocks Vs (every block 0..j is split
// by the time of a restart); Y is split once per call. Ys: shared scratch of
// at least 4 (j + 1) x 16 doubles.
__device__ void ritz_vectors(Ctx& x, uint32_t j, double* Ys, bool both) {
  int const n = 4 * (int)(j + 1);
  float* Yh = reinterpret_cast<float*>(Ys);
  float* Yl = Yh + n * 8;
  for (int e = threadIdx.x; e < n * 8; e += blockDim.x) df_split(ldcg(x.c.Y + e), Yh[e], Yl[e]);
  __syncthreads();
  uint64_t const D = x.c.D;
  Row4s const* Vs = reinterpret_cast<Row4s const*>(x.c.Vs);
  for (int half = 0; half < (both ? 2 : 1); ++half) {
    double* out = half ? x.c.W2 : x.c.W;
    for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += blockDim.x) {
      float S[4] = {}, E[4] = {};
      for (int b = 0; b <= (int)j; ++b) {
        Row4s const a = Vs[(uint64_t)b * D + r];
        float const ah[4] = {a.h.x, a.h.y, a.h.z, a.h.w}, al[4] = {a.l.x, a.l.y, a.l.z, a.l.w};
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          int const k = (4 * b + s) * 8 + 4 * half;
#pragma unroll
          for (int i = 0; i < 4; ++i) df_mac(ah[s], al[s], Yh[k + i], Yl[k + i], S[i], E[i]);
        }
      }
      *reinterpret_cast<Row4*>(out + r * 4) = mk4((double)S[0] + (double)E[0], (double)S[1] + (double)E[1],
                                                  (double)S[2] + (double)E[2], (double)S[3] + (double)E[3]);
    }
  }
  __syncthreads();
}

__device__ void copy_block(Ctx& x, double* dst, double const* src) {
  for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += blockDim.x)
    *reinterpret_cast<Row4*>(dst + r * 4) = *reinterpret_cast<Row4 const*>(src + r * 4);
  __syncthreads();
}

__device__ void random_block(Ctx& x) {
  for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += blockDim.x) {
    uint32_t c[4] = {(uint32_t)r, (uint32_t)(r >> 32), 0xB10Cu, 0u};
    philox(c, (uint32_t)x.c.seed, (uint32_t)(x.c.seed >> 32));
    double v[4];
    for (int k = 0; k < 4; ++k) v[k] = 2.0 * ((double)c[k] * (1.0 / 4294967296.0)) - 1.0;
    *reinterpret_cast<Row4*>(x.c.V + r * 4) = mk4(v[0], v[1], v[2], v[3]);
  }
  __syncthreads();
}

// Whole solve of one problem by the CTAs of its group. Cycles end when the
// basis is full or the Ritz estimates converge; the lowest eight Ritz vectors
// and the last Lanczos block then seed the next cycle (thick restart: T starts
// as diag(theta_1..8) and the next step's projections supply the arrowhead
// couplings), or, after a breakdown, the lowest four alone (explicit restart).
__device__ void solve_chain(ChainDesc const& c, uint32_t rank, uint32_t ncta, uint32_t* bar, BatchArgs const& a,
                            double* red, double* tmp, double* C, double* A, double* Q, uint64_t* gs_bar,
                            uint32_t* gs_phase) {
  Ctx x{c, rank, ncta, bar, &a, 0, 0, 0, 0, 0, red, tmp, A, gs_bar, gs_phase};
  x.s0 = c.n_slices * rank / ncta;
  x.s1 = c.n_slices * (rank + 1) / ncta;
  x.r0 = std::min<uint64_t>(c.D, x.s0 * 32);
  x.r1 = std::min<uint64_t>(c.D, x.s1 * 32);
  bool const leader = rank == 0;
  constexpr int kStride = kMaxN * 4;
  __shared__ double Rb[16], norms2[4];
  uint32_t steps = 0, restarts = 0, matvecs = 0, status = 2;
  double const tol = a.tol;
  // phase timers, kept by thread 0 in shared memory (no registers held
  // across the phases)
  __shared__ unsigned long long acc[6], tmark;
  if (threadIdx.x == 0) {
    for (int q = 0; q < 6; ++q) acc[q] = 0;
    tmark = tc::global_ns();
  }
  auto lap = [&](int phase) {
    if (threadIdx.x == 0) {
      unsigned long long const now = tc::global_ns();
      acc[phase] += now - tmark;
      tmark = now;
    }
  };
  random_block(x);
  bool qr_ok;
  if (!block_qr(x, c.V, Rb, qr_ok)) {
    if (!qr_ok) return;
    status = 3;
  }
  uint32_t j0 = 0;
  while (status != 3) {
    uint32_t j = j0;
    // block whose H-image needs full projections in both passes: the
    // continuation block of a restart (arrowhead couplings) or a block with
    // replaced (random) columns
    uint32_t full_from = j0;
    bool broke = false;
    for (;; ++j) {
      double* Vj = c.V + (uint64_t)j * c.D * 4;
      if (j == j0) split_blocks(x, 0u, j0);  // later blocks come split from the QR of each step
      if (!group_barrier(bar, ncta, a)) return;  // V_j complete on every CTA before the gathers
      lap(4);
      block_spmv_df(x, j, c.W);
      ++matvecs;
      __syncthreads();
      lap(0);
      if (!cgs2(x, c.W, j + 1, C, norms2, j > full_from ? j - 1 : 0u)) return;
      lap(1);
      if (leader)
        for (int k = threadIdx.x; k < 16 * (int)(j + 1); k += blockDim.x) c.Tc[j * kStride + k] = C[k];
      ++steps;
      // QR of W -> V_{j+1}, B_j (with deflation of lost directions)
      double* Vn = c.V + (uint64_t)(j + 1) * c.D * 4;
      copy_block(x, Vn, c.W);
      bool replaced = false;
      broke = !lanczos_qr(x, Vn, j + 1, norms2, Rb, steps, replaced);
      if (replaced) full_from = j + 1;
      if (*(volatile int*)a.error) return;
      if (leader)
        for (int k = threadIdx.x; k < 16; k += blockDim.x) c.Bblk[j * 16 + k] = broke ? 0.0 : Rb[k];
      lap(2);
      bool const full = j + 1 >= c.m_blocks || steps >= a.max_steps || broke;
      if (full || (j + 1) % a.rr_every == 0) {
        __threadfence();
        if (!group_barrier(bar, ncta, a)) return;  // T and B visible to the leader
        if (leader) {
          double const worst = rayleigh_ritz(c, j, !broke, A, Q);
          if (threadIdx.x == 0) {
            c.flag[0] = (worst <= 0.5 * tol) ? 1u : 0u;
            __threadfence();
          }
        }
        if (!group_barrier(bar, ncta, a)) return;
        lap(3);
        if (ldcg(c.flag) != 0u || full) break;
      }
    }
    bool const thick = !broke && j >= 1 && c.m_blocks >= 3;
    ritz_vectors(x, j, A, thick);  // A: the dynamic shared area, free outside the Jacobi solve
    if (!group_barrier(bar, ncta, a)) return;  // every CTA done reading the old basis
    if (thick && j + 1 != 2) copy_block(x, c.V + 2 * c.D * 4, c.V + (uint64_t)(j + 1) * c.D * 4);
    copy_block(x, c.V, c.W);
    if (thick) copy_block(x, c.V + c.D * 4, c.W2);
    if (!group_barrier(bar, ncta, a)) return;  // Psi rows visible to every CTA's SpMV gathers
    lap(4);
    // true residuals of the lowest four Ritz pairs
    block_spmv(x, c.V, c.W);
    ++matvecs;
    __syncthreads();
    double th[8];
    for (int i = 0; i < 8; ++i) th[i] = ldcg(c.out + i);
    {
      double p[4] = {};
      for (uint64_t r = x.r0 + threadIdx.x; r < x.r1; r += blockDim.x) {
        Row4 const w = *reinterpret_cast<Row4 const*>(c.W + r * 4);
        Row4 const v = *reinterpret_cast<Row4 const*>(c.V + r * 4);
        double const d[4] = {w.x - th[0] * v.x, w.y - th[1] * v.y, w.z - th[2] * v.z, w.w - th[3] * v.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) p[i] = fma(d[i], d[i], p[i]);
      }
      cta_sum<4>(p, red, tmp);
      if (!group_sum(x, tmp, 4, tmp + 16)) return;
    }
    lap(5);
    bool all = true;
    for (uint32_t i = 0; i < c.nev; ++i) all = all && sqrt(tmp[16 + i]) <= tol;
    __syncthreads();
    if (leader && threadIdx.x == 0)
      for (uint32_t i = 0; i < 4; ++i) c.out[8 + i] = sqrt(tmp[16 + i]);
    if (all) {
      status = 1;
      break;
    }
    if (steps >= a.max_steps) break;
    ++restarts;
    if (thick) {
      // T of the new cycle: diag(theta_1..8) on blocks 0 and 1
      if (leader) {
        for (int k = threadIdx.x; k < 2 * kStride; k += blockDim.x) c.Tc[k] = 0.0;
        __syncthreads();
        if (threadIdx.x < 8) {
          int const i = threadIdx.x, b = i / 4, a4 = i % 4;
          c.Tc[b * kStride + b * 16 + a4 * 4 + a4] = th[i];
        }
        __threadfence();
      }
      j0 = 2;
    } else {
      if (!block_qr(x, c.V, Rb, qr_ok)) {
        if (!qr_ok) return;
        status = 3;
        break;
      }
      j0 = 0;
    }
  }
  if (leader && threadIdx.x == 0) {
    c.stats[0] = steps;
    c.stats[1] = restarts;
    c.stats[2] = matvecs;
    c.stats[3] = status;
    for (int q = 0; q < 6; ++q) c.prof[q] = acc[q];
  }
}

__global__ void __launch_bounds__(256, 2) k_batch_lanczos(BatchArgs a) {
  __shared__ double red[8 * 16];
  __shared__ __align__(16) double tmp[2 * kPart];  // also read as float4 (split Gram-Schmidt coefficients)
  __shared__ double C[kPart];
  extern __shared__ __align__(128) double dyn[];  // A [kMaxN^2], Q [kMaxN^2] (leader work); row-stream stages
  __shared__ uint64_t gs_bar[kGsStages];
  uint32_t gs_phase = 0;
  if (threadIdx.x == 0) {
    for (int q = 0; q < kGsStages; ++q) tc::mbar_init(&gs_bar[q], 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  uint32_t const gi = a.cta_group[blockIdx.x];
  GroupDesc const g = a.groups[gi];
  uint32_t const rank = blockIdx.x - g.cta0;
  for (uint32_t q = 0; q < g.count; ++q) {
    ChainDesc const& c = a.chains[a.order[g.first + q]];
    solve_chain(c, rank, g.ncta, g.bar, a, red, tmp, C, dyn, dyn + kMaxN * kMaxN, gs_bar, &gs_phase);
    if (*(volatile int*)a.error) return;
    if (!group_barrier(g.bar, g.ncta, a)) return;
  }
}

// chains[blockIdx.y].table_s = its FP64 matrix-element table split into
// double-float pairs.
__global__ void k_split_tables(ChainDesc const* __restrict__ chains) {
  ChainDesc const& c = chains[blockIdx.y];
  double const* t = static_cast<double const*>(c.S.table);
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < c.S.n_codes; k += gridDim.x * blockDim.x) {
    float h, l;
    df_split(t[k], h, l);
    c.table_s[k] = make_float2(h, l);
  }
}

// [D][4] block -> column-major D x nev with stride ld
__global__ void k_unpack_block(double const* __restrict__ V, uint64_t D, uint32_t nev, double* __restrict__ out,
                               uint64_t ld) {
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < D * nev; e += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t const i = e % D, c = e / D;
    out[c * ld + i] = V[i * 4 + c];
  }
}

// ------------------------------------------------------------ host side ---

// Groups of the persistent launch. A problem's block step on n CTAs is
// modelled as fixed + work / n: `fixed` is the part that more CTAs do not
// shorten (the leader's Rayleigh-Ritz solve, the group barriers), work the
// part that is split over the group's rows. The layout minimises the
// modelled makespan T on `grid` CTAs:
// - a problem with fixed + work > T gets a group of its own with
//   ceil(work / (T - fixed)) CTAs (at most max_ctas, its slice count);
// - the other problems are packed, first fit by decreasing work, into
//   one-CTA groups that solve them one after another within T;
// - T is the smallest bound (bisection) that needs no more than `grid` CTAs;
//   CTAs left over go one at a time to the multi-CTA group with the largest
//   modelled time.
struct BatchLayout {
  std::vector<GroupDesc> groups;
  std::vector<uint32_t> cta_group, order, group_of_chain;
};

BatchLayout batch_layout(std::vector<double> const& work, std::vector<uint32_t> const& max_ctas, double fixed,
                         unsigned grid) {
  size_t const count = work.size();
  std::vector<uint32_t> idx(count);
  std::iota(idx.begin(), idx.end(), 0u);
  std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return work[a] > work[b]; });
  struct Try {
    std::vector<uint32_t> n;  // CTAs of a problem's own group, 0 when packed
    std::vector<std::vector<uint32_t>> bins;
    std::vector<double> load;
    unsigned ctas = 0;
  };
  auto attempt = [&](double T, Try& t) {
    t.n.assign(count, 0);
    t.bins.clear();
    t.load.clear();
    t.ctas = 0;
    for (uint32_t i : idx) {
      double const alone = fixed + work[i];
      if (alone <= T) {
        size_t b = 0;
        while (b < t.bins.size() && t.load[b] + alone > T) ++b;
        if (b == t.bins.size()) {
          t.bins.emplace_back();
          t.load.push_back(0.0);
          ++t.ctas;
        }
        t.bins[b].push_back(i);
        t.load[b] += alone;
      } else {
        if (T <= fixed) return false;
        double const need = std::ceil(work[i] / (T - fixed));
        if (need > (double)std::max<uint32_t>(1, max_ctas[i]) || need > (double)grid) return false;
        t.n[i] = (uint32_t)need;
        t.ctas += t.n[i];
      }
      if (t.ctas > grid) return false;
    }
    return true;
  };
  Try best;
  double hi = 0.0;
  for (double w : work) hi += fixed + w;
  hi = hi * 1.001 + 1.0;
  if (!attempt(hi, best)) {  // cannot happen: everything fits in one bin
    best.n.assign(count, 0);
    best.bins.assign(1, idx);
    best.ctas = 1;
  }
  double lo = 0.0;
  for (int it = 0; it < 64 && hi - lo > 1e-6 * hi; ++it) {
    double const mid = 0.5 * (lo + hi);
    Try t;
    if (attempt(mid, t)) {
      hi = mid;
      best = std::move(t);
    } else {
      lo = mid;
    }
  }
  // CTAs left over: to the slowest multi-CTA groups
  unsigned left = grid - std::min(grid, best.ctas);
  while (left > 0) {
    double worst = -1.0;
    uint32_t wi = UINT32_MAX;
    for (uint32_t i = 0; i < count; ++i)
      if (best.n[i] > 0 && best.n[i] < std::max<uint32_t>(1, max_ctas[i])) {
        double const t = fixed + work[i] / best.n[i];
        if (t > worst) {
          worst = t;
          wi = i;
        }
      }
    if (wi == UINT32_MAX) break;
    ++best.n[wi];
    --left;
  }
  BatchLayout L;
  L.group_of_chain.assign(count, 0);
  uint32_t cta = 0;
  for (uint32_t i : idx)
    if (best.n[i] > 0) {
      L.group_of_chain[i] = (uint32_t)L.groups.size();
      L.groups.push_back(GroupDesc{cta, best.n[i], (uint32_t)L.order.size(), 1, nullptr});
      L.order.push_back(i);
      cta += best.n[i];
    }
  for (auto const& bin : best.bins) {
    L.groups.push_back(GroupDesc{cta, 1, (uint32_t)L.order.size(), (uint32_t)bin.size(), nullptr});
    for (uint32_t i : bin) {
      L.group_of_chain[i] = (uint32_t)L.groups.size() - 1;
      L.order.push_back(i);
    }
    cta += 1;
  }
  for (uint32_t g = 0; g < L.groups.size(); ++g)
    for (uint32_t k = 0; k < L.groups[g].ncta; ++k) L.cta_group.push_back(g);
  return L;
}

struct Plan {
  unsigned threads = 256, ctas_per_sm = 1;
};

// Caller's fixed launch shape (sed_set_batched_launch); threads == 0: tune.
std::atomic<unsigned> g_force_threads{0}, g_force_per_sm{0};

std::mutex g_tune_mu;
std::map<std::tuple<int, unsigned, uint64_t>, Plan> g_tuned;

size_t dyn_smem() { return 2 * (size_t)kMaxN * kMaxN * sizeof(double); }

}  // namespace
}  // namespace sed

using namespace sed;

extern "C" {

int sed_eigh_batched(unsigned count, ls_operator* const ops[], sed_eigh_options const* opts, double* eigenvalues,
                     double* residuals, void* const eigenvectors[], uint64_t const ldv[], sed_batch_info* info) {
  auto t_start = std::chrono::steady_clock::now();
  if (count == 0) return LS_SUCCESS;
  if (!ops || !opts || !eigenvalues) return fail(LS_INVALID_ARGUMENT, "sed_eigh_batched: NULL argument");
  sed_eigh_options o{};
  sed_eigh_options_init(&o);
  std::memcpy(&o, opts, std::min<size_t>(sizeof(o), opts->struct_size ? opts->struct_size : sizeof(o)));
  uint32_t const nev = o.nev ? o.nev : 1;
  if (nev > (uint32_t)kB) return fail(LS_INVALID_ARGUMENT, "sed_eigh_batched: nev must be 1..4");
  if (o.block_size != 0 && o.block_size != 1 && o.block_size != (uint32_t)kB)
    return fail(LS_INVALID_ARGUMENT, "sed_eigh_batched: block_size must be 4");
  double const tol = o.tol > 0 ? o.tol : 1e-8;
  uint32_t const m_req = o.max_basis ? std::max<uint32_t>(2, o.max_basis / kB) : 12;
  int device = -1;
  if (int st = current_device(&device)) return st;
  std::vector<OperatorData*> od(count);
  for (unsigned i = 0; i < count; ++i) {
    if (!ops[i]) return fail(LS_INVALID_ARGUMENT, "sed_eigh_batched: NULL operator");
    od[i] = ops[i]->d.get();
    OperatorData& op = *od[i];
    if (!op.basis->built) return fail(LS_CACHE_NOT_BUILT, "basis has not been built (call ls_build)");
    if (op.basis->device != device) return fail(LS_INVALID_ARGUMENT, "sed_eigh_batched: operators on another device");
    if (!op.is_real) return fail(LS_OPERATOR_IS_COMPLEX, "sed_eigh_batched: operators must be real");
    if (op.basis->D < 2 * (uint64_t)kB) return fail(LS_INVALID_ARGUMENT, "sed_eigh_batched: dimension below 8");
    if (int st = operator_ensure_ready(op)) return st;
    if (!op.stream.ready)
      if (int st = operator_record_stream(op, op.cuda_stream)) return st;
  }
  for (unsigned i = 0; i < count; ++i) SED_TRY_CUDA(cudaStreamSynchronize(od[i]->cuda_stream));
  if (eigenvectors)
    for (unsigned i = 0; i < count; ++i)
      if (int st = wait_for_caller({eigenvectors[i]})) return st;
  auto t_setup = std::chrono::steady_clock::now();
  cudaStream_t stream = nullptr;
  SED_TRY_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sguard{stream};

  int sms = 0, coop = 0;
  SED_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  SED_TRY_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device));
  if (!coop) return fail(LS_CUDA_ERROR, "sed_eigh_batched: device lacks cooperative launch");
  SED_TRY_CUDA(cudaFuncSetAttribute(k_batch_lanczos, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_smem()));
  // co-resident CTAs per SM for each block size (the cooperative launch
  // needs the whole grid resident)
  int occ128 = 0, occ256 = 0;
  SED_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ128, k_batch_lanczos, 128, dyn_smem()));
  SED_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ256, k_batch_lanczos, 256, dyn_smem()));
  int const max_per_sm = std::min(3, std::max(occ128, occ256));
  if (max_per_sm < 1) return fail(LS_CUDA_ERROR, "sed_eigh_batched: kernel does not fit on an SM");

  // work model per problem: streamed bytes of a block matvec plus the FP64
  // reorthogonalisation (rows x stored columns)
  std::vector<double> work(count);
  for (unsigned i = 0; i < count; ++i) {
    double const D = (double)od[i]->basis->D, E = (double)od[i]->stream.n_entries;
    work[i] = E * 4.0 + D * 40.0 + D * 16.0 * m_req * 6.0;
  }

  // Per-problem device arena
  std::vector<uint32_t> m_blocks(count);
  std::vector<size_t> off_V(count), off_Vs(count), off_Xs(count), off_Ts(count), off_W(count), off_W2(count), off_T(count), off_B(count), off_Y(count), off_out(count);
  size_t total = 0;
  auto take = [&](size_t bytes) {
    size_t const o = total;
    total += (bytes + 255) & ~size_t(255);
    return o;
  };
  for (unsigned i = 0; i < count; ++i) {
    uint64_t const D = od[i]->basis->D;
    uint32_t m = std::min<uint32_t>(std::min<uint32_t>(m_req, kMaxBlocks), (uint32_t)std::min<uint64_t>(kMaxBlocks, D / kB - 1));
    m = std::max<uint32_t>(m, 1);
    m_blocks[i] = m;
    off_V[i] = take((size_t)(m + 1) * D * kB * 8);
    off_Vs[i] = take((size_t)(m + 1) * D * kB * 8);  // Row4s: 8 floats a row
    off_Xs[i] = take((size_t)D * kB * 8);
    off_Ts[i] = take((size_t)std::max<uint32_t>(1, od[i]->tables->n_codes) * sizeof(float2));
    off_W[i] = take((size_t)D * kB * 8);
    off_W2[i] = take((size_t)D * kB * 8);
    off_T[i] = take((size_t)kMaxBlocks * kMaxN * 4 * 8);
    off_B[i] = take((size_t)kMaxBlocks * 16 * 8);
    off_Y[i] = take((size_t)kMaxN * 8 * 8);
    off_out[i] = take(kOutBytes);
  }

  // Candidate launch shapes: 128 or 256 threads per CTA, 1 to 3 CTAs per SM
  // (as many as stay co-resident); the autotuner times each on a short trial
  // (two block steps of every problem) and keeps the fastest per (device,
  // count, size). A caller-fixed shape replaces the candidates.
  std::vector<Plan> cands;
  for (unsigned th : {256u, 128u}) {
    int const occ = th == 128 ? occ128 : occ256;
    for (unsigned per = 1; per <= (unsigned)std::min(occ, 3); ++per) cands.push_back(Plan{th, per});
  }
  if (unsigned const ft = g_force_threads.load()) {
    unsigned const fp = g_force_per_sm.load();
    int const occ = ft == 128 ? occ128 : occ256;
    if ((ft != 128 && ft != 256) || fp < 1 || (int)fp > std::min(occ, 3))
      return fail(LS_INVALID_ARGUMENT, "sed_eigh_batched: the fixed launch shape (" + std::to_string(ft) + " threads, " +
                                           std::to_string(fp) + " CTAs per SM) is not co-resident on this device");
    cands.assign(1, Plan{ft, fp});
  }
  uint64_t sumD = 0;
  for (unsigned i = 0; i < count; ++i) sumD += od[i]->basis->D;
  auto key = std::make_tuple(device, count, sumD);
  Plan plan = cands[0];
  bool tuned = cands.size() == 1;  // a fixed shape needs no trial runs
  if (!tuned) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      plan = it->second;
      tuned = true;
    }
  }

  // group layout for a given grid (batch_layout), the fixed part of a block
  // step expressed in rows of the batch's mean work per row
  using Layout = BatchLayout;
  std::vector<uint32_t> max_ctas(count);
  double sum_work = 0.0, sum_rows = 0.0;
  for (unsigned i = 0; i < count; ++i) {
    max_ctas[i] = (uint32_t)std::min<uint64_t>(od[i]->stream.n_slices, UINT32_MAX);
    sum_work += work[i];
    sum_rows += (double)od[i]->basis->D;
  }
  double const fixed = kLayoutFixedRows * sum_work / std::max(1.0, sum_rows);
  auto make_layout = [&](unsigned grid) { return batch_layout(work, max_ctas, fixed, grid); };

  unsigned max_per_cand = 1;
  for (Plan const& p : cands) max_per_cand = std::max(max_per_cand, p.ctas_per_sm);
  unsigned const max_grid = (unsigned)sms * max_per_cand;
  size_t const part_bytes = 2 * (size_t)max_grid * kPart * 8;
  std::vector<size_t> off_part(count);
  for (unsigned i = 0; i < count; ++i) off_part[i] = take(part_bytes);  // enough for any group size
  size_t const off_groups = take(sizeof(GroupDesc) * max_grid);
  size_t const off_ctag = take(4 * (size_t)max_grid);
  size_t const off_order = take(4 * (size_t)count);
  size_t const off_bars = take(8 * (size_t)max_grid);
  size_t const off_chains = take(sizeof(ChainDesc) * count);
  size_t const off_err = take(16);
  DeviceBuffer arena;
  if (int st = arena.allocate(total)) return st;
  char* base = arena.as<char>();

  std::vector<ChainDesc> chains(count);
  for (unsigned i = 0; i < count; ++i) {
    OperatorData& op = *od[i];
    ChainDesc& c = chains[i];
    c.S = stream_view(op);
    c.D = op.basis->D;
    c.n_slices = op.stream.n_slices;
    c.V = reinterpret_cast<double*>(base + off_V[i]);
    c.Vs = reinterpret_cast<float*>(base + off_Vs[i]);
    c.Xs = reinterpret_cast<float*>(base + off_Xs[i]);
    c.table_s = reinterpret_cast<float2*>(base + off_Ts[i]);
    c.W = reinterpret_cast<double*>(base + off_W[i]);
    c.part = reinterpret_cast<double*>(base + off_part[i]);
    c.W2 = reinterpret_cast<double*>(base + off_W2[i]);
    c.Tc = reinterpret_cast<double*>(base + off_T[i]);
    c.Bblk = reinterpret_cast<double*>(base + off_B[i]);
    c.Y = reinterpret_cast<double*>(base + off_Y[i]);
    c.out = reinterpret_cast<double*>(base + off_out[i]);
    c.stats = reinterpret_cast<uint32_t*>(base + off_out[i] + kStatsOff);
    c.flag = reinterpret_cast<uint32_t*>(base + off_out[i] + kStatsOff + 16);
    c.prof = reinterpret_cast<uint64_t*>(base + off_out[i] + kProfOff);
    c.m_blocks = m_blocks[i];
    c.nev = nev;
    c.packed = op.stream.packed ? 1u : 0u;
    c.seed = o.seed + 0x9E3779B97F4A7C15ull * (i + 1);
  }
  SED_TRY_CUDA(cudaMemcpyAsync(base + off_chains, chains.data(), sizeof(ChainDesc) * count, cudaMemcpyHostToDevice, stream));
  {
    uint32_t max_codes = 1;
    for (unsigned i = 0; i < count; ++i) max_codes = std::max(max_codes, od[i]->tables->n_codes);
    k_split_tables<<<dim3((max_codes + 255) / 256, count), 256, 0, stream>>>(
        reinterpret_cast<ChainDesc const*>(base + off_chains));
    note_launches(1);
  }

  uint32_t const max_steps_total = o.max_iter ? std::max<uint32_t>(1, o.max_iter / kB) : 2000;
  auto run = [&](Plan const& p, uint32_t max_steps, float* ms) -> int {
    unsigned const grid = (unsigned)sms * p.ctas_per_sm;
    Layout L = make_layout(grid);
    for (auto& g : L.groups) g.bar = reinterpret_cast<uint32_t*>(base + off_bars) + 2 * (&g - L.groups.data());
    unsigned const used = (unsigned)L.cta_group.size();
    SED_TRY_CUDA(cudaMemcpyAsync(base + off_groups, L.groups.data(), sizeof(GroupDesc) * L.groups.size(), cudaMemcpyHostToDevice, stream));
    SED_TRY_CUDA(cudaMemcpyAsync(base + off_ctag, L.cta_group.data(), 4 * (size_t)used, cudaMemcpyHostToDevice, stream));
    SED_TRY_CUDA(cudaMemcpyAsync(base + off_order, L.order.data(), 4 * (size_t)count, cudaMemcpyHostToDevice, stream));
    SED_TRY_CUDA(cudaMemsetAsync(base + off_bars, 0, 8 * (size_t)max_grid, stream));
    SED_TRY_CUDA(cudaMemsetAsync(base + off_err, 0, 16, stream));
    for (unsigned i = 0; i < count; ++i) SED_TRY_CUDA(cudaMemsetAsync(base + off_out[i], 0, kOutBytes, stream));
    BatchArgs a;
    a.chains = reinterpret_cast<ChainDesc const*>(base + off_chains);
    a.groups = reinterpret_cast<GroupDesc const*>(base + off_groups);
    a.cta_group = reinterpret_cast<uint32_t const*>(base + off_ctag);
    a.order = reinterpret_cast<uint32_t const*>(base + off_order);
    a.tol = tol;
    a.max_steps = max_steps;
    a.rr_every = 4;  // measured on the 128-chain workload: 772 ms against 797 ms every 2 steps, same step counts
    a.error = reinterpret_cast<int*>(base + off_err);
    a.wait_ns = device_wait_ns(kBarrierNs);
    a.copy_wait_ns = device_wait_ns(kGsWaitNs);
    a.extra_arrivals = g_barrier_extra_arrivals.load();
    cudaEvent_t e0, e1;
    SED_TRY_CUDA(cudaEventCreate(&e0));
    SED_TRY_CUDA(cudaEventCreate(&e1));
    void* kargs[] = {&a};
    SED_TRY_CUDA(cudaEventRecord(e0, stream));
    cudaError_t le = cudaLaunchCooperativeKernel((void const*)k_batch_lanczos, dim3(used), dim3(p.threads), kargs,
                                                 dyn_smem(), stream);
    note_launches(1);
    SED_TRY_CUDA(cudaEventRecord(e1, stream));
    int err = 0;
    SED_TRY_CUDA(cudaMemcpyAsync(&err, base + off_err, 4, cudaMemcpyDeviceToHost, stream));
    cudaError_t se = cudaStreamSynchronize(stream);
    if (ms) cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    SED_TRY_CUDA(le);
    SED_TRY_CUDA(se);
    if (err) return fail(LS_DEVICE_TIMEOUT, err == 3 ? "sed_eigh_batched: a wait for a shared-memory copy timed out"
                                                    : "sed_eigh_batched: a group barrier timed out");
    return LS_SUCCESS;
  };

  if (!tuned && cands.size() > 1) {
    float best = 3e38f;
    for (Plan const& p : cands) {
      float ms = 0;
      if (int st = run(p, 2, &ms)) return st;
      if (ms < best) {
        best = ms;
        plan = p;
      }
    }
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[key] = plan;
  }
  auto t_solve0 = std::chrono::steady_clock::now();
  float solve_ms = 0;
  if (int st = run(plan, max_steps_total, &solve_ms)) return st;

  // results
  std::vector<double> outs(12);
  std::vector<uint32_t> stats(4);
  bool all_ok = true;
  uint64_t max_steps = 0, max_restarts = 0, breakdowns = 0;
  std::string first_bad;
  for (unsigned i = 0; i < count; ++i) {
    SED_TRY_CUDA(cudaMemcpy(outs.data(), base + off_out[i], 96, cudaMemcpyDeviceToHost));
    SED_TRY_CUDA(cudaMemcpy(stats.data(), base + off_out[i] + kStatsOff, 16, cudaMemcpyDeviceToHost));
    for (uint32_t k = 0; k < nev; ++k) {
      eigenvalues[(size_t)i * nev + k] = outs[k];
      if (residuals) residuals[(size_t)i * nev + k] = outs[8 + k];
    }
    max_steps = std::max<uint64_t>(max_steps, stats[0]);
    max_restarts = std::max<uint64_t>(max_restarts, stats[1]);
    if (stats[3] != 1) {
      if (all_ok) {
        char buf[256];
        std::snprintf(buf, sizeof buf, " (first: problem %u, D = %llu, %u block steps, %u restarts, status %u, "
                      "residuals %.2e %.2e %.2e %.2e)", i, (unsigned long long)od[i]->basis->D, stats[0], stats[1],
                      stats[3], outs[8], outs[9], outs[10], outs[11]);
        first_bad = buf;
      }
      all_ok = false;
    }
    if (stats[3] == 3) ++breakdowns;
    if (eigenvectors && eigenvectors[i]) {
      uint64_t const D = od[i]->basis->D;
      uint64_t const ld = ldv ? ldv[i] : D;
      if (ld < D) return fail(LS_INVALID_ARGUMENT, "sed_eigh_batched: ldv below the dimension");
      DeviceBuffer tmpv;
      if (int st = tmpv.allocate((size_t)ld * nev * 8)) return st;
      { k_unpack_block<<<grid_size(D * nev, device), kBlock, 0, stream>>>(reinterpret_cast<double const*>(base + off_V[i]), D, nev, tmpv.as<double>(), ld); note_launches(1); }
      SED_TRY_CUDA(cudaMemcpyAsync(eigenvectors[i], tmpv.ptr, ((size_t)ld * (nev - 1) + D) * 8, cudaMemcpyDefault, stream));
      SED_TRY_CUDA(cudaStreamSynchronize(stream));
    }
  }
  if (logging_enabled()) {
    unsigned worst = 0;
    uint64_t worst_t = 0;
    std::vector<uint64_t> prof(8);
    Layout const L0 = make_layout((unsigned)sms * plan.ctas_per_sm);
    for (unsigned i = 0; i < count; ++i) {
      SED_TRY_CUDA(cudaMemcpy(prof.data(), base + off_out[i] + kProfOff, 64, cudaMemcpyDeviceToHost));
      SED_TRY_CUDA(cudaMemcpy(stats.data(), base + off_out[i] + kStatsOff, 16, cudaMemcpyDeviceToHost));
      uint64_t t = 0;
      for (int q = 0; q < 6; ++q) t += prof[q];
      GroupDesc const& g = L0.groups[L0.group_of_chain[i]];
      log_line("sed_eigh_batched: problem %u: D = %llu, group %u (%u CTAs, %u problems), %u block steps, %.2f ms "
               "(rayleigh-ritz %.2f ms)", i, (unsigned long long)od[i]->basis->D, L0.group_of_chain[i], g.ncta,
               g.count, stats[0], t * 1e-6, prof[3] * 1e-6);
      if (t > worst_t) {
        worst_t = t;
        worst = i;
      }
    }
    SED_TRY_CUDA(cudaMemcpy(prof.data(), base + off_out[worst] + kProfOff, 64, cudaMemcpyDeviceToHost));
    SED_TRY_CUDA(cudaMemcpy(stats.data(), base + off_out[worst] + kStatsOff, 16, cudaMemcpyDeviceToHost));
    unsigned const ncta = L0.groups[L0.group_of_chain[worst]].ncta;
    log_line("sed_eigh_batched: slowest problem %u (D = %llu, %u CTAs, %u block steps, %u restarts): spmv %.2f ms, "
             "cgs2 %.2f ms, qr %.2f ms, rayleigh-ritz %.2f ms, ritz/restart %.2f ms, residual %.2f ms",
             worst, (unsigned long long)od[worst]->basis->D, ncta, stats[0], stats[1], prof[0] * 1e-6,
             prof[1] * 1e-6, prof[2] * 1e-6, prof[3] * 1e-6, prof[4] * 1e-6, prof[5] * 1e-6);
  }
  auto t_end = std::chrono::steady_clock::now();
  if (info) {
    info->block_steps_max = max_steps;
    info->restarts_max = max_restarts;
    info->seconds_total = std::chrono::duration<double>(t_end - t_start).count();
    info->seconds_setup = std::chrono::duration<double>(t_setup - t_start).count();
    info->seconds_solve = std::chrono::duration<double>(t_end - t_solve0).count();
    info->kernel_ms = solve_ms;
    info->ctas_per_sm = plan.ctas_per_sm;
    info->threads_per_cta = plan.threads;
    info->grid = (uint32_t)(sms * plan.ctas_per_sm);
  }
  if (logging_enabled())
    log_line("sed_eigh_batched: %u problems, %.3f ms in one launch (%u CTAs/SM), max %llu block steps", count,
             solve_ms, plan.ctas_per_sm, (unsigned long long)max_steps);
  if (!all_ok)
    return fail(LS_NOT_CONVERGED, std::string(breakdowns ? "sed_eigh_batched: Krylov breakdown in some problems"
                                                         : "sed_eigh_batched: some problems did not converge") +
                                      first_bad);
  return LS_SUCCESS;
}

}  // extern "C"

extern "C" void sed_set_batched_launch(unsigned threads_per_cta, unsigned ctas_per_sm) {
  sed::g_force_threads.store(threads_per_cta ? threads_per_cta : 0u);
  sed::g_force_per_sm.store(threads_per_cta ? ctas_per_sm : 0u);
}

extern "C" unsigned sed_debug_batched_layout(unsigned count, double const* work, uint32_t const* max_ctas, double fixed,
                                             unsigned grid, uint32_t* group_of, uint32_t* ncta, uint32_t* nprob) {
  if (count == 0 || grid == 0 || !work || !max_ctas || !group_of || !ncta || !nprob || !(fixed >= 0.0)) return 0;
  std::vector<double> w(work, work + count);
  std::vector<uint32_t> m(max_ctas, max_ctas + count);
  for (double x : w)
    if (!(x >= 0.0)) return 0;
  sed::BatchLayout const L = sed::batch_layout(w, m, fixed, grid);
  if (L.groups.size() > grid) return 0;
  for (unsigned i = 0; i < count; ++i) group_of[i] = L.group_of_chain[i];
  for (size_t g = 0; g < L.groups.size(); ++g) {
    ncta[g] = L.groups[g].ncta;
    nprob[g] = L.groups[g].count;
  }
  return (unsigned)L.groups.size();
}
