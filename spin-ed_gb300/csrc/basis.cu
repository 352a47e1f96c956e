// basis.cu — symmetry-adapted spin basis: construction, representative
// enumeration on the GPU, export (src/SpinED/Internal.hs:157-254).
//
// ls_build enumerates every word of the fixed-Hamming-weight space (or all
// 2^n words) in increasing order and keeps the orbit minima whose stabiliser
// carries the trivial character. Three passes keep the output sorted without
// any sort:
//   1. mark:  one thread per 32 consecutive words (unranked once, then the
//             next word of equal weight) writes a 32-bit mask of the words that
//             are representatives;
//   2. scan:  per-tile popcounts, an exclusive scan over tiles;
//   3. write: each tile re-walks its marked words and writes them, with their
//             stabiliser orders, at the scanned offsets.
// A prefix table over the top bits of the representatives then serves the
// index lookups of the matvec.
#include <algorithm>
#include <vector>
#include <cstring>

#include "sed_internal.hpp"

namespace sed {
namespace {

constexpr unsigned kThreads = 256;
constexpr unsigned kTileWords = kThreads * 8;  // bitmap words per tile

constexpr unsigned kMaxSegs = 1024;  // top-row segments of the rank space (2^row_bits <= 1024)

// Marks representatives: bitmap word t holds ranks 32 t .. 32 t + 31. With
// segments (n_seg > 0), only the bitmap words listed in them are examined
// (the others were zeroed): on a torus a representative's top row must be
// the smallest rotation of itself and of its inverse, and the words with a
// given top row form one contiguous rank range, so whole ranges are skipped.
template <class W>
__global__ void k_mark(__grid_constant__ const PlanView P, uint64_t const* __restrict__ binom, unsigned n, int hw,
                       uint64_t space, uint64_t n_words, uint32_t* __restrict__ bitmap,
                       uint64_t const* __restrict__ seg_begin, uint64_t const* __restrict__ seg_prefix, uint32_t n_seg) {
  __shared__ uint16_t srow[2048], sline[2048];
  __shared__ uint64_t sb[kMaxSegs], sp[kMaxSegs + 1];
  stage_lines(P, sline);
  RowTab RT = stage_rows(P, srow);
  attach_lines(P, sline, RT);
  for (uint32_t q = threadIdx.x; q < n_seg; q += blockDim.x) {
    sb[q] = seg_begin[q];
    sp[q] = seg_prefix[q];
  }
  if (threadIdx.x == 0 && n_seg) sp[n_seg] = seg_prefix[n_seg];
  __syncthreads();
  uint64_t const total = n_seg ? sp[n_seg] : n_words;
  for (uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total;
       u += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t t = u;
    if (n_seg) {  // segment holding u: the last with prefix <= u
      uint32_t lo = 0, hi = n_seg - 1;
      while (lo < hi) {
        uint32_t const mid = (lo + hi + 1) >> 1;
        if (sp[mid] <= u) lo = mid;
        else hi = mid - 1;
      }
      t = sb[lo] + (u - sp[lo]);
    }
    uint64_t const r0 = t * 32;
    unsigned const count = (unsigned)min((uint64_t)32, space - r0);
    uint64_t x = unrank_word(r0, n, hw, binom);
    uint32_t mask = 0;
    for (unsigned k = 0; k < count; ++k) {
      if (representative_weight<W>((W)x, P, RT)) mask |= 1u << k;
      if (k + 1 < count) x = hw >= 0 ? next_same_weight(x) : x + 1;
    }
    bitmap[t] = mask;
  }
}

__global__ void k_tile_counts(uint32_t const* __restrict__ bitmap, uint64_t n_words,
                              uint64_t* __restrict__ tile_count) {
  __shared__ uint64_t part[kThreads / 32];
  uint64_t const base = (uint64_t)blockIdx.x * kTileWords;
  uint64_t c = 0;
  for (unsigned j = 0; j < 8; ++j) {
    uint64_t const w = base + (uint64_t)j * kThreads + threadIdx.x;
    if (w < n_words) c += __popc(bitmap[w]);
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t s = 0;
    for (unsigned i = 0; i < kThreads / 32; ++i) s += part[i];
    tile_count[blockIdx.x] = s;
  }
}

// Exclusive scan of n values in place by one block; out[n] = total.
__global__ void k_scan_serial(uint64_t* __restrict__ v, uint64_t n) {
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

__global__ void k_write(uint64_t const* __restrict__ binom, unsigned n, int hw, uint64_t space,
                        uint32_t const* __restrict__ bitmap, uint64_t n_words,
                        uint64_t const* __restrict__ tile_offset, uint64_t* __restrict__ reps) {
  __shared__ uint32_t scan[kThreads];
  uint64_t const w0 = (uint64_t)blockIdx.x * kTileWords + (uint64_t)threadIdx.x * 8;
  uint32_t m[8];
  uint32_t c = 0;
  for (unsigned j = 0; j < 8; ++j) {
    m[j] = (w0 + j < n_words) ? bitmap[w0 + j] : 0u;
    c += __popc(m[j]);
  }
  scan[threadIdx.x] = c;
  __syncthreads();
  for (unsigned o = 1; o < kThreads; o <<= 1) {
    uint32_t const v = threadIdx.x >= o ? scan[threadIdx.x - o] : 0u;
    __syncthreads();
    scan[threadIdx.x] += v;
    __syncthreads();
  }
  uint64_t pos = tile_offset[blockIdx.x] + scan[threadIdx.x] - c;
  for (unsigned j = 0; j < 8; ++j) {
    if (!m[j]) continue;
    uint64_t const r0 = (w0 + j) * 32;
    unsigned const count = (unsigned)min((uint64_t)32, space - r0);
    uint64_t x = unrank_word(r0, n, hw, binom);
    for (unsigned k = 0; k < count; ++k) {
      if (m[j] >> k & 1u) reps[pos++] = x;
      if (k + 1 < count) x = hw >= 0 ? next_same_weight(x) : x + 1;
    }
  }
}

// Stabiliser orders of the written representatives, one thread per entry.
template <class W>
__global__ void k_weights(__grid_constant__ const PlanView P, uint64_t const* __restrict__ reps, uint64_t D,
                          uint32_t* __restrict__ weights) {
  __shared__ uint16_t srow[2048], sline[2048];
  stage_lines(P, sline);
  RowTab RT = stage_rows(P, srow);
  attach_lines(P, sline, RT);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D;
       i += (uint64_t)gridDim.x * blockDim.x)
    weights[i] = representative_weight<W>((W)reps[i], P, RT);
}

template <class W>
__global__ void k_check_reps(__grid_constant__ const PlanView P, uint64_t const* __restrict__ reps, uint64_t D,
                             uint32_t* __restrict__ weights, unsigned n, int hw,
                             uint32_t* __restrict__ bad) {
  __shared__ uint16_t srow[2048], sline[2048];
  stage_lines(P, sline);
  RowTab RT = stage_rows(P, srow);
  attach_lines(P, sline, RT);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t const x = reps[i];
    uint32_t w = 0;
    bool ok = (n == 64 || (x >> n) == 0) && (hw < 0 || __popcll(x) == hw);
    if (ok) w = representative_weight<W>((W)x, P, RT);
    if (i + 1 < D && reps[i + 1] <= x) ok = false;
    weights[i] = w;
    if (!ok || w == 0) bad[0] = 1u;  // any writer stores the same value
  }
}

__global__ void k_prefix(uint64_t const* __restrict__ reps, uint64_t D, unsigned shift,
                         uint64_t n_keys, uint64_t* __restrict__ prefix) {
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k <= n_keys;
       k += (uint64_t)gridDim.x * blockDim.x) {
    if (k == n_keys) {
      prefix[k] = D;
      continue;
    }
    uint64_t const key = k << shift;
    uint64_t lo = 0, hi = D;
    while (lo < hi) {
      uint64_t const mid = (lo + hi) >> 1;
      if (reps[mid] < key)
        lo = mid + 1;
      else
        hi = mid;
    }
    prefix[k] = lo;
  }
}

unsigned grid_for(uint64_t work, int device) {
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  uint64_t const want = (work + kThreads - 1) / kThreads;
  uint64_t const cap = (uint64_t)sms * 16;
  return (unsigned)std::max<uint64_t>(1, std::min(want, cap));
}

}  // namespace

int basis_upload_plan(BasisData& b, cudaStream_t stream) {
  if (b.plan_buf.ptr) return LS_SUCCESS;
  SymPlanHost const& p = b.plan;
  auto align = [](size_t v) { return (v + 15) & ~(size_t)15; };
  struct Part {
    void const* src;
    size_t bytes;
    size_t off;
  };
  std::vector<Part> parts = {
      {p.benes_mask.data(), p.benes_mask.size() * 8, 0}, {p.benes_shift.data(), p.benes_shift.size() * 4, 0},
      {p.h_mask.data(), p.h_mask.size() * 8, 0},         {p.h_rot.data(), p.h_rot.size() * 4, 0},
      {p.coset_phase.data(), p.coset_phase.size() * 4, 0}, {p.h_phase.data(), p.h_phase.size() * 4, 0},
      {p.row_min.data(), p.row_min.size() * 2, 0},       {p.row_set.data(), p.row_set.size() * 2, 0},
      {p.rot_mask.data(), p.rot_mask.size() * 8, 0},     {p.rot_rot.data(), p.rot_rot.size() * 4, 0},
      {p.rot_exp.data(), p.rot_exp.size() * 4, 0},       {p.sh_mask.data(), p.sh_mask.size() * 8, 0},
      {p.sh_rot.data(), p.sh_rot.size() * 4, 0},         {p.sh_exp.data(), p.sh_exp.size() * 4, 0},
      {p.pos.data(), p.pos.size(), 0},
      {p.line_row.data(), p.line_row.size() * 2, 0},     {p.line_col.data(), p.line_col.size() * 2, 0},
  };
  size_t total = 16;
  for (auto& q : parts) {
    q.off = total;
    total += align(q.bytes);
  }
  std::vector<uint8_t> host(total, 0);
  for (auto const& q : parts)
    if (q.bytes) std::memcpy(host.data() + q.off, q.src, q.bytes);
  if (int st = b.plan_buf.allocate(total)) return st;
  SED_TRY_CUDA(cudaMemcpyAsync(b.plan_buf.ptr, host.data(), total, cudaMemcpyHostToDevice, stream));
  uint8_t* base = b.plan_buf.as<uint8_t>();
  PlanView v = p.view();
  v.benes_mask = (uint64_t const*)(base + parts[0].off);
  v.benes_shift = (uint32_t const*)(base + parts[1].off);
  v.h_mask = (uint64_t const*)(base + parts[2].off);
  v.h_rot = (uint32_t const*)(base + parts[3].off);
  v.coset_phase = (uint32_t const*)(base + parts[4].off);
  v.h_phase = (uint32_t const*)(base + parts[5].off);
  v.row_min = (uint16_t const*)(base + parts[6].off);
  v.row_set = (uint16_t const*)(base + parts[7].off);
  v.rot_mask = (uint64_t const*)(base + parts[8].off);
  v.rot_rot = (uint32_t const*)(base + parts[9].off);
  v.rot_exp = (uint32_t const*)(base + parts[10].off);
  v.sh_mask = (uint64_t const*)(base + parts[11].off);
  v.sh_rot = (uint32_t const*)(base + parts[12].off);
  v.sh_exp = (uint32_t const*)(base + parts[13].off);
  v.pos = (uint8_t const*)(base + parts[14].off);
  v.line_row = (uint16_t const*)(base + parts[15].off);
  v.line_col = (uint16_t const*)(base + parts[16].off);
  b.plan_dev = v;
  std::vector<uint64_t> binom(65 * 65, 0);
  for (unsigned i = 0; i <= 64; ++i) {
    binom[i * 65] = 1;
    for (unsigned j = 1; j <= 64; ++j)
      binom[i * 65 + j] = i == 0 ? 0 : binom[(i - 1) * 65 + j - 1] + binom[(i - 1) * 65 + j];
  }
  if (int st = b.binom.allocate(binom.size() * 8)) return st;
  SED_TRY_CUDA(cudaMemcpyAsync(b.binom.ptr, binom.data(), binom.size() * 8, cudaMemcpyHostToDevice, stream));
  SED_TRY_CUDA(cudaStreamSynchronize(stream));
  return LS_SUCCESS;
}

IndexView BasisData::index_view() const {
  IndexView I{};
  I.reps = reps.as<uint64_t const>();
  I.prefix = prefix.as<uint64_t const>();
  I.D = D;
  I.bits = prefix_bits;
  I.shift = prefix_shift;
  return I;
}

int basis_build_index(BasisData& b, cudaStream_t stream) {
  uint64_t max_rep = 0;
  if (b.D) SED_TRY_CUDA(cudaMemcpy(&max_rep, b.reps.as<uint64_t>() + b.D - 1, 8, cudaMemcpyDeviceToHost));
  unsigned bitlen = 0;
  while (bitlen < 64 && (max_rep >> bitlen)) ++bitlen;
  unsigned want = 1;
  while (want < 26 && ((uint64_t)1 << want) < b.D) ++want;  // about one key per entry
  b.prefix_bits = std::max(1u, std::min(bitlen ? bitlen : 1u, want));
  b.prefix_shift = bitlen > b.prefix_bits ? bitlen - b.prefix_bits : 0;
  uint64_t const n_keys = (uint64_t)1 << b.prefix_bits;
  if (int st = b.prefix.allocate((n_keys + 1) * 8)) return st;
  { k_prefix<<<grid_for(n_keys + 1, b.device), kThreads, 0, stream>>>(
      b.reps.as<uint64_t>(), b.D, b.prefix_shift, n_keys, b.prefix.as<uint64_t>()); note_launches(1); }
  SED_TRY_CUDA(cudaGetLastError());
  return LS_SUCCESS;
}

namespace {

int ensure_plan_checked(BasisData& b) {
  if (b.plan_checked) return LS_SUCCESS;
  if (int st = check_plan(b.plan)) return st;
  b.plan_checked = true;
  return LS_SUCCESS;
}

int build_impl(BasisData& b, uint64_t const* given, uint64_t given_size) {
  if (b.device < 0 || !b.plan_buf.ptr)
    if (int st = current_device(&b.device)) return st;
  ScopedDevice dev(b.device);
  cudaStream_t stream;
  SED_TRY_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } guard{stream};
  if (int st = basis_upload_plan(b, stream)) return st;
  bool const wide = b.plan.n_bits > 32;
  PlanView const P = b.plan_dev;
  b.built = false;
  b.reps.reset();
  b.weights.reset();
  b.prefix.reset();
  if (given) {
    if (int st = ensure_plan_checked(b)) return st;
    b.D = given_size;
    if (int st = b.reps.allocate(std::max<uint64_t>(1, given_size) * 8)) return st;
    if (int st = b.weights.allocate(std::max<uint64_t>(1, given_size) * 4)) return st;
    if (given_size)
      SED_TRY_CUDA(cudaMemcpyAsync(b.reps.ptr, given, given_size * 8, cudaMemcpyDefault, stream));
    DeviceBuffer bad;
    if (int st = bad.allocate(4)) return st;
    SED_TRY_CUDA(cudaMemsetAsync(bad.ptr, 0, 4, stream));
    if (given_size) {
      unsigned const grid = grid_for(given_size, b.device);
      if (wide)
        { k_check_reps<uint64_t><<<grid, kThreads, 0, stream>>>(P, b.reps.as<uint64_t>(), given_size,
                                                             b.weights.as<uint32_t>(), b.n, b.hw,
                                                             bad.as<uint32_t>()); note_launches(1); }
      else
        { k_check_reps<uint32_t><<<grid, kThreads, 0, stream>>>(P, b.reps.as<uint64_t>(), given_size,
                                                             b.weights.as<uint32_t>(), b.n, b.hw,
                                                             bad.as<uint32_t>()); note_launches(1); }
      SED_TRY_CUDA(cudaGetLastError());
    }
    uint32_t bad_h = 0;
    SED_TRY_CUDA(cudaMemcpyAsync(&bad_h, bad.ptr, 4, cudaMemcpyDeviceToHost, stream));
    SED_TRY_CUDA(cudaStreamSynchronize(stream));
    if (bad_h)
      return fail(LS_NOT_A_REPRESENTATIVE,
                  "ls_build_unsafe: the list is not a strictly increasing list of representatives "
                  "of this sector");
  } else {
    // Space size.
    uint64_t space;
    if (b.hw >= 0) {
      uint64_t row[65] = {1};
      for (unsigned i = 1; i <= b.n; ++i)
        for (unsigned j = i; j >= 1; --j) row[j] += row[j - 1];  // Pascal row n
      space = row[b.hw];
    } else {
      if (b.n >= 48) return fail(LS_OUT_OF_MEMORY, "ls_build: 2^n words do not fit the device");
      space = (uint64_t)1 << b.n;
    }
    uint64_t const n_words = (space + 31) / 32;
    uint64_t const n_tiles = (n_words + kTileWords - 1) / kTileWords;
    DeviceBuffer bitmap, tiles, segs;
    if (int st = bitmap.allocate(std::max<uint64_t>(1, n_words) * 4)) return st;
    if (int st = tiles.allocate((n_tiles + 1) * 8)) return st;
    // Top-row segments (tori): the rank range of the words with top row T is
    // [lo_T, lo_T + cnt_T) in increasing T; keep the T whose value is its own
    // smallest rotation and no larger than its inverse's smallest rotation.
    std::vector<uint64_t> seg_b, seg_p;
    if (b.plan.rows == 1 && b.plan.row_bits <= 10 && b.n >= b.plan.row_bits) {
      unsigned const B = b.plan.row_bits, low = b.n - B;
      uint32_t const rm = (1u << B) - 1;
      uint64_t lo = 0, kept = 0;
      for (uint32_t T = 0; T <= rm; ++T) {
        int const need = b.hw - __builtin_popcount(T);
        uint64_t const cnt = b.hw < 0 ? ((uint64_t)1 << low)
                                      : (need < 0 || (unsigned)need > low ? 0 : host_binom(low, (unsigned)need));
        bool ok = b.plan.row_min[T] == T;
        if (b.plan.inv) ok = ok && b.plan.row_min[T ^ rm] >= T;
        if (ok && cnt) {
          // a bitmap word shared with the neighbouring range is examined by
          // both segments: same word, same result
          uint64_t const wb = lo / 32, we = (lo + cnt + 31) / 32;
          seg_b.push_back(wb);
          seg_p.push_back(kept);
          kept += we - wb;
        }
        lo += cnt;
      }
      seg_p.push_back(kept);
      if (seg_b.size() > kMaxSegs || lo != space) {
        seg_b.clear();
        seg_p.clear();
      }
    }
    uint32_t const n_seg = (uint32_t)seg_b.size();
    if (n_seg) {
      if (int st = segs.allocate((2 * (size_t)n_seg + 1) * 8)) return st;
      SED_TRY_CUDA(cudaMemcpyAsync(segs.ptr, seg_b.data(), n_seg * 8, cudaMemcpyHostToDevice, stream));
      SED_TRY_CUDA(cudaMemcpyAsync(segs.as<uint64_t>() + n_seg, seg_p.data(), (n_seg + 1) * 8, cudaMemcpyHostToDevice,
                                   stream));
      SED_TRY_CUDA(cudaMemsetAsync(bitmap.ptr, 0, std::max<uint64_t>(1, n_words) * 4, stream));
    }
    uint64_t const work = n_seg ? seg_p.back() : n_words;
    unsigned const grid = grid_for(std::max<uint64_t>(1, work), b.device) * 4;
    uint64_t const* sbeg = n_seg ? segs.as<uint64_t>() : nullptr;
    uint64_t const* spre = n_seg ? segs.as<uint64_t>() + n_seg : nullptr;
    if (wide)
      { k_mark<uint64_t><<<grid, kThreads, 0, stream>>>(P, b.binom.as<uint64_t>(), b.n, b.hw, space,
                                                       n_words, bitmap.as<uint32_t>(), sbeg, spre, n_seg); note_launches(1); }
    else
      { k_mark<uint32_t><<<grid, kThreads, 0, stream>>>(P, b.binom.as<uint64_t>(), b.n, b.hw, space,
                                                       n_words, bitmap.as<uint32_t>(), sbeg, spre, n_seg); note_launches(1); }
    SED_TRY_CUDA(cudaGetLastError());
    // the plan's host self-check runs while the scan runs on the device
    if (int st = ensure_plan_checked(b)) {
      cudaStreamSynchronize(stream);
      return st;
    }
    if (n_tiles) {
      { k_tile_counts<<<(unsigned)n_tiles, kThreads, 0, stream>>>(bitmap.as<uint32_t>(), n_words,
                                                                tiles.as<uint64_t>()); note_launches(1); }
      SED_TRY_CUDA(cudaGetLastError());
    }
    { k_scan_serial<<<1, 1024, 0, stream>>>(tiles.as<uint64_t>(), n_tiles); note_launches(1); }
    SED_TRY_CUDA(cudaGetLastError());
    uint64_t D = 0;
    SED_TRY_CUDA(cudaMemcpyAsync(&D, tiles.as<uint64_t>() + n_tiles, 8, cudaMemcpyDeviceToHost, stream));
    SED_TRY_CUDA(cudaStreamSynchronize(stream));
    b.D = D;
    if (int st = b.reps.allocate(std::max<uint64_t>(1, D) * 8)) return st;
    if (int st = b.weights.allocate(std::max<uint64_t>(1, D) * 4)) return st;
    if (n_tiles) {
      { k_write<<<(unsigned)n_tiles, kThreads, 0, stream>>>(b.binom.as<uint64_t>(), b.n, b.hw, space,
                                                          bitmap.as<uint32_t>(), n_words, tiles.as<uint64_t>(),
                                                          b.reps.as<uint64_t>()); note_launches(1); }
      SED_TRY_CUDA(cudaGetLastError());
    }
    if (D) {
      unsigned const grid = grid_for(D, b.device);
      if (wide)
        { k_weights<uint64_t><<<grid, kThreads, 0, stream>>>(P, b.reps.as<uint64_t>(), D, b.weights.as<uint32_t>()); note_launches(1); }
      else
        { k_weights<uint32_t><<<grid, kThreads, 0, stream>>>(P, b.reps.as<uint64_t>(), D, b.weights.as<uint32_t>()); note_launches(1); }
      SED_TRY_CUDA(cudaGetLastError());
    }
    SED_TRY_CUDA(cudaStreamSynchronize(stream));
  }
  if (int st = basis_build_index(b, stream)) return st;
  SED_TRY_CUDA(cudaStreamSynchronize(stream));
  b.built = true;
  if (logging_enabled()) log_line("basis built: %llu representatives", (unsigned long long)b.D);
  return LS_SUCCESS;
}

}  // namespace

bool characters_real(BasisData const& b) {
  for (uint32_t ph : b.plan.coset_phase)
    if ((2 * ph) % b.plan.L) return false;
  for (uint32_t ph : b.plan.h_phase)
    if ((2 * ph) % b.plan.L) return false;
  return true;
}

}  // namespace sed

using namespace sed;

extern "C" {

int ls_create_spin_basis(ls_spin_basis** ptr, ls_group const* group, unsigned number_spins,
                         int hamming_weight, int spin_inversion) {
  if (!ptr || !group) return fail(LS_INVALID_ARGUMENT, "ls_create_spin_basis: NULL argument");
  if (number_spins == 0 || number_spins > 64)
    return fail(LS_INVALID_NUMBER_SPINS, "number of spins must be in 1..64, got " + std::to_string(number_spins));
  if (group->d.n && group->d.n != number_spins)
    return fail(LS_INVALID_NUMBER_SPINS, "symmetries act on " + std::to_string(group->d.n) +
                                             " sites but the basis has " + std::to_string(number_spins));
  if (hamming_weight < -1 || hamming_weight > (int)number_spins)
    return fail(LS_INVALID_HAMMING_WEIGHT, "Hamming weight must be -1 or in 0..number_spins");
  if (spin_inversion < -1 || spin_inversion > 1)
    return fail(LS_INVALID_SPIN_INVERSION, "spin inversion must be -1, 0 or +1");
  if (spin_inversion != 0 && hamming_weight != -1 && 2 * hamming_weight != (int)number_spins)
    return fail(LS_INVALID_SPIN_INVERSION,
                "spin inversion needs Hamming weight number_spins / 2 (or no Hamming weight)");
  try {
    auto d = std::make_shared<BasisData>();
    d->n = number_spins;
    d->hw = hamming_weight;
    d->inv = spin_inversion;
    d->group = group->d;
    if (int st = build_plan(d->group, number_spins, spin_inversion, d->plan, false)) return st;
    d->device = -1;  // bound to the current device by ls_build
    auto* b = new ls_spin_basis;
    b->d = std::move(d);
    *ptr = b;
    return LS_SUCCESS;
  } catch (std::bad_alloc const&) {
    return fail(LS_OUT_OF_MEMORY, "ls_create_spin_basis");
  } catch (std::exception const& e) {
    return fail(LS_SYSTEM_ERROR, e.what());
  }
}

void ls_destroy_spin_basis(ls_spin_basis* basis) { delete basis; }

int ls_build(ls_spin_basis* basis) {
  if (!basis) return fail(LS_INVALID_ARGUMENT, "ls_build: NULL basis");
  std::lock_guard<std::mutex> lock(basis->d->mu);
  try {
    return build_impl(*basis->d, nullptr, 0);
  } catch (std::exception const& e) {
    return fail(LS_SYSTEM_ERROR, e.what());
  }
}

int ls_build_unsafe(ls_spin_basis* basis, uint64_t size, uint64_t const representatives[]) {
  if (!basis || (size && !representatives)) return fail(LS_INVALID_ARGUMENT, "ls_build_unsafe: NULL argument");
  std::lock_guard<std::mutex> lock(basis->d->mu);
  try {
    {
      ScopedDevice dev(basis->d->device);
      if (int st = wait_for_caller({representatives})) return st;
    }
    return build_impl(*basis->d, representatives, size);
  } catch (std::exception const& e) {
    return fail(LS_SYSTEM_ERROR, e.what());
  }
}

int ls_get_number_states(ls_spin_basis const* basis, uint64_t* out) {
  if (!basis || !out) return fail(LS_INVALID_ARGUMENT, "ls_get_number_states: NULL argument");
  if (!basis->d->built) return fail(LS_CACHE_NOT_BUILT, "basis has not been built (call ls_build)");
  *out = basis->d->D;
  return LS_SUCCESS;
}

int ls_get_states(ls_states** ptr, ls_spin_basis const* basis) {
  if (!ptr || !basis) return fail(LS_INVALID_ARGUMENT, "ls_get_states: NULL argument");
  BasisData& b = *basis->d;
  if (!b.built) return fail(LS_CACHE_NOT_BUILT, "basis has not been built (call ls_build)");
  try {
    auto* s = new ls_states;
    s->data.reset(new uint64_t[b.D ? b.D : 1]);
    s->size = b.D;
    ScopedDevice dev(b.device);
    if (b.D) {
      cudaError_t e = cudaMemcpy(s->data.get(), b.reps.ptr, b.D * 8, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) {
        delete s;
        return fail(LS_CUDA_ERROR, std::string("ls_get_states: ") + cudaGetErrorString(e));
      }
    }
    *ptr = s;
    return LS_SUCCESS;
  } catch (std::bad_alloc const&) {
    return fail(LS_OUT_OF_MEMORY, "ls_get_states");
  }
}

uint64_t const* ls_states_get_data(ls_states const* states) {
  return states ? states->data.get() : nullptr;
}
uint64_t ls_states_get_size(ls_states const* states) { return states ? states->size : 0; }
void ls_destroy_states(ls_states* states) { delete states; }

int sed_basis_get_norms(ls_spin_basis const* basis, double* out) {
  if (!basis || !out) return fail(LS_INVALID_ARGUMENT, "sed_basis_get_norms: NULL argument");
  BasisData& b = *basis->d;
  if (!b.built) return fail(LS_CACHE_NOT_BUILT, "basis has not been built (call ls_build)");
  std::vector<uint32_t> w(b.D);
  ScopedDevice dev(b.device);
  if (b.D) SED_TRY_CUDA(cudaMemcpy(w.data(), b.weights.ptr, b.D * 4, cudaMemcpyDeviceToHost));
  double const G = (double)b.plan.group_order;
  for (uint64_t i = 0; i < b.D; ++i) out[i] = std::sqrt((double)w[i] / G);
  return LS_SUCCESS;
}

uint64_t const* sed_basis_device_states(ls_spin_basis const* basis) {
  return (basis && basis->d->built) ? basis->d->reps.as<uint64_t const>() : nullptr;
}

int sed_basis_state_info(ls_spin_basis const* basis, uint64_t bits, uint64_t* representative,
                         unsigned* phase, unsigned* modulus) {
  if (!basis || !representative) return fail(LS_INVALID_ARGUMENT, "sed_basis_state_info: NULL argument");
  BasisData& b = *basis->d;
  if (b.n < 64 && (bits >> b.n)) return fail(LS_INVALID_STATE, "state has bits above number_spins");
  {
    std::lock_guard<std::mutex> lock(b.mu);
    if (int st = ensure_plan_checked(b)) return st;
  }
  PlanView const P = b.plan.view();
  uint64_t rep;
  uint32_t ph;
  if (b.plan.n_bits > 32) {
    auto c = canonicalize<uint64_t>(bits, P);
    rep = c.rep;
    ph = c.phase;
  } else {
    auto c = canonicalize<uint32_t>((uint32_t)bits, P);
    rep = c.rep;
    ph = c.phase;
  }
  *representative = rep;
  if (phase) *phase = ph;
  if (modulus) *modulus = b.plan.L;
  return LS_SUCCESS;
}

int sed_basis_index(ls_spin_basis const* basis, uint64_t representative, uint64_t* index) {
  if (!basis || !index) return fail(LS_INVALID_ARGUMENT, "sed_basis_index: NULL argument");
  BasisData& b = *basis->d;
  if (!b.built) return fail(LS_CACHE_NOT_BUILT, "basis has not been built (call ls_build)");
  // Host-side binary search over a copy of the bracketing prefix entries.
  ScopedDevice dev(b.device);
  uint64_t const key = representative >> b.prefix_shift;
  if (key >= ((uint64_t)1 << b.prefix_bits)) return LS_NOT_A_REPRESENTATIVE;
  uint64_t range[2];
  SED_TRY_CUDA(cudaMemcpy(range, b.prefix.as<uint64_t>() + key, 16, cudaMemcpyDeviceToHost));
  std::vector<uint64_t> slice(range[1] - range[0]);
  if (!slice.empty())
    SED_TRY_CUDA(cudaMemcpy(slice.data(), b.reps.as<uint64_t>() + range[0], slice.size() * 8,
                            cudaMemcpyDeviceToHost));
  auto it = std::lower_bound(slice.begin(), slice.end(), representative);
  if (it == slice.end() || *it != representative) return LS_NOT_A_REPRESENTATIVE;
  *index = range[0] + (uint64_t)(it - slice.begin());
  return LS_SUCCESS;
}

}  // extern "C"
