// binning.cu -- from per-record footprints to per-tile Gaussian lists.
//
//  scan      inclusive prefix sum of tiles_touched (reference: thrust::inclusive_scan,
//            cuda_rasterizer/rasterizer_impl.cu:244), total key count kept on the device
//  emit      one thread per key writes (global_tile << 32 | gaussian) in Gaussian-major,
//            row-then-column order (reference: getGaussianTileKeys, rasterizer_impl.cu:82-124)
//  sort      the project's own stable LSD radix sort on the tile bits only: emission order is
//            already ascending in Gaussian id, so a stable sort by tile yields (tile, Gaussian)
//            order, identical to the reference's full 64-bit thrust::sort of unique keys
//            (rasterizer_impl.cu:287)
//  ranges    [first, last+1) of every non-empty tile; empty tiles keep {0,0}
//            (reference: getPerTileRanges, rasterizer_impl.cu:127-152)
//  tile-major binning (the default where it applies): the keys written directly in sorted order
//            with their ranges, no scan, emission pass or sort
//
// Every kernel reads the key count from device memory and uses a fixed grid, so the sequence
// needs no host synchronisation and can be captured in a CUDA graph.
#include "fe_kernels.cuh"

namespace fe {

namespace {

constexpr int kScanThreads = 256;
constexpr int64_t kSmallScan = 65536;  // inputs up to this size use the single-CTA scan
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;

__device__ __forceinline__ int64_t chunk_of(int64_t n, int nblocks, int granule) {
  int64_t c = (n + nblocks - 1) / nblocks;
  return (c + granule - 1) / granule * granule;
}

// Block-wide exclusive scan of one value per thread (kScanThreads threads); returns the block total.
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T& excl, T* warp_sums) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    T s = lane < kScanThreads / 32 ? warp_sums[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < kScanThreads / 32) warp_sums[lane] = s;
  }
  __syncthreads();
  const T warp_prefix = warp ? warp_sums[warp - 1] : T(0);
  const T total = warp_sums[kScanThreads / 32 - 1];
  excl = warp_prefix + x - v;
  __syncthreads();
  return total;
}

__global__ void scan_reduce_kernel(const uint32_t* __restrict__ in, int64_t n,
                                   unsigned long long* __restrict__ bsum) {
  const int64_t chunk = chunk_of(n, gridDim.x, kScanThreads);
  const int64_t s = blockIdx.x * chunk, e = min(n, s + chunk);
  unsigned long long acc = 0;
  for (int64_t i = s + threadIdx.x; i < e; i += kScanThreads) acc += in[i];
  __shared__ unsigned long long red[kScanThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) t += red[w];
    bsum[blockIdx.x] = t;
  }
}

// One block: exclusive scan of the per-block sums; records the total key count.
__global__ void scan_spine_kernel(unsigned long long* __restrict__ bsum, int nb, int64_t capacity,
                                  Control* __restrict__ ctrl) {
  __shared__ unsigned long long ws[kScanThreads / 32];
  unsigned long long carry = 0;
  for (int base = 0; base < nb; base += kScanThreads) {
    const int i = base + threadIdx.x;
    const unsigned long long v = i < nb ? bsum[i] : 0ull;
    unsigned long long ex;
    const unsigned long long tot = block_exclusive_scan<unsigned long long>(v, ex, ws);
    if (i < nb) bsum[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) {
    ctrl->want_keys = carry;
    const unsigned long long cap = (unsigned long long)capacity;
    ctrl->num_keys = carry < cap ? carry : cap;
    if (carry > cap) atomicOr(&ctrl->error, FE_DEVERR_CAPACITY);
  }
}

__global__ void scan_down_kernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                 int64_t n, const unsigned long long* __restrict__ boff) {
  __shared__ unsigned long long ws[kScanThreads / 32];
  const int64_t chunk = chunk_of(n, gridDim.x, kScanThreads);
  const int64_t s = blockIdx.x * chunk, e = min(n, s + chunk);
  unsigned long long carry = boff[blockIdx.x];
  for (int64_t base = s; base < e; base += kScanThreads) {
    const int64_t i = base + threadIdx.x;
    const unsigned long long v = i < e ? in[i] : 0u;
    unsigned long long ex;
    const unsigned long long tot = block_exclusive_scan<unsigned long long>(v, ex, ws);
    if (i < e) {
      const unsigned long long incl = carry + ex + v;
      out[i] = incl > 0xffffffffull ? 0xffffffffu : (uint32_t)incl;
    }
    carry += tot;
  }
}

// One warp per record: the lanes write the record's keys, row by row, at its scan offset
// (coalesced), skipping anything beyond the device-side key count. Without `foot` every row spans
// the record's rectangle; with it each row spans the tiles its footprint reaches there
// (foot_row_tiles), and the lanes first take 32 rows at a time to form the rows' spans and their
// offsets.
__global__ void emit_keys_kernel(ViewsArg va, const uint32_t* __restrict__ incl,
                                 const TileRect* __restrict__ rects,
                                 const FootRows* __restrict__ foot, int tile_w, int tile_h,
                                 int64_t n, const Control* __restrict__ ctrl,
                                 uint64_t* __restrict__ keys) {
  const int64_t K = (int64_t)ctrl->num_keys;
  const int lane = threadIdx.x & 31;
  const unsigned full = 0xffffffffu;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const int64_t end = (int64_t)incl[i];
    const int64_t off = i ? (int64_t)incl[i - 1] : 0;
    if (end == off || off >= K) continue;
    const TileRect r = rects[i];
    const int vi = find_view<&ViewDev::rec_base>(va, i);
    const ViewDev& V = view_at(va, vi);
    const uint64_t gid = (uint64_t)(i - V.rec_base);
    if (!foot) {
      const int w = r.x1 - r.x0;
      const int64_t cnt = min(end, K) - off;
      for (int64_t j = lane; j < cnt; j += 32) {
        const int x = r.x0 + (int)(j % w), y = r.y0 + (int)(j / w);
        const uint64_t tile = (uint64_t)(V.tile_base + (int64_t)y * V.gx + x);
        keys[off + j] = (tile << 32) | gid;
      }
      continue;
    }
    const FootRows f = foot[i];
    int64_t o = off;
    for (int y0 = r.y0; y0 < r.y1 && o < K; y0 += 32) {
      const int y = y0 + lane;
      int x0 = 0, x1 = 0;
      if (y < r.y1) foot_row_tiles(f, r, y, tile_w, tile_h, x0, x1);
      const int w = x1 - x0;
      int incl_w = w;
#pragma unroll
      for (int s = 1; s < 32; s <<= 1) {
        const int t = __shfl_up_sync(full, incl_w, s);
        if (lane >= s) incl_w += t;
      }
      const int rows = min(32, r.y1 - y0);
      for (int l = 0; l < rows; ++l) {
        const int wl = __shfl_sync(full, w, l);
        const int xl = __shfl_sync(full, x0, l);
        const int64_t ol = o + __shfl_sync(full, incl_w - w, l);
        const uint64_t row_tile = (uint64_t)(V.tile_base + (int64_t)(y0 + l) * V.gx + xl);
        for (int j = lane; j < wl; j += 32)
          if (ol + j < K) keys[ol + j] = ((row_tile + (uint64_t)j) << 32) | gid;
      }
      o += __shfl_sync(full, incl_w, 31);
    }
  }
}

// Single-CTA inclusive scan for small inputs: 1024 threads x 16 consecutive values per pass
// (16-byte loads and stores when the arrays are aligned), all loads of a pass issued up front.
__global__ void __launch_bounds__(1024) scan_small_kernel(const uint32_t* __restrict__ in,
                                                          uint32_t* __restrict__ out, int64_t n,
                                                          int64_t capacity,
                                                          Control* __restrict__ ctrl) {
  constexpr int kPer = 16;
  __shared__ unsigned long long ws[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool vec = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
  unsigned long long carry = 0;
  for (int64_t base = 0; base < n; base += 1024 * kPer) {
    const int64_t i0 = base + (int64_t)kPer * threadIdx.x;
    const bool whole = vec && i0 + kPer <= n;
    uint32_t v[kPer];
    if (whole) {
#pragma unroll
      for (int q = 0; q < kPer / 4; ++q) {
        const uint4 w = reinterpret_cast<const uint4*>(in + i0)[q];
        v[4 * q] = w.x; v[4 * q + 1] = w.y; v[4 * q + 2] = w.z; v[4 * q + 3] = w.w;
      }
    } else {
#pragma unroll
      for (int q = 0; q < kPer; ++q) v[q] = i0 + q < n ? in[i0 + q] : 0u;
    }
    unsigned long long t = 0;
#pragma unroll
    for (int q = 0; q < kPer; ++q) t += v[q];
    unsigned long long x = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
      unsigned long long s2 = ws[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(0xffffffffu, s2, o);
        if (lane >= o) s2 += y;
      }
      ws[lane] = s2;
    }
    __syncthreads();
    unsigned long long run = carry + (warp ? ws[warp - 1] : 0ull) + x - t;
    const unsigned long long total = ws[31];
    uint32_t r[kPer];
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
      run += v[q];
      r[q] = run > 0xffffffffull ? 0xffffffffu : (uint32_t)run;
    }
    if (whole) {
#pragma unroll
      for (int q = 0; q < kPer / 4; ++q)
        reinterpret_cast<uint4*>(out + i0)[q] =
            make_uint4(r[4 * q], r[4 * q + 1], r[4 * q + 2], r[4 * q + 3]);
    } else {
#pragma unroll
      for (int q = 0; q < kPer; ++q)
        if (i0 + q < n) out[i0 + q] = r[q];
    }
    carry += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    ctrl->want_keys = carry;
    const unsigned long long cap = (unsigned long long)capacity;
    ctrl->num_keys = carry < cap ? carry : cap;
    if (carry > cap) atomicOr(&ctrl->error, FE_DEVERR_CAPACITY);
  }
}

// Number of sort blocks that receive keys: at least kSortKeysPerBlock keys per block, at most the
// grid.
constexpr int kSortKeysPerBlock = 2048;
__device__ __forceinline__ int sort_blocks_used(int64_t K, int grid) {
  const int64_t b = (K + kSortKeysPerBlock - 1) / kSortKeysPerBlock;
  return (int)(b < 1 ? 1 : (b > grid ? grid : b));
}

// Per-block digit histograms, digit-major: hist[digit * grid + b] (grid = the launch grid), so
// that each digit's counts are contiguous for the scan.
__global__ void sort_hist_kernel(const uint64_t* __restrict__ keys, const Control* __restrict__ ctrl,
                                 int shift, uint32_t* __restrict__ hist) {
  __shared__ uint32_t cnt[256];
  const int64_t K = (int64_t)ctrl->num_keys;
  const int nb = sort_blocks_used(K, gridDim.x);
  if ((int)blockIdx.x >= nb) return;
  const int64_t chunk = chunk_of(K, nb, kSortThreads);
  const int64_t s = blockIdx.x * chunk, e = min(K, s + chunk);
  cnt[threadIdx.x] = 0;
  __syncthreads();
#pragma unroll 4
  for (int64_t i = s + threadIdx.x; i < e; i += kSortThreads)
    atomicAdd(&cnt[(uint32_t)(keys[i] >> shift) & 255u], 1u);
  __syncthreads();
  hist[threadIdx.x * gridDim.x + blockIdx.x] = cnt[threadIdx.x];
}

// One block per digit: exclusive scan of that digit's per-block counts (in block order, one
// contiguous row of hist), written back in place; the digit total goes to hist[256 * grid + d].
// Each thread owns a contiguous run of blocks so the scan keeps block order.
__global__ void sort_scan_kernel(uint32_t* __restrict__ hist, const Control* __restrict__ ctrl,
                                 int grid) {
  __shared__ uint32_t ws[kScanThreads / 32];
  const int nb = sort_blocks_used((int64_t)ctrl->num_keys, grid);
  const int d = blockIdx.x;
  uint32_t* row = hist + (int64_t)d * grid;
  const int per = (nb + kScanThreads - 1) / kScanThreads;
  const int b0 = threadIdx.x * per, b1 = min(nb, b0 + per);
  uint32_t run = 0;
  for (int b = b0; b < b1; ++b) run += row[b];
  uint32_t ex;
  const uint32_t total = block_exclusive_scan<uint32_t>(run, ex, ws);
  for (int b = b0; b < b1; ++b) {
    const uint32_t c = row[b];
    row[b] = ex;
    ex += c;
  }
  if (threadIdx.x == 0) hist[grid * 256 + d] = total;
}

// Stable scatter: keys are taken in order 256 at a time; ranks within a 256-key slice come from
// warp match-any groups plus per-warp digit counts scanned across warps in warp order. Digit
// bases: the scanned digit totals plus this block's row entries of the digit-major hist.
__global__ void sort_scatter_kernel(const uint64_t* __restrict__ in, uint64_t* __restrict__ out,
                                    const Control* __restrict__ ctrl, int shift,
                                    const uint32_t* __restrict__ hist) {
  __shared__ uint32_t off[256];
  __shared__ uint32_t tot[256];
  __shared__ uint32_t wc[kSortWarps][256];
  __shared__ uint32_t ws[kScanThreads / 32];
  const int64_t K = (int64_t)ctrl->num_keys;
  const int nb = sort_blocks_used(K, gridDim.x);
  if ((int)blockIdx.x >= nb) return;
  const int64_t chunk = chunk_of(K, nb, kSortThreads);
  const int64_t s = blockIdx.x * chunk, e = min(K, s + chunk);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  {
    // Digit bases: exclusive scan of the 256 digit totals.
    uint32_t base;
    block_exclusive_scan<uint32_t>(hist[gridDim.x * 256 + tid], base, ws);
    off[tid] = base + hist[tid * gridDim.x + blockIdx.x];
  }
  const uint32_t lt_mask = (1u << lane) - 1u;
  // The next slice's key is loaded one iteration ahead, so the ranking below does not wait on it.
  uint64_t next = (s + tid < e) ? in[s + tid] : 0ull;
  for (int64_t base = s; base < e; base += kSortThreads) {
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) wc[w][tid] = 0;
    const int64_t i = base + tid;
    const bool valid = i < e;
    const uint64_t key = next;
    next = (i + kSortThreads < e) ? in[i + kSortThreads] : 0ull;
    const uint32_t d = valid ? ((uint32_t)(key >> shift) & 255u) : 256u;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t rank = __popc(peers & lt_mask);
    __syncthreads();
    if (valid && rank == 0) wc[warp][d] = __popc(peers);
    __syncthreads();
    {
      uint32_t run = 0;
#pragma unroll
      for (int w = 0; w < kSortWarps; ++w) {
        const uint32_t c = wc[w][tid];
        wc[w][tid] = run;
        run += c;
      }
      tot[tid] = run;
    }
    __syncthreads();
    if (valid) out[off[d] + wc[warp][d] + rank] = key;
    __syncthreads();
    off[tid] += tot[tid];
  }
}

// Tile ranges of a sorted key list, one key per thread: a key whose tile differs from its
// predecessor's starts its tile's range, one whose tile differs from its successor's ends it.
// Empty tiles keep their zeroed range.
constexpr int kRangeThreads = 256;

__global__ void __launch_bounds__(kRangeThreads) ranges_kernel(const uint64_t* __restrict__ keys,
                                                               const Control* __restrict__ ctrl,
                                                               uint2* __restrict__ ranges) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int64_t K = (int64_t)ctrl->num_keys;
  for (int64_t base = (int64_t)blockIdx.x * kRangeThreads; base < K;
       base += (int64_t)gridDim.x * kRangeThreads) {
    const int64_t k = base + threadIdx.x;
    const bool valid = k < K;
    const uint32_t tile = valid ? (uint32_t)(keys[k] >> 32) : 0u;
    uint32_t prev = __shfl_up_sync(full, tile, 1);
    uint32_t next = __shfl_down_sync(full, tile, 1);
    if (valid) {
      if (lane == 0 && k > 0) prev = (uint32_t)(keys[k - 1] >> 32);
      if (lane == 31 && k + 1 < K) next = (uint32_t)(keys[k + 1] >> 32);
      if (k == 0 || prev != tile) ranges[tile].x = (uint32_t)k;
      if (k == K - 1 || next != tile) ranges[tile].y = (uint32_t)(k + 1);
    }
  }
}

// ---- Tile-major binning ---------------------------------------------------------------------
// The keys of a tile are its Gaussians in ascending id: the order the stable sort of the
// Gaussian-major key list produces. The preprocess has added every record's keys in each tile row
// to that row's key count (row_tot, per view) and the total to ctrl->want_keys. One block per
// (view, tile row) then takes the row's base (the keys of the rows before it), per-tile counts
// from a difference array over the covering spans (each record's tiles in the row: its
// rectangle's, or with `foot` the ones its footprint reaches there), writes the tile ranges, and
// places the keys: the covering spans in id order (order-preserving compaction into shared
// memory) are walked 32 at a time by a warp per tile, a ballot giving each span its slot.
constexpr int kRowThreads = kScanThreads;  // block_exclusive_scan works on kScanThreads threads
constexpr int kRowWarps = kRowThreads / 32;
constexpr int kRowPer = 4;                          // rectangles per thread per filter segment
constexpr int kRowSeg = kRowThreads * kRowPer;      // rectangles filtered per segment
constexpr int kTilesPer = kMaxRowTiles / kRowThreads;  // tiles per thread in the row scans
constexpr int kTileBlock = 8;  // tiles a warp emits at once

struct RowRect {
  uint16_t x0, x1;
  uint32_t gid;
};

__device__ __forceinline__ bool covers_row(const TileRect& r, int row) {
  return r.y0 <= row && row < r.y1 && r.x0 < r.x1;
}

// Sum over the block (kRowThreads threads); every thread gets the result.
__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long v,
                                                            unsigned long long* ws) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) ws[warp] = v;
  __syncthreads();
  unsigned long long t = 0;
#pragma unroll
  for (int w = 0; w < kRowWarps; ++w) t += ws[w];
  return t;
}

// Order-preserving compaction of the segment's records that reach `row` into `list` with their
// span of tiles in the row (thread t takes records s0 + kRowPer t .. + kRowPer - 1); returns their
// number. Without `foot` a record's span is its rectangle's; with it, the tiles its footprint
// reaches in the row (records whose footprint misses the row are left out). Ends with a barrier
// after the list is written.
__device__ __forceinline__ uint32_t filter_row(const TileRect* __restrict__ vr,
                                               const FootRows* __restrict__ vf, int tile_w,
                                               int tile_h, int n, int s0, int row, RowRect* list,
                                               uint32_t* ws) {
  const int tid = threadIdx.x;
  uint16_t x0[kRowPer], x1[kRowPer];
  uint32_t hits = 0, c = 0;
#pragma unroll
  for (int q = 0; q < kRowPer; ++q) {
    const int i = s0 + kRowPer * tid + q;
    const TileRect r = i < n ? vr[i] : TileRect{0, 0, 0, 0};
    bool h = covers_row(r, row);
    x0[q] = r.x0;
    x1[q] = r.x1;
    if (h && vf) {
      int a, b;
      foot_row_tiles(vf[i], r, row, tile_w, tile_h, a, b);
      x0[q] = (uint16_t)a;
      x1[q] = (uint16_t)b;
      h = b > a;
    }
    hits |= (uint32_t)h << q;
    c += h;
  }
  uint32_t at;
  const uint32_t total = block_exclusive_scan<uint32_t>(c, at, ws);  // ends with a barrier
#pragma unroll
  for (int q = 0; q < kRowPer; ++q)
    if ((hits >> q) & 1u) list[at++] = RowRect{x0[q], x1[q], (uint32_t)(s0 + kRowPer * tid + q)};
  __syncthreads();
  return total;
}

// Row bases of many views, in two launches instead of a sum over all earlier views in every
// emission block (quadratic in the number of views). row_tot holds per view (stride max_gy + 1)
// the key counts of its rows; entry max_gy is free for the view's total.
// Pass 1, one warp per view: the exclusive prefix of the row counts within the view, in place;
// the view's key total into entry max_gy.
__global__ void __launch_bounds__(kRowThreads) row_offsets_kernel(ViewsArg va, int n_views,
                                                                   int max_gy,
                                                                   unsigned long long* row_tot) {
  const int lane = threadIdx.x & 31;
  const int v = (int)blockIdx.x * kRowWarps + (threadIdx.x >> 5);
  if (v >= n_views) return;  // (uniform over the warp)
  const unsigned full = 0xffffffffu;
  const int gy = view_at(va, v).gy;
  unsigned long long* d = row_tot + (int64_t)v * (max_gy + 1);
  unsigned long long off_carry = 0;   // keys of the rows before this chunk
  for (int r0 = 0; r0 < gy; r0 += 32) {
    const int r = r0 + lane;
    const unsigned long long k = r < gy ? d[r] : 0ull;
    unsigned long long incl = k;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(full, incl, o);
      if (lane >= o) incl += y;
    }
    if (r < gy) d[r] = off_carry + incl - k;
    off_carry += __shfl_sync(full, incl, 31);
  }
  if (lane == 0) d[max_gy] = off_carry;
}

// Pass 2, one block: exclusive prefix of the view totals over the views, into entry max_gy.
// Thread t takes the consecutive views [t vpt, t vpt + vpt).
__global__ void __launch_bounds__(kRowThreads) view_bases_kernel(int n_views, int max_gy,
                                                                  unsigned long long* row_tot) {
  __shared__ unsigned long long ws[kRowWarps];
  const int stride = max_gy + 1;
  const int vpt = (n_views + kRowThreads - 1) / kRowThreads;
  const int v0 = (int)threadIdx.x * vpt, v1 = min(n_views, v0 + vpt);
  unsigned long long mine = 0;
  for (int v = v0; v < v1; ++v) mine += row_tot[(int64_t)v * stride + max_gy];
  unsigned long long base;
  block_exclusive_scan<unsigned long long>(mine, base, ws);
  for (int v = v0; v < v1; ++v) {
    unsigned long long* t = row_tot + (int64_t)v * stride + max_gy;
    const unsigned long long tot = *t;
    *t = base;
    base += tot;
  }
}

__device__ __forceinline__ void tile_emit_body(
    ViewsArg va, const TileRect* __restrict__ rects, const FootRows* __restrict__ foot,
    int tile_w, int tile_h, const unsigned long long* __restrict__ row_tot, bool bases,
    int64_t capacity, Control* __restrict__ ctrl, uint2* __restrict__ ranges,
    uint32_t* __restrict__ tile_view,
    uint64_t* __restrict__ keys, uint32_t* __restrict__ order, int64_t n_tiles, int nseg) {
  __shared__ RowRect list[kRowSeg];
  __shared__ int diff[kMaxRowTiles + 1];         // +1 at x0, -1 at x1 of every covering rectangle
  __shared__ uint32_t pos[kMaxRowTiles];  // per tile: next key slot within the row
  __shared__ unsigned long long wsu[kRowWarps];
  __shared__ uint32_t ws[kRowWarps];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned full = 0xffffffffu;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const unsigned slot = blockIdx.y * gridDim.x + blockIdx.x;
  const unsigned long long want = ctrl->want_keys, cap = (unsigned long long)capacity;
  const unsigned long long K = want < cap ? want : cap;
  if (slot == 0 && tid == 0) {
    ctrl->num_keys = K;
    if (want > cap) atomicOr(&ctrl->error, FE_DEVERR_CAPACITY);
  }
  const ViewDev& V = view_at(va, blockIdx.y);
  // nseg blocks share a row: each forms the whole row's tile counts but writes the ranges, work
  // classes and keys of its own slice of the row's tiles [x_lo, x_hi) only.
  const int row = (int)blockIdx.x / nseg, seg = (int)blockIdx.x - row * nseg;
  if (row >= V.gy) return;  // (uniform over the block)
  if (V.gx > kMaxRowTiles) {  // the host plans this path only for narrower views
    if (tid == 0) atomicOr(&ctrl->error, FE_DEVERR_CAPACITY);
    return;
  }
  const int gx = V.gx, n = V.n;
  const int seg_w = (gx + nseg - 1) / nseg;
  const int x_lo = seg * seg_w, x_hi = min(gx, x_lo + seg_w);
  if (x_lo >= x_hi) return;  // (uniform over the block)
  const int64_t tile0 = V.tile_base + (int64_t)row * gx;
  const TileRect* vr = rects + V.rec_base;
  const FootRows* vf = foot ? foot + V.rec_base : nullptr;

  // row_tot holds, per view, the key counts of its rows (stride max_gy + 1). With `bases` set,
  // row_offsets_kernel and view_bases_kernel have already turned them into row offsets within
  // the view and view bases.
  const int stride = (int)gridDim.x / nseg + 1;
  unsigned long long row_base;
  if (bases) {  // view base (entry max_gy) + the row's offset within the view
    row_base = row_tot[(int64_t)blockIdx.y * stride + stride - 1] +
               row_tot[(int64_t)blockIdx.y * stride + row];
  } else {
    long long b = 0;
    for (int idx = tid; idx < (int)blockIdx.y * stride; idx += kRowThreads) {
      const int v2 = idx / stride, r2 = idx - v2 * stride;
      if (r2 < view_at(va, v2).gy) b += (long long)row_tot[idx];
    }
    for (int r2 = tid; r2 < row; r2 += kRowThreads)
      b += (long long)row_tot[(int64_t)blockIdx.y * stride + r2];
    row_base = block_sum_u64((unsigned long long)b, wsu);
  }
  // Keys of this row: slot p (relative to the row's base) for p < lim.
  uint64_t* row_keys = keys + row_base;
  const unsigned long long left = K > row_base ? K - row_base : 0ull;
  const uint32_t lim = left < 0xffffffffull ? (uint32_t)left : 0xffffffffu;
  for (int x = tid; x <= gx; x += kRowThreads) diff[x] = 0;
  __syncthreads();
  uint32_t total = 0;
  for (int s0 = 0; s0 < n; s0 += kRowSeg) {
    total = filter_row(vr, vf, tile_w, tile_h, n, s0, row, list, ws);
    for (uint32_t j = tid; j < total; j += kRowThreads) {
      atomicAdd(&diff[list[j].x0], 1);
      atomicAdd(&diff[list[j].x1], -1);
    }
    __syncthreads();
  }
  // Tile counts (prefix of the difference array) and their exclusive prefix, kTilesPer
  // consecutive tiles per thread.
  int cnt[kTilesPer];
  uint32_t dsum = 0;
#pragma unroll
  for (int q = 0; q < kTilesPer; ++q) {
    const int x = kTilesPer * tid + q;
    cnt[q] = x < gx ? diff[x] : 0;
    dsum += (uint32_t)cnt[q];
  }
  uint32_t dex;
  block_exclusive_scan<uint32_t>(dsum, dex, ws);
  unsigned long long csum = 0;
  {
    int run = (int)dex;
#pragma unroll
    for (int q = 0; q < kTilesPer; ++q) {
      run += cnt[q];
      cnt[q] = run;
      csum += (unsigned)run;
    }
  }
  unsigned long long cex;
  {
    // Exclusive scan of the per-thread count sums (64-bit: a row can hold more than 2^32 keys).
    unsigned long long x = csum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(full, x, o);
      if (lane >= o) x += y;
    }
    __syncthreads();
    if (lane == 31) wsu[warp] = x;
    __syncthreads();
    unsigned long long before = 0;
    for (int w = 0; w < warp; ++w) before += wsu[w];
    cex = before + x - csum;
  }
  uint2 rgq[kTilesPer];
#pragma unroll
  for (int q = 0; q < kTilesPer; ++q) {
    const int x = kTilesPer * tid + q;
    rgq[q] = make_uint2(0u, 0u);
    if (x >= x_lo && x < x_hi) {
      pos[x] = cex < lim ? (uint32_t)cex : lim;  // (slots from lim on are dropped)
      const unsigned long long lo = min(row_base + cex, K);
      const unsigned long long hi = min(row_base + cex + (unsigned)cnt[q], K);
      // every tile of the slice: empty tiles (or tiles whose keys were all dropped) get {0,0}
      rgq[q] = hi > lo ? make_uint2((uint32_t)lo, (uint32_t)hi) : make_uint2(0u, 0u);
      ranges[tile0 + x] = rgq[q];
      if (tile_view) tile_view[tile0 + x] = blockIdx.y;
    }
    cex += (unsigned)cnt[q];
  }
  if (order) {
    // Work classes: every tile of the row joins its class's list (order + c n_tiles), a shared
    // count per class and one global atomic per class and row giving the slots.
    __shared__ uint32_t cls_n[kTileClasses], cls_base[kTileClasses];
    if (tid < kTileClasses) cls_n[tid] = 0u;
    __syncthreads();
    int cl[kTilesPer];
    uint32_t rank[kTilesPer];
#pragma unroll
    for (int q = 0; q < kTilesPer; ++q) {
      const int x = kTilesPer * tid + q;
      cl[q] = tile_class((uint32_t)cnt[q]);
      rank[q] = (x >= x_lo && x < x_hi) ? atomicAdd(&cls_n[cl[q]], 1u) : 0u;
    }
    __syncthreads();
    if (tid < kTileClasses && cls_n[tid] != 0u)
      cls_base[tid] = atomicAdd(&ctrl->tile_class[tid], cls_n[tid]);
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kTilesPer; ++q) {
      const int x = kTilesPer * tid + q;
      if (x >= x_lo && x < x_hi)
        reinterpret_cast<uint4*>(order)[(int64_t)cl[q] * n_tiles + cls_base[cl[q]] + rank[q]] =
            make_uint4((uint32_t)(tile0 + x), rgq[q].x, rgq[q].y, blockIdx.y);
    }
  }
  __syncthreads();
  for (int s0 = 0; s0 < n; s0 += kRowSeg) {
    // (with a single segment the list is still in shared memory)
    if (n > kRowSeg) total = filter_row(vr, vf, tile_w, tile_h, n, s0, row, list, ws);
    // Each warp takes kTileBlock of its tiles at a time (tiles warp + kRowWarps t of the slice),
    // keeping their next slots in registers, and reads each 32-entry chunk of the list once for
    // all of them.
    for (int xb = x_lo + warp; xb < x_hi; xb += kRowWarps * kTileBlock) {
      // the warp's tiles in this pass: xb + kRowWarps t for t < nt (uniform over the warp)
      const int nt = min(kTileBlock, (x_hi - xb + kRowWarps - 1) / kRowWarps);
      uint32_t p[kTileBlock];
#pragma unroll
      for (int t = 0; t < kTileBlock; ++t) {
        const int x = xb + kRowWarps * t;
        p[t] = x < x_hi ? (uint32_t)pos[x] : 0u;
      }
      for (uint32_t j0 = 0; j0 < total; j0 += 32) {
        const uint32_t j = j0 + lane;
        RowRect e{0, 0, 0};
        if (j < total) e = list[j];
#pragma unroll
        for (int t = 0; t < kTileBlock; ++t) {
          if (t >= nt) break;
          const int x = xb + kRowWarps * t;
          const bool cov = e.x0 <= x && x < e.x1;
          const uint32_t bal = __ballot_sync(full, cov);
          if (cov) {
            const uint32_t k = p[t] + __popc(bal & lt_mask);
            if (k < lim) row_keys[k] = ((uint64_t)(tile0 + x) << 32) | e.gid;
          }
          p[t] += __popc(bal);
        }
      }
      if (lane == 0) {
#pragma unroll
        for (int t = 0; t < kTileBlock; ++t) {
          const int x = xb + kRowWarps * t;
          if (x < x_hi) pos[x] = p[t];
        }
      }
    }
    __syncthreads();  // the list is rewritten by the next segment
  }
}

// The emission kernel at the registers its single-wave launches run fastest with (48), and a copy
// sized for 8 resident blocks per SM (32 registers, a few spills) for launches of many waves.
__global__ void __launch_bounds__(kRowThreads) tile_emit_kernel(
    ViewsArg va, const TileRect* __restrict__ rects, const FootRows* __restrict__ foot,
    int tile_w, int tile_h, const unsigned long long* __restrict__ row_tot, bool bases,
    int64_t capacity, Control* __restrict__ ctrl, uint2* __restrict__ ranges,
    uint32_t* __restrict__ tile_view,
    uint64_t* __restrict__ keys, uint32_t* __restrict__ order, int64_t n_tiles, int nseg) {
  tile_emit_body(va, rects, foot, tile_w, tile_h, row_tot, bases, capacity, ctrl, ranges,
                 tile_view, keys, order, n_tiles, nseg);
}
__global__ void __launch_bounds__(kRowThreads, 8) tile_emit_kernel_waves(
    ViewsArg va, const TileRect* __restrict__ rects, const FootRows* __restrict__ foot,
    int tile_w, int tile_h, const unsigned long long* __restrict__ row_tot, bool bases,
    int64_t capacity, Control* __restrict__ ctrl, uint2* __restrict__ ranges,
    uint32_t* __restrict__ tile_view,
    uint64_t* __restrict__ keys, uint32_t* __restrict__ order, int64_t n_tiles, int nseg) {
  tile_emit_body(va, rects, foot, tile_w, tile_h, row_tot, bases, capacity, ctrl, ranges,
                 tile_view, keys, order, n_tiles, nseg);
}

// Tile-major emission for batches of narrow views (at most 32 tiles per row) once the row bases
// are formed: one warp per (view, tile row), lane x owning tile x of the row, no block barriers.
// Same outputs as tile_emit_body: each tile's keys in Gaussian-id order from the row's base,
// every tile's range and view, and the work-class list entries. Lanes take the view's records
// 32 at a time; a ballot per tile gives the chunk's records covering it and each one's rank.
constexpr int kWarpRowWarps = 8;
constexpr int kWarpRowTiles = 32;
constexpr int kWarpRowCache = 512;  // records whose span masks the key pass reuses

// Bit x set when record i of the view reaches tile x of `row` (its footprint's span in the row,
// or its rectangle's without footprint rows).
__device__ __forceinline__ uint32_t row_span_mask(const TileRect* __restrict__ vr,
                                                  const FootRows* __restrict__ vf, int tile_w,
                                                  int tile_h, int n, int i, int row) {
  if (i >= n) return 0u;
  const TileRect r = vr[i];
  if (!covers_row(r, row)) return 0u;
  int a = r.x0, b = r.x1;
  if (vf) foot_row_tiles(vf[i], r, row, tile_w, tile_h, a, b);
  if (b <= a) return 0u;
  const uint32_t below_b = b >= 32 ? 0xffffffffu : ((1u << b) - 1u);
  return below_b & ~((1u << a) - 1u);
}

__global__ void __launch_bounds__(kWarpRowWarps * 32) tile_emit_warp_kernel(
    ViewsArg va, const TileRect* __restrict__ rects, const FootRows* __restrict__ foot,
    int tile_w, int tile_h, const unsigned long long* __restrict__ row_tot, int stride,
    int64_t capacity, Control* __restrict__ ctrl, uint2* __restrict__ ranges,
    uint32_t* __restrict__ tile_view, uint64_t* __restrict__ keys, uint32_t* __restrict__ order,
    int64_t n_tiles) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned full = 0xffffffffu;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const unsigned long long want = ctrl->want_keys, cap = (unsigned long long)capacity;
  const unsigned long long K = want < cap ? want : cap;
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
    ctrl->num_keys = K;
    if (want > cap) atomicOr(&ctrl->error, FE_DEVERR_CAPACITY);
  }
  const int v = (int)blockIdx.y;
  const ViewDev& V = view_at(va, v);
  const int row = (int)blockIdx.x * kWarpRowWarps + warp;
  if (row >= V.gy) return;  // (uniform over the warp)
  const int gx = V.gx, n = V.n;
  if (gx > kWarpRowTiles) {  // the host plans this kernel only for narrower views
    if (lane == 0) atomicOr(&ctrl->error, FE_DEVERR_CAPACITY);
    return;
  }
  const int64_t tile0 = V.tile_base + (int64_t)row * gx;
  const TileRect* vr = rects + V.rec_base;
  const FootRows* vf = foot ? foot + V.rec_base : nullptr;
  // View base (entry stride - 1) + the row's offset within the view.
  const unsigned long long row_base =
      row_tot[(int64_t)v * stride + stride - 1] + row_tot[(int64_t)v * stride + row];
  uint64_t* row_keys = keys + row_base;
  const unsigned long long left = K > row_base ? K - row_base : 0ull;
  const uint32_t lim = left < 0xffffffffull ? (uint32_t)left : 0xffffffffu;

  // Keys of each tile (lane x: tile x), then their exclusive prefix along the row. The span
  // masks of the first kWarpRowCache records are kept for the key pass; only tiles that some
  // record of a chunk reaches are visited.
  __shared__ uint32_t s_mask[kWarpRowWarps][kWarpRowCache];
  uint32_t cnt = 0;
  for (int s0 = 0; s0 < n; s0 += 32) {
    const uint32_t m = row_span_mask(vr, vf, tile_w, tile_h, n, s0 + lane, row);
    if (s0 < kWarpRowCache) s_mask[warp][s0 + lane] = m;
    for (uint32_t u = __reduce_or_sync(full, m); u; u &= u - 1u) {
      const int x = __ffs(u) - 1;
      const uint32_t c = (uint32_t)__popc(__ballot_sync(full, (m >> x) & 1u));
      if (lane == x) cnt += c;
    }
  }
  uint32_t incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(full, incl, o);
    if (lane >= o) incl += y;
  }
  const uint32_t ex = incl - cnt;
  uint2 rg = make_uint2(0u, 0u);
  if (lane < gx) {
    const unsigned long long lo = min(row_base + ex, K), hi = min(row_base + ex + cnt, K);
    // every tile of the row: empty tiles (or tiles whose keys were all dropped) get {0,0}
    rg = hi > lo ? make_uint2((uint32_t)lo, (uint32_t)hi) : make_uint2(0u, 0u);
    ranges[tile0 + lane] = rg;
    if (tile_view) tile_view[tile0 + lane] = (uint32_t)v;
  }
  if (order) {
    // Work classes: the lanes of one class share one global atomic for their slots.
    const int cl = lane < gx ? tile_class(cnt) : -1;
    const unsigned same = __match_any_sync(full, cl);
    const int leader = __ffs(same) - 1;
    uint32_t base = 0;
    if (lane < gx && lane == leader)
      base = atomicAdd(&ctrl->tile_class[cl], (uint32_t)__popc(same));
    base = __shfl_sync(full, base, leader);
    if (lane < gx) {
      const uint32_t rank = (uint32_t)__popc(same & lt_mask);
      reinterpret_cast<uint4*>(order)[(int64_t)cl * n_tiles + base + rank] =
          make_uint4((uint32_t)(tile0 + lane), rg.x, rg.y, (uint32_t)v);
    }
  }
  // Keys: tile x's next slot is lane x's p; a record's rank among the chunk's records covering x
  // is the ballot's bits below its lane.
  uint32_t p = ex;
  for (int s0 = 0; s0 < n; s0 += 32) {
    const int i = s0 + lane;
    const uint32_t m = s0 < kWarpRowCache ? s_mask[warp][i]
                                          : row_span_mask(vr, vf, tile_w, tile_h, n, i, row);
    for (uint32_t u = __reduce_or_sync(full, m); u; u &= u - 1u) {
      const int x = __ffs(u) - 1;
      const uint32_t bal = __ballot_sync(full, (m >> x) & 1u);
      const uint32_t px = __shfl_sync(full, p, x);
      if ((m >> x) & 1u) {
        const uint32_t k = px + (uint32_t)__popc(bal & lt_mask);
        if (k < lim) row_keys[k] = ((uint64_t)(tile0 + x) << 32) | (uint32_t)i;
      }
      if (lane == x) p += (uint32_t)__popc(bal);
    }
  }
}

inline int grid_for(int64_t work, int threads, int cap) {
  const int64_t b = (work + threads - 1) / threads;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

int scan_grid(int64_t n) { return grid_for(n, 4 * kScanThreads, 1024); }
int sort_grid(int64_t key_capacity) { return grid_for(key_capacity, kSortKeysPerBlock, 2 * 152); }

void launch_scan(const uint32_t* touched, uint32_t* incl, int64_t n, int64_t capacity,
                 unsigned long long* scratch, Control* ctrl, cudaStream_t st) {
  if (n <= kSmallScan) {
    scan_small_kernel<<<1, 1024, 0, st>>>(touched, incl, n, capacity, ctrl);
    return;
  }
  const int nb = scan_grid(n);
  scan_reduce_kernel<<<nb, kScanThreads, 0, st>>>(touched, n, scratch);
  scan_spine_kernel<<<1, kScanThreads, 0, st>>>(scratch, nb, capacity, ctrl);
  scan_down_kernel<<<nb, kScanThreads, 0, st>>>(touched, incl, n, scratch);
}

void launch_emit_keys(const ViewsArg& va, const uint32_t* incl, const TileRect* rects,
                      const FootRows* foot, int tile_w, int tile_h, int64_t n,
                      const Control* ctrl, uint64_t* keys, int64_t capacity, cudaStream_t st) {
  (void)capacity;
  emit_keys_kernel<<<grid_for(n * 32, 256, 152 * 16), 256, 0, st>>>(va, incl, rects, foot, tile_w,
                                                                    tile_h, n, ctrl, keys);
}

uint64_t* launch_sort(uint64_t* a, uint64_t* b, int key_bits, const Control* ctrl,
                      int64_t capacity, uint32_t* hist, cudaStream_t st) {
  const int nb = sort_grid(capacity);
  uint64_t* src = a;
  uint64_t* dst = b;
  for (int lo = 0; lo < key_bits; lo += 8) {
    const int shift = 32 + lo;
    sort_hist_kernel<<<nb, kSortThreads, 0, st>>>(src, ctrl, shift, hist);
    sort_scan_kernel<<<256, kScanThreads, 0, st>>>(hist, ctrl, nb);
    sort_scatter_kernel<<<nb, kSortThreads, 0, st>>>(src, dst, ctrl, shift, hist);
    uint64_t* t = src;
    src = dst;
    dst = t;
  }
  return src;
}


void launch_tile_binning_emit(const ViewsArg& va, int n_views, int max_gy, int max_gx,
                              const TileRect* rects, const FootRows* foot, int tile_w, int tile_h,
                              unsigned long long* row_tot, int64_t capacity, Control* ctrl,
                              uint2* ranges, uint32_t* tile_view, uint64_t* keys, uint32_t* order,
                              int64_t n_tiles, cudaStream_t st) {
  if (n_views <= 0 || max_gy <= 0) return;
  // Beyond a few dozen views the per-block sums over earlier views cost more than two extra
  // launches that form all row bases.
  const bool bases = n_views > kRowBaseViews;
  if (bases) {
    row_offsets_kernel<<<(unsigned)((n_views + kRowWarps - 1) / kRowWarps), kRowThreads, 0, st>>>(
        va, n_views, max_gy, row_tot);
    view_bases_kernel<<<1, kRowThreads, 0, st>>>(n_views, max_gy, row_tot);
    if (max_gx <= kWarpRowTiles) {
      // Narrow views: a warp per tile row instead of a block sized for 1024-tile rows.
      const dim3 grid((unsigned)((max_gy + kWarpRowWarps - 1) / kWarpRowWarps), (unsigned)n_views);
      tile_emit_warp_kernel<<<grid, kWarpRowWarps * 32, 0, st>>>(
          va, rects, foot, tile_w, tile_h, row_tot, max_gy + 1, capacity, ctrl, ranges, tile_view,
          keys, order, n_tiles);
      return;
    }
  }
  // Launches of few rows (single views) split each row over up to 8 blocks so that the key
  // writing, the longest part of a row's work, is spread over more SMs.
  const int64_t rows = (int64_t)max_gy * n_views;
  const int nseg = rows >= 2 * 152 ? 1 : (int)std::min<int64_t>(8, (2 * 152 + rows - 1) / rows);
  const dim3 grid((unsigned)(max_gy * nseg), (unsigned)n_views);
  // Many row blocks (several waves: the 1135-view batch has 18 K) go faster with more of them
  // resident at a time, at 32 registers and a few spills (110 -> 100 us there); a single wave
  // (16 views of 640x480: 480 blocks) goes faster with the 48 registers it needs (22.5 us
  // against 26.5).
  if ((int64_t)grid.x * grid.y > 2 * 5 * 152)
    tile_emit_kernel_waves<<<grid, kRowThreads, 0, st>>>(va, rects, foot, tile_w, tile_h, row_tot,
                                                         bases, capacity, ctrl, ranges, tile_view,
                                                         keys, order, n_tiles, nseg);
  else
    tile_emit_kernel<<<grid, kRowThreads, 0, st>>>(va, rects, foot, tile_w, tile_h, row_tot, bases,
                                                   capacity, ctrl, ranges, tile_view, keys, order,
                                                   n_tiles, nseg);
}

void launch_ranges(const uint64_t* keys, const Control* ctrl, int64_t capacity, uint2* ranges,
                   cudaStream_t st) {
  ranges_kernel<<<grid_for(capacity, kRangeThreads, 152 * 8), kRangeThreads, 0, st>>>(keys, ctrl,
                                                                                   ranges);
}

}  // namespace fe
