// Forward composite, sm_103a: tile ranges, bucket bookkeeping, bucket-parallel
// alpha compositing and the associative (colour, transmittance) merge.
//
// Restates FB csrc/cuda_rasterizer/render.cu: a tile's depth-sorted list is
// cut into fixed-size buckets, every bucket is composited independently from
// T = 1, C = 0, and a per-pixel merge folds the buckets front to back with
// C += T * C_b, T *= T_b, stopping after the bucket that drops T below 1e-4.
// GB300 changes:
//   * bucket bookkeeping never leaves the device (FB copies the bucket total
//     to the host mid-frame); the composite kernel is persistent and reads the
//     total from device memory;
//   * the merge is fused into the composite as a per-tile chain: a warp that
//     finishes bucket k of a tile folds it into the tile's running prefix as
//     soon as bucket k-1 has been folded (the same operations, in the same
//     order, as FB's merge), and publishes which pixels are still above the
//     1e-4 cut-off.  Buckets are handed out round by round (every tile's
//     bucket 0, then every tile's bucket 1, ...), so when a warp starts a
//     bucket the tile's earlier buckets are usually folded already, and the
//     8x4 sub-blocks whose pixels have all stopped are skipped: FB composites
//     them and the merge discards them;
//   * a bucket's records are staged once into shared memory (coalesced
//     per-lane loads, structure-of-arrays) and broadcast from there;
//   * each lane owns a column strip of 8 pixels, so a Gaussian's row terms are
//     shared and every sample store is a contiguous 512-byte warp store;
//   * the sample state is 16 bytes per pixel and bucket and holds the prefix
//     after the bucket (FB keeps 40).
#include <algorithm>

#include "render_common.cuh"

namespace fgs {
namespace {

constexpr int kFwdWarps = 4;
// Blocks per SM of the composite kernel: 6 (80 registers, 16 B of spills)
// for frames of up to kFwdFewTiles tiles, 7 (72 registers, 72 B of spills) above.
// A 1297x840 frame (4346 tiles, ~12 buckets per warp): 0.178 -> 0.169 ms with
// 6; the 16-camera C4 frame (58k tiles, ~180 buckets per warp): 1.87 ms with
// 7, 1.93 with 6.
constexpr uint32_t kFwdFewTiles = 16384;

__global__ void __launch_bounds__(256) k_tile_ranges(const unsigned long long* __restrict__ keys, long long n_cap,
                                                     const int* n_dev, uint32_t num_tiles,
                                                     uint32_t* __restrict__ ranges) {
  pdl_wait();  // the preceding kernel of the stream is done
  pdl_trigger();
  // 4 consecutive keys per thread (two 16-byte loads when aligned), compared
  // with their predecessors: a tile boundary writes the end of one range and
  // the start of the next.
  constexpr int kPer = 4;
  const long long n = n_dev ? min(n_cap, (long long)(unsigned int)*n_dev) : n_cap;
  const long long i0 = (blockIdx.x * 256ll + threadIdx.x) * kPer;
  if (i0 >= n) return;
  unsigned long long k[kPer];
  if (i0 + kPer <= n && ((reinterpret_cast<uintptr_t>(keys) & 15) == 0)) {
    const ulonglong2 a = __ldg(reinterpret_cast<const ulonglong2*>(keys + i0));
    const ulonglong2 b = __ldg(reinterpret_cast<const ulonglong2*>(keys + i0) + 1);
    k[0] = a.x; k[1] = a.y; k[2] = b.x; k[3] = b.y;
  } else {
#pragma unroll
    for (int r = 0; r < kPer; ++r) k[r] = i0 + r < n ? keys[i0 + r] : 0ull;
  }
  uint32_t pt = i0 > 0 ? (uint32_t)(keys[i0 - 1] >> 32) : 0xffffffffu;
#pragma unroll
  for (int r = 0; r < kPer; ++r) {
    const long long i = i0 + r;
    if (i >= n) break;
    const uint32_t t = (uint32_t)(k[r] >> 32);
    if (t >= num_tiles) {  // not a key of this frame
      raise_error(kErrCapacity);
      return;
    }
    if (i == 0) {
      ranges[2 * t] = 0;
    } else if (pt != t && pt < num_tiles) {
      ranges[2 * pt + 1] = (uint32_t)i;
      ranges[2 * t] = (uint32_t)i;
    }
    if (i == n - 1) ranges[2 * t + 1] = (uint32_t)n;
    pt = t;
  }
}

// Bucket bookkeeping (FB render.cu:418-433 counts buckets per tile, scans them
// with CUB and copies the total to the host), plus the forward work queue.
// Per tile: nb = ceil(n / bs) buckets, their inclusive offsets and the
// bucket -> tile map.  Queue order: round k holds bucket k of every tile that
// has one (k < kRounds; in any order inside the round), then buckets
// k >= kRounds tile after tile.  A tile's bucket k therefore always comes
// after its bucket k-1, which is what the composite's per-tile chain waits
// on, and by the time a round starts the previous one is mostly folded.
//   k_bucket_count  per-block scans of [max(nb - kRounds, 0), nb], histogram
//                   of min(nb, kRounds);
//   k_round_offsets one block: round sizes (tiles with nb > k) and their
//                   exclusive offsets;
//   k_bucket_fill   offsets, bucket -> tile map, queue slots (one atomic per
//                   warp and round).
__device__ __forceinline__ uint32_t tile_buckets(const uint32_t* __restrict__ ranges, int t, int bs) {
  return (ranges[2 * t + 1] - ranges[2 * t] + (uint32_t)bs - 1) / (uint32_t)bs;
}

__device__ __forceinline__ void scan_values(uint32_t nb, uint32_t (&v)[kScanValues]) {
  v[0] = nb > (uint32_t)kRounds ? nb - kRounds : 0u;
  v[1] = nb;
}

// Inclusive block scan (kScanTiles threads) of every value; tot = block totals.
__device__ __forceinline__ void block_scan(uint32_t (&v)[kScanValues], uint32_t (&tot)[kScanValues],
                                           uint32_t (*s_warp)[kScanValues]) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int j = 0; j < kScanValues; ++j) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, v[j], o);
      if (lane >= o) v[j] += u;
    }
    if (lane == 31) s_warp[warp][j] = v[j];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int j = 0; j < kScanValues; ++j) {
      uint32_t w = s_warp[lane][j];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += u;
      }
      s_warp[lane][j] = w;  // inclusive over warps
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kScanValues; ++j) {
    v[j] += warp ? s_warp[warp - 1][j] : 0u;
    tot[j] = s_warp[kScanTiles / 32 - 1][j];
  }
}

__global__ void __launch_bounds__(kScanTiles) k_bucket_count(int T, const uint32_t* __restrict__ ranges, int bs,
                                                             uint32_t* __restrict__ block_sums,
                                                             uint32_t* __restrict__ round_hist,
                                                             uint32_t* __restrict__ bucket_sum) {
  pdl_wait();  // the preceding kernel of the stream is done
  pdl_trigger();
  __shared__ uint32_t s_warp[kScanTiles / 32][kScanValues];
  const int t = blockIdx.x * kScanTiles + threadIdx.x;
  const uint32_t nb = t < T ? tile_buckets(ranges, t, bs) : 0u;
  if (t == 0) bucket_sum[4] = 0;  // buckets of the stop granularity, summed by k_bucket_fill
  if (t < T) {  // one atomic per distinct count in the warp
    const uint32_t bin = min(nb, (uint32_t)kRounds);
    const uint32_t peers = __match_any_sync(__activemask(), bin);
    if ((peers & lanemask_lt()) == 0) atomicAdd(round_hist + bin, (uint32_t)__popc(peers));
  }
  uint32_t v[kScanValues], tot[kScanValues];
  scan_values(nb, v);
  block_scan(v, tot, s_warp);
  if (threadIdx.x < kScanValues) {
#pragma unroll
    for (int j = 0; j < kScanValues; ++j)
      if ((int)threadIdx.x == j) block_sums[(size_t)blockIdx.x * kScanValues + j] = tot[j];
  }
}

// One block: round k has cnt[k] = #tiles with nb > k = sum_{n > k} hist[n]
// slots; round_off[k] = sum_{j < k} cnt[j], round_off[kRounds] = first tail slot.
__global__ void __launch_bounds__(1024) k_round_offsets(const uint32_t* __restrict__ round_hist,
                                                        uint32_t* __restrict__ round_off,
                                                        uint32_t* __restrict__ round_fill) {
  pdl_wait();  // the preceding kernel of the stream is done
  pdl_trigger();
  constexpr int kPer = kRounds / 1024;
  __shared__ uint32_t s_warp[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // suffix sums of hist over n > k: thread tid owns k in [tid*kPer, tid*kPer + kPer), scanned from the top
  uint32_t h[kPer];
  uint32_t local = 0;
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    h[j] = round_hist[tid * kPer + j + 1];  // hist[k + 1]
    local += h[j];
  }
  // exclusive suffix over threads: sum of `local` of threads > tid
  uint32_t incl = local;  // inclusive prefix over threads in reverse order
  const int rlane = 31 - lane;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_down_sync(0xffffffffu, incl, o);
    if (rlane >= o) incl += u;
  }
  if (lane == 0) s_warp[warp] = incl;
  __syncthreads();
  uint32_t above = 0;
  for (int w = warp + 1; w < 32; ++w) above += s_warp[w];
  const uint32_t suffix = above + incl - local;  // hist entries owned by threads above this one
  // cnt[k] = hist[k+1] + hist[k+2] + ... ; walk this thread's range downwards
  uint32_t cnt[kPer];
  uint32_t run = suffix;
#pragma unroll
  for (int j = kPer - 1; j >= 0; --j) {
    run += h[j];
    cnt[j] = run;
  }
  __syncthreads();
  // exclusive prefix of cnt over k
  uint32_t csum = 0;
#pragma unroll
  for (int j = 0; j < kPer; ++j) csum += cnt[j];
  uint32_t pre = csum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, pre, o);
    if (lane >= o) pre += u;
  }
  if (lane == 31) s_warp[warp] = pre;
  __syncthreads();
  uint32_t wbase = 0, total = 0;
  for (int w = 0; w < 32; ++w) {
    if (w < warp) wbase += s_warp[w];
    total += s_warp[w];
  }
  uint32_t off = wbase + pre - csum;
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    round_off[tid * kPer + j] = off;
    round_fill[tid * kPer + j] = 0;
    off += cnt[j];
  }
  if (tid == 0) round_off[kRounds] = total;
}

__global__ void __launch_bounds__(kScanTiles) k_bucket_fill(int T, const uint32_t* __restrict__ ranges, int bs,
                                                            int split, long long max_buckets,
                                                            const uint32_t* __restrict__ block_sums,
                                                            const uint32_t* __restrict__ round_off,
                                                            uint32_t* __restrict__ round_fill,
                                                            uint32_t* __restrict__ bucket_off,
                                                            uint2* __restrict__ bucket_queue,
                                                            uint32_t* __restrict__ tile_stage, uint32_t* bucket_sum) {
  pdl_wait();  // the preceding kernel of the stream is done
  pdl_trigger();
  __shared__ uint32_t s_warp[kScanTiles / 32][kScanValues];
  __shared__ uint32_t s_base[kScanValues], s_total[kScanValues];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (warp < kScanValues) {  // totals of the preceding blocks and of all blocks, one value per warp
    uint32_t before = 0, all = 0;
    for (int i = lane; i < (int)gridDim.x; i += 32) {
      const uint32_t x = block_sums[(size_t)i * kScanValues + warp];
      all += x;
      if (i < (int)blockIdx.x) before += x;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      before += __shfl_xor_sync(0xffffffffu, before, o);
      all += __shfl_xor_sync(0xffffffffu, all, o);
    }
    if (lane == 0) { s_base[warp] = before; s_total[warp] = all; }
  }
  const int t = blockIdx.x * kScanTiles + tid;
  const uint32_t nb = t < T ? tile_buckets(ranges, t, bs) : 0u;
  {  // buckets of the stop granularity (FB's count): one atomic per warp
    uint32_t nf = t < T ? tile_buckets(ranges, t, bs * split) : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nf += __shfl_xor_sync(0xffffffffu, nf, o);
    if (lane == 0 && nf) atomicAdd(bucket_sum + 4, nf);
  }
  uint32_t v[kScanValues], tot[kScanValues];
  scan_values(nb, v);
  block_scan(v, tot, s_warp);  // its barriers also publish s_base / s_total
  const uint32_t total = s_total[1];
  const bool overflow = (long long)total > max_buckets;
  if (blockIdx.x == 0 && tid == 0) {
    bucket_sum[0] = overflow ? 0u : total;  // nothing is composited when the samples do not fit
    bucket_sum[1] = total;
    bucket_sum[2] = 0;  // forward work cursor
    if (overflow) raise_error(kErrCapacity);
  }
  const uint32_t end = s_base[1] + v[1];
  if (t < T) {
    tile_stage[t] = 0;
    bucket_off[t] = end;
  }
  if (overflow) return;
  // Rounds, 32 at a time: lane j requests the slots of round k0 + j for every
  // tile of the warp that reaches it (one atomic per warp and round, the 32
  // in flight together), then each tile writes its entries.  A warp holding a
  // deep tile (clustered scenes: thousands of buckets) takes ceil(rounds / 32)
  // steps instead of one dependent atomic per round.
  const uint32_t nr = min(nb, (uint32_t)kRounds);
  uint32_t wmax = nr;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
  for (uint32_t k0 = 0; k0 < wmax; k0 += kWarp) {
    uint32_t my_act = 0;  // tiles of the warp that reach round k0 + lane
#pragma unroll 4
    for (int j = 0; j < kWarp; ++j) {
      const uint32_t act = __ballot_sync(0xffffffffu, k0 + (uint32_t)j < nr);
      if (lane == j) my_act = act;
    }
    uint32_t base = 0;
    if (my_act) base = atomicAdd(round_fill + k0 + lane, (uint32_t)__popc(my_act));
#pragma unroll 4
    for (int j = 0; j < kWarp; ++j) {
      const uint32_t act = __shfl_sync(0xffffffffu, my_act, j);
      const uint32_t b = __shfl_sync(0xffffffffu, base, j);
      if ((act >> lane) & 1u)
        bucket_queue[round_off[k0 + j] + b + __popc(act & lanemask_lt())] = make_uint2((uint32_t)t, k0 + j);
    }
  }
  if (t >= T) return;
  const uint32_t tail = round_off[kRounds] + s_base[0] + v[0] - (nb > kRounds ? nb - kRounds : 0u);
  for (uint32_t k = kRounds; k < nb; ++k) bucket_queue[tail + (k - kRounds)] = make_uint2((uint32_t)t, k);
}

// Tiles without buckets (and every tile when the buckets did not fit): the
// merge's output for an empty list, background with T = 1.
__global__ void __launch_bounds__(kTilePixels) k_empty_tiles(const Views views, const uint32_t* __restrict__ ranges,
                                                             const uint32_t* bucket_sum, float* __restrict__ out_color,
                                                             float* __restrict__ pix_color,
                                                             int* __restrict__ last_contrib,
                                                             float* __restrict__ Ts_final,
                                                             uint32_t* __restrict__ max_contrib) {
  pdl_wait();  // the preceding kernel of the stream is done
  pdl_trigger();
  const int p = threadIdx.x;
  const bool all = bucket_sum[0] == 0;  // the buckets did not fit: every tile gets the empty-list output
  for (uint32_t tile = blockIdx.x; tile < views.tiles; tile += gridDim.x) {  // block-uniform
    if (!all && ranges[2 * tile + 1] > ranges[2 * tile]) continue;
    const ViewDesc& cam = views.v[views.of_tile(tile)];
    const int lt = (int)tile - (int)cam.tile_off, bx = views.bx, by = views.by;
    const int px = (lt % cam.gx) * bx + p % bx, py = (lt / cam.gx) * by + p / bx;
    if (p == 0) max_contrib[tile] = 0;
    if (px >= cam.W || py >= cam.H) continue;
    const size_t HW = (size_t)cam.W * cam.H, pix = (size_t)py * cam.W + px;
    float* oc = out_color + 3 * (size_t)cam.pix_off;
    float* pc = pix_color + 3 * (size_t)cam.pix_off;
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      oc[ch * HW + pix] = cam.bg[ch];
      pc[ch * HW + pix] = 0.f;
    }
    last_contrib[cam.pix_off + pix] = 0;
    Ts_final[cam.pix_off + pix] = 1.f;
  }
}

struct FwdArgs {
  Views views;
  const float* splat;
  const uint32_t* vals;
  const uint32_t* ranges;
  const uint2* bucket_queue;
  const uint32_t* bucket_off;
  uint32_t* bucket_sum;
  float4* samples;
  uint32_t* tile_stage;
  uint32_t* tile_alive;
  float* out_color;     // per view (3, H, W), view k at 3 * pix_off
  float* pix_color;     // same layout, without background
  int* last_contrib;    // per view (H, W), view k at pix_off
  float* Ts_final;
  uint32_t* max_contrib;
  int bs;      // Gaussians per (sub-)bucket
  int split;   // sub-buckets per bucket of the stop granularity
  int chain;   // the tile's fold chain covers its first `chain` buckets (store mode)
};

template <int BX, bool RECOMPUTE, int MIN_BLOCKS>
__global__ void __launch_bounds__(kFwdWarps * kWarp, MIN_BLOCKS) k_render_fwd(const FwdArgs a) {
  pdl_wait();  // the preceding kernel of the stream is done
  pdl_trigger();
  using M = TileMap<BX>;
  constexpr int BY = kTilePixels / BX;
  __shared__ BucketStage s_stage[kFwdWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  BucketStage& st = s_stage[warp];
  const int B = (int)a.bucket_sum[0];
  // Queue entries are prefetched one ahead; a bucket's own reads (offsets,
  // tile range, stage and alive words) are independent of one another.
  int q = next_bucket(a.bucket_sum + 2, lane), q_next = 0;
  uint2 e_cur = make_uint2(0u, 0u), e_next = e_cur;
  if (q < B) e_cur = a.bucket_queue[q];
  for (; q < B; q = q_next, e_cur = e_next) {
    q_next = next_bucket(a.bucket_sum + 2, lane);
    if (q_next < B) e_next = a.bucket_queue[q_next];
    const BucketInfo bi = bucket_info(e_cur, a.bucket_off, a.ranges, a.bs);
    const int b = bi.b;
    const ViewDesc& cam = a.views.v[a.views.of_tile((uint32_t)bi.tile)];
    const int lt = bi.tile - (int)cam.tile_off;  // tile index inside its view
    const int tx0 = (lt % cam.gx) * BX, ty0 = (lt / cam.gx) * BY;
    uint32_t* stage_word = a.tile_stage + bi.tile;
    uint32_t* alive_words = a.tile_alive + (size_t)bi.tile * kPxPerThread;

    const StageIds sid = load_stage_ids(a.vals + bi.start, bi.n, lane);  // in flight with the reads below
    // Sub-blocks that may still need this bucket: from whatever prefix state
    // the tile has published so far (a superset of the state after bucket k-1;
    // the alive words are read together with the stage and used once it shows
    // that some bucket was folded).
    uint32_t spec = (1u << kPxPerThread) - 1u;
    if (bi.local > 0) {
      uint32_t w = 0u;
      if (lane < kPxPerThread) {
        const uint32_t sw = ld_acquire_u32(stage_word);
        const uint32_t aw = ld_volatile_u32(alive_words + lane);
        w = sw > 0 ? aw : ~0u;
      }
      spec = __ballot_sync(0xffffffffu, w != 0u);
    }

    float T[kPxPerThread], Cr[kPxPerThread], Cg[kPxPerThread], Cb[kPxPerThread];
    if (spec != 0u) stage_bucket<BX>(st, a.splat, sid, bi.n, lane, tx0, ty0);
    {
      float pxc[M::kCols], pyr[M::kRows];
#pragma unroll
      for (int c = 0; c < M::kCols; ++c) pxc[c] = (float)(tx0 + 8 * c + (lane & 7));
#pragma unroll
      for (int r = 0; r < M::kRows; ++r) pyr[r] = (float)(ty0 + 4 * r + (lane >> 3));
      composite_bucket<BX>(st, bi.n, spec, pxc, pyr, T, Cr, Cg, Cb);
    }
    __syncwarp();

    if (!RECOMPUTE && bi.local >= a.chain) {
      // Past the tile's chain: keep this bucket's own (C, T) for the
      // sub-blocks that may still need it; k_deep_merge folds it in.
      if (spec != 0u) {
        float4* agg = a.samples + (size_t)b * kTilePixels;
#pragma unroll
        for (int r = 0; r < M::kRows; ++r)
#pragma unroll
          for (int cc = 0; cc < M::kCols; ++cc) {
            const int k = r * M::kCols + cc;
            if ((spec >> k) & 1u) __stcg(agg + M::pix(r, cc, lane), make_float4(Cr[k], Cg[k], Cb[k], T[k]));
          }
      }
      q = q_next;
      continue;
    }

    // Fold into the tile's prefix (FB's merge, render.cu:285-391, per pixel
    // and in bucket order): C += T_prefix * C_b, T_prefix *= T_b; a pixel
    // stops after the bucket of the stop granularity that takes T below 1e-4
    // (tested after its last sub-bucket only), or at the tile's last bucket,
    // and then writes its outputs.
    const bool last_bucket = bi.local == bi.nb_tile - 1;
    const bool stop_point = (bi.local + 1) % a.split == 0;  // end of a bucket of the stop granularity
    const int ntile = (int)(a.ranges[2 * bi.tile + 1] - a.ranges[2 * bi.tile]);
    const int contrib = min(ntile, (bi.local + 1) * a.bs);
    const size_t HW = (size_t)cam.W * cam.H;
    float4* out = a.samples + (size_t)(RECOMPUTE ? bi.tile : b) * kTilePixels;
    const float4* prev = RECOMPUTE ? out : a.samples + (size_t)(b - 1) * kTilePixels;
    // The link of the tile's chain: wait for bucket k-1's fold, then load the
    // alive words with the first half of the prefix samples, and the second
    // half after the first is folded (two round trips; the samples of pixels
    // that stopped are read and ignored).
    uint32_t prev_w = 0u;
    if (bi.local > 0) {
      // Every pixel of the tile has stopped: nothing to fold, write or publish
      // (kStageDead already satisfies the waits of every later bucket).
      if (wait_stage(stage_word, (uint32_t)bi.local, lane) == kStageDead) {
        q = q_next;
        continue;
      }
      if (lane < kPxPerThread) prev_w = ld_volatile_u32(alive_words + lane);
    }
    bool any_before = false, any_after = false;
    uint32_t my_word = 0;
    constexpr int kHalfRows = M::kRows / 2;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      float4 pre[kHalfRows * M::kCols];
#pragma unroll
      for (int rr = 0; rr < kHalfRows; ++rr)
#pragma unroll
        for (int cc = 0; cc < M::kCols; ++cc)
          pre[rr * M::kCols + cc] = bi.local > 0 ? __ldcg(prev + M::pix(h * kHalfRows + rr, cc, lane))
                                                 : make_float4(0.f, 0.f, 0.f, 1.f);
#pragma unroll
      for (int rr = 0; rr < kHalfRows; ++rr)
#pragma unroll
        for (int cc = 0; cc < M::kCols; ++cc) {
          const int r = h * kHalfRows + rr;
          const int k = r * M::kCols + cc;
          const float4 pk = pre[rr * M::kCols + cc];
          const int p = M::pix(r, cc, lane);
          const int px = tx0 + 8 * cc + (lane & 7), py = ty0 + 4 * r + (lane >> 3);
          bool alive;
          if (bi.local == 0) {
            alive = px < cam.W && py < cam.H;
          } else {
            alive = (__shfl_sync(0xffffffffu, prev_w, k) >> lane) & 1u;
          }
          any_before |= __any_sync(0xffffffffu, alive);
          if (alive) {
            const float nr = fmaf(pk.w, Cr[k], pk.x);
            const float ng = fmaf(pk.w, Cg[k], pk.y);
            const float nbl = fmaf(pk.w, Cb[k], pk.z);
            const float nt = pk.w * T[k];
            out[p] = make_float4(nr, ng, nbl, nt);
            if ((stop_point && nt < kTMin) || last_bucket) {
              alive = false;
              const size_t pix = (size_t)py * cam.W + px;
              float* oc = a.out_color + 3 * (size_t)cam.pix_off;
              float* pc = a.pix_color + 3 * (size_t)cam.pix_off;
              oc[pix] = nr + nt * cam.bg[0];
              oc[HW + pix] = ng + nt * cam.bg[1];
              oc[2 * HW + pix] = nbl + nt * cam.bg[2];
              pc[pix] = nr;
              pc[HW + pix] = ng;
              pc[2 * HW + pix] = nbl;
              a.last_contrib[cam.pix_off + pix] = contrib;
              a.Ts_final[cam.pix_off + pix] = nt;
            }
          }
          const uint32_t word = __ballot_sync(0xffffffffu, alive);
          any_after |= word != 0u;
          if (lane == k) my_word = word;
        }
    }
    if (lane < kPxPerThread) st_volatile_u32(alive_words + lane, my_word);
    if (lane == 0 && any_before && !any_after) a.max_contrib[bi.tile] = (uint32_t)contrib;
    // The bucket that stops the tile's last pixel ends the chain: its later
    // buckets skip their waits instead of handing an empty prefix along.
    publish_stage(stage_word, any_after ? (uint32_t)bi.local + 1u : kStageDead, lane);
    q = q_next;
  }
}

// The buckets of deep tiles past their chain (local index >= FwdArgs::chain),
// folded pixel-parallel once the composite kernel is done: FB's mergeResults
// (render.cu:285-391) for those buckets.  One thread per pixel walks the
// tile's remaining buckets in order from the chain's prefix, C += T C_b,
// T *= T_b, overwriting each bucket's own (C_b, T_b) with the prefix after it
// (what the backward reads), and stops after the bucket of the stop
// granularity that takes T below 1e-4, or at the tile's last bucket, where it
// writes its outputs.  Loads run kMergeAhead buckets ahead of the fold.
constexpr int kMergeAhead = 4;

template <int BX>
__global__ void __launch_bounds__(kTilePixels) k_deep_merge(const FwdArgs a) {
  pdl_wait();  // the preceding kernel of the stream is done
  pdl_trigger();
  using M = TileMap<BX>;
  constexpr int BY = kTilePixels / BX;
  __shared__ uint32_t s_max;
  if (a.bucket_sum[0] == 0) return;  // the buckets did not fit: k_empty_tiles writes every tile
  const int p = threadIdx.x, x = p % BX, y = p / BX;
  const int k = (y / 4) * M::kCols + x / 8;  // the pixel's sub-block slot and lane in the composite kernels
  const int owner = (y % 4) * 8 + (x % 8);
  for (uint32_t tile = blockIdx.x; tile < a.views.tiles; tile += gridDim.x) {  // block-uniform
    const int first = tile ? (int)a.bucket_off[tile - 1] : 0;
    const int nb = (int)a.bucket_off[tile] - first;
    if (nb <= a.chain || a.tile_stage[tile] == kStageDead) continue;  // the chain wrote every output
    const ViewDesc& cam = a.views.v[a.views.of_tile(tile)];
    const int lt = (int)tile - (int)cam.tile_off;
    const int px = (lt % cam.gx) * BX + x, py = (lt / cam.gx) * BY + y;
    const int ntile = (int)(a.ranges[2 * tile + 1] - a.ranges[2 * tile]);
    if (p == 0) s_max = 0u;
    __syncthreads();
    uint32_t contrib = 0u;
    if ((a.tile_alive[(size_t)tile * kPxPerThread + k] >> owner) & 1u) {  // still compositing after the chain
      float4* slot = a.samples + (size_t)first * kTilePixels + p;
      float4 pre = __ldcg(slot + (size_t)(a.chain - 1) * kTilePixels);
      float4 ahead[kMergeAhead];
#pragma unroll
      for (int j = 0; j < kMergeAhead; ++j)
        ahead[j] = a.chain + j < nb ? __ldcg(slot + (size_t)(a.chain + j) * kTilePixels)
                                    : make_float4(0.f, 0.f, 0.f, 1.f);
      for (int l0 = a.chain; l0 < nb && contrib == 0u; l0 += kMergeAhead) {
        float4 cur[kMergeAhead];
#pragma unroll
        for (int j = 0; j < kMergeAhead; ++j) {
          cur[j] = ahead[j];
          const int ln = l0 + kMergeAhead + j;
          ahead[j] = ln < nb ? __ldcg(slot + (size_t)ln * kTilePixels) : make_float4(0.f, 0.f, 0.f, 1.f);
        }
#pragma unroll
        for (int j = 0; j < kMergeAhead; ++j) {
          const int l = l0 + j;
          if (l >= nb || contrib != 0u) break;
          const float4 c = cur[j];
          pre = make_float4(fmaf(pre.w, c.x, pre.x), fmaf(pre.w, c.y, pre.y), fmaf(pre.w, c.z, pre.z), pre.w * c.w);
          __stcg(slot + (size_t)l * kTilePixels, pre);
          if (((l + 1) % a.split == 0 && pre.w < kTMin) || l == nb - 1) {
            contrib = (uint32_t)min(ntile, (l + 1) * a.bs);
            const size_t HW = (size_t)cam.W * cam.H, pix = (size_t)py * cam.W + px;
            float* oc = a.out_color + 3 * (size_t)cam.pix_off;
            float* pc = a.pix_color + 3 * (size_t)cam.pix_off;
            oc[pix] = pre.x + pre.w * cam.bg[0];
            oc[HW + pix] = pre.y + pre.w * cam.bg[1];
            oc[2 * HW + pix] = pre.z + pre.w * cam.bg[2];
            pc[pix] = pre.x;
            pc[HW + pix] = pre.y;
            pc[2 * HW + pix] = pre.z;
            a.last_contrib[cam.pix_off + pix] = (int)contrib;
            a.Ts_final[cam.pix_off + pix] = pre.w;
          }
        }
      }
    }
    if (contrib) atomicMax(&s_max, contrib);
    __syncthreads();
    if (p == 0) a.max_contrib[tile] = s_max;
    __syncthreads();
  }
}

// Self-check of the bounded waits: one warp waits, as a bucket of the chain
// does, for a stage that nothing publishes; the wait gives up after
// kSpinLimit polls, raises the timeout bit and the warp returns.
__global__ void k_selftest_wait(uint32_t* flag) { wait_stage(flag, 1u, threadIdx.x & 31); }

}  // namespace
}  // namespace fgs

FGS_DEFINE_ERROR_ACCESSOR(render)

extern "C" fgs_status fgs_selftest_wait(uint32_t* flag, void* stream) {
  using namespace fgs;
  if (!flag) return FGS_ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  FGS_TRY(cudaMemsetAsync(flag, 0, sizeof(uint32_t), s));
  k_selftest_wait<<<1, kWarp, 0, s>>>(flag);
  FGS_LAUNCH_CHECK();
  return FGS_OK;
}

namespace fgs {
fgs_status run_tile_ranges(int64_t n_cap, const int32_t* n_dev, uint32_t tiles, const uint64_t* keys_sorted,
                           uint32_t* ranges, cudaStream_t s, void* zero_also, size_t zero_bytes) {
  {
    const fgs_status z = zero_async(ranges, sizeof(uint32_t) * 2 * (size_t)tiles, s, zero_also, zero_bytes);
    if (z != FGS_OK) return z;
  }
  if (n_cap > 0) {
    KernelTimer kt__(FGS_K_TILE_RANGES, s);
    (void)launch_pdl(k_tile_ranges, dim3((unsigned)((n_cap + 1023) / 1024)), dim3(256), 0, s, 
        reinterpret_cast<const unsigned long long*>(keys_sorted), n_cap, n_dev, tiles, ranges);
    kt__.stop();
    FGS_LAUNCH_CHECK();
  }
  return FGS_OK;
}

fgs_status run_render_fwd(const Views& views, int64_t n_cap, const int32_t* n_dev, int bucket_size,
                          const float* splat, const uint64_t* keys_sorted, const uint32_t* values_sorted,
                          uint32_t* ranges, float* out_color, int32_t* last_contributor, float* Ts_final,
                          const ImageState& im, const SampleState& sm, int64_t max_buckets, bool recompute,
                          cudaStream_t s, int chain) {
  if (chain < 1) return FGS_ERR_BAD_ARG;
  // the ranges and the round histogram of the bucket setup are cleared by one launch
  fgs_status st = run_tile_ranges(n_cap, n_dev, views.tiles, keys_sorted, ranges, s, im.round_hist,
                                  sizeof(uint32_t) * (kRounds + 1));
  if (st != FGS_OK) return st;
  const int split = bucket_split(bucket_size), sub = sub_bucket_size(bucket_size);
  {
    KernelTimer kt__(FGS_K_BUCKET_SETUP, s, 3);
    const unsigned nblk = (views.tiles + kScanTiles - 1) / kScanTiles;
    (void)launch_pdl(k_bucket_count, dim3(nblk), dim3(kScanTiles), 0, s, (int)views.tiles, ranges, sub,
                     im.block_sums, im.round_hist, im.bucket_sum);
    (void)launch_pdl(k_round_offsets, dim3(1), dim3(1024), 0, s, im.round_hist, im.round_off, im.round_fill);
    (void)launch_pdl(k_bucket_fill, dim3(nblk), dim3(kScanTiles), 0, s, (int)views.tiles, ranges, sub, split,
                     max_buckets, im.block_sums, im.round_off, im.round_fill, im.bucket_off, sm.bucket_queue,
                     im.tile_stage, im.bucket_sum);
    kt__.stop();
  }
  FGS_LAUNCH_CHECK();
  FwdArgs fa{views, splat, values_sorted, ranges, sm.bucket_queue, im.bucket_off, im.bucket_sum,
             sm.samples, im.tile_stage, im.tile_alive, out_color, im.pix_color, last_contributor, Ts_final,
             im.max_contrib, sub, split, chain};
  {
    KernelTimer kt__(FGS_K_RENDER_FWD, s);
    const int nt = kFwdWarps * kWarp;
    auto launch = [&](auto kernel) {
      (void)launch_pdl(kernel, dim3(num_sms() * resident_blocks(kernel, nt, 0)), dim3(nt), 0, s, fa);
    };
    auto by_tile = [&](auto rc, auto mb) {
      constexpr bool R = decltype(rc)::value;
      constexpr int B = decltype(mb)::value;
      if (views.bx == 8) launch(k_render_fwd<8, R, B>);
      else if (views.bx == 16) launch(k_render_fwd<16, R, B>);
      else launch(k_render_fwd<32, R, B>);
    };
    using Few = std::integral_constant<int, 6>;
    using Many = std::integral_constant<int, 7>;
    // recompute mode: the samples hold one running prefix per tile
    if (recompute) {
      if (views.tiles <= kFwdFewTiles) by_tile(std::true_type{}, Few{});
      else by_tile(std::true_type{}, Many{});
    } else {
      if (views.tiles <= kFwdFewTiles) by_tile(std::false_type{}, Few{});
      else by_tile(std::false_type{}, Many{});
    }
    kt__.stop();
  }
  FGS_LAUNCH_CHECK();
  if (!recompute) {
    KernelTimer kt__(FGS_K_DEEP_MERGE, s);
    const unsigned grid = std::min<unsigned>(views.tiles, (unsigned)num_sms() * 8);
    if (views.bx == 8) (void)launch_pdl(k_deep_merge<8>, dim3(grid), dim3(kTilePixels), 0, s, fa);
    else if (views.bx == 16) (void)launch_pdl(k_deep_merge<16>, dim3(grid), dim3(kTilePixels), 0, s, fa);
    else (void)launch_pdl(k_deep_merge<32>, dim3(grid), dim3(kTilePixels), 0, s, fa);
    kt__.stop();
    FGS_LAUNCH_CHECK();
  }
  {
    KernelTimer kt__(FGS_K_EMPTY_TILES, s);
    (void)launch_pdl(k_empty_tiles, dim3(std::min<unsigned>(views.tiles, (unsigned)num_sms() * 8)), dim3(kTilePixels),
                     0, s, views, ranges, im.bucket_sum, out_color, im.pix_color, last_contributor, Ts_final,
                     im.max_contrib);
    kt__.stop();
  }
  FGS_LAUNCH_CHECK();
  return FGS_OK;
}

bool tile_shape_ok(int bx, int by) { return bx * by == kTilePixels && (bx == 8 || bx == 16 || bx == 32); }
}  // namespace fgs

using namespace fgs;

extern "C" fgs_status fgs_tile_ranges(int64_t num_rendered, int num_tiles, const uint64_t* keys_sorted,
                                      uint32_t* ranges, void* stream) {
  if (num_rendered < 0 || num_tiles <= 0 || !ranges || (num_rendered > 0 && !keys_sorted)) return FGS_ERR_BAD_ARG;
  return run_tile_ranges(num_rendered, nullptr, (uint32_t)num_tiles, keys_sorted, ranges, (cudaStream_t)stream);
}

extern "C" int64_t fgs_max_buckets(int64_t num_rendered, int width, int height, int block_x, int block_y,
                                   int bucket_size) {
  if (width <= 0 || height <= 0 || block_x <= 0 || block_y <= 0 || bucket_size <= 0 || num_rendered < 0) return -1;
  const int64_t T = (int64_t)((width + block_x - 1) / block_x) * ((height + block_y - 1) / block_y);
  // Sub-buckets (the units of the sample state); every tile wastes at most
  // one partially filled one.
  const int64_t sub = bucket_size > kMaxBucket ? bucket_size : sub_bucket_size(bucket_size);
  return (num_rendered + sub - 1) / sub + std::min<int64_t>(T, num_rendered);
}

extern "C" fgs_status fgs_state_bytes(int width, int height, int block_x, int block_y, int64_t max_buckets,
                                      size_t* image_bytes, size_t* sample_bytes) {
  if (width <= 0 || height <= 0 || block_x <= 0 || block_y <= 0 || max_buckets < 0) return FGS_ERR_BAD_ARG;
  const size_t T = (size_t)((width + block_x - 1) / block_x) * ((height + block_y - 1) / block_y);
  if (image_bytes) *image_bytes = carve_image(nullptr, (size_t)width * height, T).bytes;
  const int64_t mb = std::max<int64_t>(max_buckets, 1);
  if (sample_bytes) *sample_bytes = carve_sample(nullptr, mb, mb).bytes;
  return FGS_OK;
}

extern "C" fgs_status fgs_render_fwd(int P, int64_t num_rendered, int width, int height, int block_x, int block_y,
                                     int bucket_size, const float* splat_buffer, const uint64_t* keys_sorted,
                                     const uint32_t* values_sorted, uint32_t* ranges, const float* bg,
                                     float* out_color, int32_t* last_contributor, float* Ts_final,
                                     void* image_state, size_t image_bytes, void* sample_state,
                                     size_t sample_bytes, int64_t max_buckets, uint32_t* bucket_sum_host,
                                     void* stream) {
  (void)P;
  if (width <= 0 || height <= 0 || !tile_shape_ok(block_x, block_y) || bucket_size < 1 ||
      bucket_size > kMaxBucket || num_rendered < 0 || max_buckets < 0)
    return FGS_ERR_BAD_ARG;
  if (!splat_buffer || !ranges || !bg || !out_color || !last_contributor || !Ts_final || !image_state ||
      !sample_state || (num_rendered > 0 && (!keys_sorted || !values_sorted)))
    return FGS_ERR_BAD_ARG;
  if (((uintptr_t)splat_buffer & 15) || ((uintptr_t)image_state & 255) || ((uintptr_t)sample_state & 255))
    return FGS_ERR_BAD_ARG;
  const Views views = single_view(width, height, block_x, block_y, nullptr, nullptr, nullptr, bg, 1.f, 1.f, 1.f, 1.f);
  const ImageState im = carve_image(image_state, (size_t)width * height, views.tiles);
  const int64_t mb = std::max<int64_t>(max_buckets, 1);
  const SampleState sm = carve_sample(sample_state, mb, mb);
  if (image_bytes < im.bytes || sample_bytes < sm.bytes) return FGS_ERR_CAPACITY;
  cudaStream_t s = (cudaStream_t)stream;
  const fgs_status st = run_render_fwd(views, num_rendered, nullptr, bucket_size, splat_buffer, keys_sorted,
                                       values_sorted, ranges, out_color, last_contributor, Ts_final, im, sm,
                                       max_buckets, false, s);
  if (st != FGS_OK) return st;
  if (bucket_sum_host) {
    uint32_t hs[5] = {0, 0, 0, 0, 0};
    FGS_TRY(cudaMemcpyAsync(hs, im.bucket_sum, sizeof(hs), cudaMemcpyDeviceToHost, s));
    FGS_TRY(cudaStreamSynchronize(s));
    *bucket_sum_host = hs[4];
    if ((int64_t)hs[1] > max_buckets) return FGS_ERR_CAPACITY;
  }
  return FGS_OK;
}
