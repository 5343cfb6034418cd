// State layout shared by the forward and backward composite kernels.
#pragma once
#include <map>
#include <mutex>
#include <tuple>

#include "internal.cuh"

namespace fgs {

constexpr int kTilePixels = 256;   // block_x * block_y must equal this
constexpr int kPxPerThread = 8;    // pixels per lane: one warp covers a tile
constexpr int kMaxBucket = 128;    // largest supported bucket size

// A bucket of bucket_size Gaussians is the merge's stop granularity (FB's
// BUCKET_SIZE: a pixel stops after the bucket that takes its transmittance
// below 1e-4).  Buckets larger than kSubBucket are composited as the fewest
// equal sub-buckets of at most kSubBucket Gaussians (FB's 128: two of 64),
// each with its own prefix sample, and the stop test runs only after a
// bucket's last sub-bucket, so the outputs keep the bucket's stop semantics
// while a tile's chain has more links to spread over the GPU, and a warp
// stages at most kSubBucket records.
// "Bucket" in the composite kernels, the bookkeeping and the sample state
// means the sub-bucket.
constexpr int kSubBucket = 64;  // largest composited (sub-)bucket: the size of the shared-memory stage
inline int bucket_split(int bucket_size) {
  // fewest equal sub-buckets of at most kSubBucket Gaussians that tile the bucket
  int s = (bucket_size + kSubBucket - 1) / kSubBucket;
  while (s < bucket_size && bucket_size % s != 0) ++s;
  return s < 1 ? 1 : s;
}
inline int sub_bucket_size(int bucket_size) { return bucket_size / bucket_split(bucket_size); }

// Per-image state (FB ImageState, rasterizer_imp.h:76-88), carved from one
// caller buffer:  pixel colour planes (3, H*W) without background,
// per-tile max contributor count, per-tile inclusive bucket offsets, a
// 16-byte header holding the bucket total and work cursors, the bucket-setup
// scan's block totals, and the per-tile chain state of the forward composite
// (number of buckets folded into the tile's running prefix, and which pixels
// are still above the transmittance cut-off).
constexpr int kScanTiles = 1024;  // tiles per bucket-setup scan block
constexpr int kRounds = 4096;     // bucket rounds of the forward work queue (local index < kRounds)
constexpr int kScanValues = 2;    // per tile: buckets past the last round, buckets
struct ImageState {
  float* pix_color;         // 3 * HW
  uint32_t* max_contrib;    // T
  uint32_t* bucket_off;     // T (inclusive scan of bucket counts)
  uint32_t* bucket_sum;     // [0] sub-buckets to render, [1] sub-buckets needed, [2], [3] work
                            // cursors, [4] buckets of bucket_size (the count FB reports),
                            // [5] entries of the backward's live-bucket list
  uint32_t* block_sums;     // ceil(T / kScanTiles) x kScanValues
  uint32_t* tile_stage;     // T: buckets of the tile folded into its prefix
  uint32_t* tile_alive;     // T x 8: per 8x4 sub-block, lanes whose pixel is still compositing
  uint32_t* round_hist;     // kRounds + 1: tiles by bucket count (capped at kRounds)
  uint32_t* round_off;      // kRounds + 1: first queue slot of every round, then of the tail
  uint32_t* round_fill;     // kRounds: slots handed out per round
  size_t bytes;
};

// Per-bucket state (FB SampleState, rasterizer_imp.h:91-102): the forward work
// queue (each entry names its tile), the backward's live list, and per (bucket, pixel) a float4
// (C.rgb, T) holding the running prefix after the bucket, which is all the
// backward needs (16 bytes per pixel and bucket instead of FB's 40).
struct SampleState {
  uint2* bucket_queue;      // max_buckets: forward processing order, entries (tile, local index)
  uint4* live;              // max_buckets: the backward's work list (store mode), one entry per
                            // bucket that some pixel reaches: bucket, tile, first pair, local << 8 | n
  float4* samples;          // max_buckets * 256
  int64_t max_buckets;
  size_t bytes;
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// pixels: all pixels of all views (colour planes of view k at 3 * pix_off).
inline ImageState carve_image(void* base, size_t pixels, size_t T) {
  char* p = static_cast<char*>(base);
  ImageState s;
  size_t off = 0;
  const size_t nblk = (T + kScanTiles - 1) / kScanTiles;
  s.bucket_sum = reinterpret_cast<uint32_t*>(p + off);  off = align_up(off + 32, 256);
  s.pix_color = reinterpret_cast<float*>(p + off);      off = align_up(off + sizeof(float) * 3 * pixels, 256);
  s.max_contrib = reinterpret_cast<uint32_t*>(p + off); off = align_up(off + sizeof(uint32_t) * T, 256);
  s.bucket_off = reinterpret_cast<uint32_t*>(p + off);  off = align_up(off + sizeof(uint32_t) * T, 256);
  s.block_sums = reinterpret_cast<uint32_t*>(p + off);  off = align_up(off + sizeof(uint32_t) * nblk * kScanValues, 256);
  s.tile_stage = reinterpret_cast<uint32_t*>(p + off);  off = align_up(off + sizeof(uint32_t) * T, 256);
  s.tile_alive = reinterpret_cast<uint32_t*>(p + off);  off = align_up(off + sizeof(uint32_t) * 8 * T, 256);
  s.round_hist = reinterpret_cast<uint32_t*>(p + off);  off = align_up(off + sizeof(uint32_t) * (kRounds + 1), 256);
  s.round_off = reinterpret_cast<uint32_t*>(p + off);   off = align_up(off + sizeof(uint32_t) * (kRounds + 1), 256);
  s.round_fill = reinterpret_cast<uint32_t*>(p + off);  off = align_up(off + sizeof(uint32_t) * kRounds, 256);
  s.bytes = off;
  return s;
}

// slots: prefix samples kept -- one per bucket (stored for the backward) or,
// in recompute mode, one per tile (the running prefix, rebuilt by the backward).
inline SampleState carve_sample(void* base, int64_t max_buckets, int64_t slots) {
  char* p = static_cast<char*>(base);
  SampleState s;
  size_t off = 0;
  s.bucket_queue = reinterpret_cast<uint2*>(p + off);   off = align_up(off + sizeof(uint2) * (size_t)max_buckets, 256);
  s.live = reinterpret_cast<uint4*>(p + off);           off = align_up(off + sizeof(uint4) * (size_t)max_buckets, 256);
  s.samples = reinterpret_cast<float4*>(p + off);       off = align_up(off + sizeof(float4) * kTilePixels * (size_t)slots, 256);
  s.max_buckets = max_buckets;
  s.bytes = off;
  return s;
}

// Pixel mapping of the compositing kernels: a warp covers one tile as a grid
// of 8 x 4 sub-blocks (2 x 4 of them for 16 x 16 tiles); lane l owns pixel
// (l & 7, l >> 3) of every sub-block.  A Gaussian is evaluated only on the
// sub-blocks its alpha >= 1/256 ellipse reaches, a warp-uniform decision.
template <int BX>
struct TileMap {
  static constexpr int kCols = BX / 8;               // sub-blocks per row
  static constexpr int kRows = kTilePixels / BX / 4;  // sub-block rows
  static_assert(kCols * kRows == kPxPerThread, "one pixel per lane per sub-block");
  // pixel index inside the tile (row-major, BX wide) of sub-block (r, c) for this lane
  __device__ static int pix(int r, int c, int lane) { return (4 * r + (lane >> 3)) * BX + 8 * c + (lane & 7); }
};

// Records of one bucket staged in shared memory, structure-of-arrays.
struct BucketStage {
  float4 pos[kSubBucket];     // floor(x), floor(y), fraction x, fraction y
  float4 quad[kSubBucket];    // A1, P, C1, log2 opacity
  float4 rgb[kSubBucket];     // r, g, b, Gaussian id bits
  uint32_t mask[kSubBucket];  // sub-blocks the Gaussian can reach (bit r * kCols + c)
};

// The record ids of a bucket a lane stages (entries lane, lane + 32), loaded
// ahead so that their latency overlaps other reads.
struct StageIds {
  uint32_t id[kSubBucket / kWarp];
};
__device__ __forceinline__ StageIds load_stage_ids(const uint32_t* __restrict__ ids, int n, int lane) {
  StageIds s;
#pragma unroll
  for (int k = 0; k < kSubBucket / kWarp; ++k) {
    const int j = lane + k * kWarp;
    s.id[k] = j < n ? ids[j] : 0u;
  }
  return s;
}

// Stage the render fields (floats 0..11) of the n records whose ids are in
// sid, and each Gaussian's sub-block mask for the tile at (tx0, ty0).
template <int BX>
__device__ __forceinline__ void stage_bucket(BucketStage& st, const float* __restrict__ splat, const StageIds& sid,
                                             int n, int lane, int tx0, int ty0) {
  using M = TileMap<BX>;
#pragma unroll
  for (int k = 0; k < kSubBucket / kWarp; ++k) {
    const int j = lane + k * kWarp;
    if (j >= n) break;
    const uint32_t id = sid.id[k];
    const float4* r = reinterpret_cast<const float4*>(splat + (size_t)id * 32);
    const float4 a = __ldg(r);        // x, y, r, g
    const float4 b = __ldg(r + 1);    // b, depth, A1, P
    const float4 c = __ldg(r + 2);    // C1, log2 o, fraction x, fraction y
    const float X = floorf(a.x), Y = floorf(a.y);
    st.pos[j] = make_float4(X, Y, c.z, c.w);
    st.quad[j] = make_float4(b.z, b.w, c.x, c.y);
    st.rgb[j] = make_float4(a.z, a.w, b.x, __uint_as_float(id));
    // Sub-blocks the ellipse alpha >= 1/256 reaches, from the exponent's own
    // form e = log2 o + A1 w^2 + C1 dy^2, w = dx + P dy (A1, C1 < 0):
    // e >= -8 needs |dy| <= sqrt(L / -C1) with L = log2 o + 8, and at a given
    // dy, w within +-W(dy) = sqrt((L + C1 dy^2) / -A1), i.e. dx within
    // -P dy +- W(dy).  Over a sub-block's 4 pixel rows that is a sheared
    // interval, much tighter than the bounding box for rotated, elongated
    // footprints.  Outside it alpha < 1/256 < 1/255 even after FP32 rounding
    // (the 1e-3 px margins cover it), so skipping those pixels changes nothing.
    const float L = c.y + 8.0f;
    uint32_t m = 0;
    if (L > 0.f) {
      const float inv_nA = -1.0f / b.z, nC = -c.x, P = b.w;
      const float ry = sqrtf(L / nC) + 1e-3f;
      const float cx = (X - (float)tx0) + c.z, cy = (Y - (float)ty0) + c.w;
#pragma unroll
      for (int sr = 0; sr < M::kRows; ++sr) {
        const float dlo = cy - (4.f * sr + 3.f), dhi = cy - 4.f * sr;  // dy over the sub-block's rows
        if (dhi < -ry || dlo > ry) continue;
        const float dys = fminf(fmaxf(0.f, dlo), dhi);  // the |dy|-smallest row offset
        const float wm = sqrtf(fmaxf(0.f, (L - nC * dys * dys) * inv_nA)) + 1e-3f;
        const float s0 = -P * dlo, s1 = -P * dhi;
        const float lo = fminf(s0, s1) - wm, hi = fmaxf(s0, s1) + wm;
#pragma unroll
        for (int sc = 0; sc < M::kCols; ++sc) {
          const float xr = cx - 8.f * sc;  // dx at the sub-block's first column
          if (xr - 7.f <= hi && xr >= lo) m |= 1u << (sr * M::kCols + sc);
        }
      }
    }
    st.mask[j] = m;
  }
  __syncwarp();
}

// Offsets from a pixel to a staged Gaussian's centre: the integer parts
// subtract exactly, the fraction adds once.
__device__ __forceinline__ float centre_offset(float whole, float frac, float pixel) {
  return (whole - pixel) + frac;
}

// The exponent's sheared offset w = dx + P dy from the exact integer offsets
// ix = X - px, iy = Y - py and the Gaussian's constant wfrac = P fy + fx:
// one rounding at the size of w itself.  Summing dx and P dy as rounded
// values lost ~1e-4 px for a far-away elongated footprint (dx and P dy near
// -1100 and +1100 px, w near 2), which moved alpha by 1e-4 relative and
// could flip its 1/255 cut; here w is good to ~1e-7 px.
__device__ __forceinline__ float shear_offset(float P, float iy, float ix, float wfrac) {
  return fmaf(P, iy, ix) + wfrac;
}

// Composites a staged bucket front to back from T = 1, C = 0 for this lane's
// 8 pixels, restricted to the sub-blocks in `live` (FB renderBucket,
// render.cu:285-391): alpha = min(0.99, o 2^e), dropped below 1/255.
// Skipped (Gaussian, sub-block) pairs have alpha < 1/256 everywhere and would
// leave C and T bit-for-bit unchanged.
//
// The 8 pixels are processed as 4 packed pairs (pixel slots 2j, 2j + 1, the
// two halves of one 8x4 sub-block row pair) with f32x2 arithmetic.  The blend
// runs on the negated alpha and colour, -wt = (-alpha) T and
// C + (-c)(-wt), which are bit-identical to C + c (alpha T) and
// T + (-alpha) T of the scalar form.
template <int BX>
__device__ __forceinline__ void composite_bucket(const BucketStage& st, int n, uint32_t live,
                                                 const float (&pxc)[TileMap<BX>::kCols],
                                                 const float (&pyr)[TileMap<BX>::kRows], float (&T)[kPxPerThread],
                                                 float (&Cr)[kPxPerThread], float (&Cg)[kPxPerThread],
                                                 float (&Cb)[kPxPerThread]) {
  using M = TileMap<BX>;
  constexpr int kPairs = kPxPerThread / 2;
  f2x T2[kPairs], R2[kPairs], G2[kPairs], B2[kPairs];
  const f2x one2 = f2_pack(1.f, 1.f), zero2 = f2_pack(0.f, 0.f);
#pragma unroll
  for (int j = 0; j < kPairs; ++j) { T2[j] = one2; R2[j] = zero2; G2[j] = zero2; B2[j] = zero2; }
  if (live != 0u) {
    for (int g = 0; g < n; ++g) {
      const uint32_t mask = st.mask[g] & live;
      if (mask == 0) continue;  // alpha < 1/256 on every live sub-block
      const float4 pos = st.pos[g];
      const float4 q4 = st.quad[g];   // A1, P, C1, log2 o
      const float4 c = st.rgb[g];
      const f2x A2 = f2_pack(q4.x, q4.x), P2 = f2_pack(q4.y, q4.y);
      const f2x nr2 = f2_pack(-c.x, -c.x), ng2 = f2_pack(-c.y, -c.y), nb2 = f2_pack(-c.z, -c.z);
      const float wfrac = fmaf(q4.y, pos.w, pos.z);  // P fy + fx (shear_offset)
      const f2x wf2 = f2_pack(wfrac, wfrac);
      float ix[M::kCols];
#pragma unroll
      for (int cc = 0; cc < M::kCols; ++cc) ix[cc] = pos.x - pxc[cc];  // exact
      auto pair_step = [&](const int j) {
        const int k0 = 2 * j, k1 = 2 * j + 1;  // pixel slots k = r * kCols + cc
        const int r0 = k0 / M::kCols, c0 = k0 % M::kCols, r1 = k1 / M::kCols, c1 = k1 % M::kCols;
        const float iy0 = pos.y - pyr[r0], iy1 = r1 == r0 ? iy0 : pos.y - pyr[r1];  // exact
        const float dy0 = iy0 + pos.w;
        const float dy1 = r1 == r0 ? dy0 : iy1 + pos.w;
        const float f0 = fmaf(q4.z * dy0, dy0, q4.w);  // log2 o + C1 dy^2
        const float f1 = r1 == r0 ? f0 : fmaf(q4.z * dy1, dy1, q4.w);
        // alpha = o * exp(-q/2) = 2^(log2 o + A1 (dx + P dy)^2 + C1 dy^2), w = dx + P dy (shear_offset)
        const f2x w2 = f2_add(f2_fma(P2, f2_pack(iy0, iy1), f2_pack(ix[c0], ix[c1])), wf2);
        const f2x e2 = f2_fma(f2_mul(A2, w2), w2, f2_pack(f0, f1));
        float e0, e1;
        f2_unpack(e2, e0, e1);
        // -alpha: -min(0.99, 2^e), and 0 where alpha < 1/255
        float n0 = fmaxf(-kAlphaMax, -ex2_approx(e0)), n1 = fmaxf(-kAlphaMax, -ex2_approx(e1));
        n0 = n0 > -kAlphaCut ? 0.f : n0;
        n1 = n1 > -kAlphaCut ? 0.f : n1;
        const f2x na2 = f2_pack(n0, n1);
        const f2x nwt2 = f2_mul(na2, T2[j]);  // -alpha T
        R2[j] = f2_fma(nr2, nwt2, R2[j]);
        G2[j] = f2_fma(ng2, nwt2, G2[j]);
        B2[j] = f2_fma(nb2, nwt2, B2[j]);
        T2[j] = f2_fma(na2, T2[j], T2[j]);    // T (1 - alpha), rounded once
      };
      // Every pixel pair has a sub-block the Gaussian reaches (the common case
      // for large footprints): the four pair chains run without per-pair
      // branches, so they interleave; otherwise pairs without one are skipped.
      if (((mask | (mask >> 1)) & 0x55u) == 0x55u) {
#pragma unroll
        for (int j = 0; j < kPairs; ++j) pair_step(j);
      } else {
#pragma unroll
        for (int j = 0; j < kPairs; ++j)
          if (((mask >> (2 * j)) & 3u) != 0u) pair_step(j);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < kPairs; ++j) {
    f2_unpack(T2[j], T[2 * j], T[2 * j + 1]);
    f2_unpack(R2[j], Cr[2 * j], Cr[2 * j + 1]);
    f2_unpack(G2[j], Cg[2 * j], Cg[2 * j + 1]);
    f2_unpack(B2[j], Cb[2 * j], Cb[2 * j + 1]);
  }
}

// tile_stage value of a tile whose pixels have all stopped: it satisfies every
// wait, and the buckets that read it do nothing.
constexpr uint32_t kStageDead = 0xffffffffu;

// Length of a tile's fold chain in the forward (store mode).  The chain folds
// a tile's first kChainBuckets (sub-)buckets one after another, which lets
// every later bucket skip the sub-blocks whose pixels have stopped; each
// link costs a few dependent L2 round trips.  A deep tile (hundreds of
// buckets in a dense cluster) would make that chain the frame's critical
// path, so its later buckets composite without waiting, store their own
// (C, T) from T = 1 in their sample slot, and k_deep_merge folds them into
// the prefix pixel-parallel once the composite kernel is done (FB's merge,
// for those buckets only).  Both orders compute the same operations on the
// same values: the results are bit-identical.  kChainBuckets is the default
// length; the batched path takes it from its launch configuration.
constexpr int kChainBuckets = 8;

// Waits until a tile's first `stage` buckets are folded into its prefix.
// Lane 0 polls (bounded); the bucket it waits for was handed out earlier and
// its warp is running, so the wait ends unless something is broken, in which
// case the timeout bit is raised and the warp carries on.
// Returns the stage every lane acquired (>= stage unless the wait expired;
// kStageDead when the tile's last pixel has stopped).
__device__ __forceinline__ uint32_t wait_stage(const uint32_t* tile_stage, uint32_t stage, int lane) {
  if (lane == 0) {
    int spins = 0;
    while (ld_acquire_u32(tile_stage) < stage) {
      if (++spins > kSpinLimit) {
        raise_error(kErrTimeout);
        break;
      }
      if (spins > 64) __nanosleep(128);
    }
  }
  __syncwarp();
  return ld_acquire_u32(tile_stage);  // every lane acquires the folded prefix
}

// Publishes that the tile's first `stage` buckets are folded (after every
// lane's prefix stores).
__device__ __forceinline__ void publish_stage(uint32_t* tile_stage, uint32_t stage, int lane) {
  __threadfence();
  __syncwarp();
  if (lane == 0) st_release_u32(tile_stage, stage);
}

// Dynamic bucket scheduling for the persistent compositing kernels: every
// warp takes the next unprocessed bucket from a device cursor, so buckets of
// very different cost balance across SMs.  Lane 0 fetches; the next index is
// requested before the current bucket is processed to hide the atomic.
__device__ __forceinline__ int next_bucket(uint32_t* cursor, int lane) {
  uint32_t b = 0;
  if (lane == 0) b = atomicAdd(cursor, 1u);
  return (int)__shfl_sync(0xffffffffu, b, 0);
}

// Blocks per SM that a kernel can keep resident, for sizing persistent grids.
// Cached per (kernel, block size, device) so that launches issue no runtime
// queries (and stay cheap while a CUDA graph is being captured).
template <typename K>
inline int resident_blocks(K kernel, int threads, size_t smem) {
  static std::mutex mu;
  static std::map<std::tuple<const void*, int, size_t, int>, int> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  const auto key = std::make_tuple(reinterpret_cast<const void*>(kernel), threads, smem, dev);
  std::lock_guard<std::mutex> lk(mu);
  const auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess || n < 1) n = 1;
  cache.emplace(key, n);
  return n;
}

// Bucket b -> (tile, first pair, pair count, index of the bucket in its tile).
struct BucketInfo {
  int tile, start, n, local;
  int b;        // global bucket index (sample slot)
  int nb_tile;  // buckets of the tile
};
// The bucket of queue entry (tile, local): the four reads are independent.
__device__ __forceinline__ BucketInfo bucket_info(uint2 qe, const uint32_t* __restrict__ bucket_off,
                                                  const uint32_t* __restrict__ ranges, int bs) {
  BucketInfo bi;
  bi.tile = (int)qe.x;
  bi.local = (int)qe.y;
  const int first = bi.tile ? (int)bucket_off[bi.tile - 1] : 0;
  const int last = (int)bucket_off[bi.tile];
  const int rs = (int)ranges[2 * bi.tile], re = (int)ranges[2 * bi.tile + 1];
  bi.b = first + bi.local;
  bi.nb_tile = last - first;
  bi.start = rs + bi.local * bs;
  bi.n = min(bs, re - bi.start);
  return bi;
}

// Launch sequences shared by the plain and the batched entry points.
// Forward: tile ranges, bucket setup, persistent composite, merge.  n_dev,
// when given, is the device-side pair count (clamped to n_cap).
// recompute: the sample state holds one running prefix per tile instead of
// one prefix per bucket (carve_sample with slots = tiles).
fgs_status run_render_fwd(const Views& views, int64_t n_cap, const int32_t* n_dev, int bucket_size,
                          const float* splat, const uint64_t* keys_sorted, const uint32_t* values_sorted,
                          uint32_t* ranges, float* out_color, int32_t* last_contributor, float* Ts_final,
                          const ImageState& im, const SampleState& sm, int64_t max_buckets, bool recompute,
                          cudaStream_t s, int chain = kChainBuckets);
// Backward composite into grad_record (records x FGS_GRAD_STRIDE, zeroed here).
// In recompute mode every needed bucket's prefix is rebuilt from the tile's
// running prefix, in bucket order per tile.
fgs_status run_render_bwd(const Views& views, int64_t records, int bucket_size, const uint32_t* values_sorted,
                          const uint32_t* ranges, const float* splat, const float* Ts_final,
                          const int32_t* last_contributor, const ImageState& im, const SampleState& sm,
                          const float* dL_dpixels, float* grad_record, bool recompute, bool abs_grad,
                          cudaStream_t s);

}  // namespace fgs
