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
//   * a bucket's records are staged once into shared memory (coalesced
//     per-lane loads, structure-of-arrays) and broadcast from there;
//   * each lane owns a column strip of 8 pixels, so a Gaussian's row terms are
//     shared and every sample store is a contiguous 512-byte warp store;
//   * the sample state is 16 bytes per pixel and bucket, updated in place by
//     the merge (FB keeps 40).
#include <algorithm>

#include "render_common.cuh"

namespace fgs {
namespace {

constexpr int kFwdWarps = 4;

__global__ void __launch_bounds__(256) k_tile_ranges(const unsigned long long* __restrict__ keys, long long n_cap,
                                                     const int* n_dev, uint32_t num_tiles,
                                                     uint32_t* __restrict__ ranges) {
  const long long n = n_dev ? min(n_cap, (long long)(unsigned int)*n_dev) : n_cap;
  const long long i = blockIdx.x * 256ll + threadIdx.x;
  if (i >= n) return;
  const uint32_t t = (uint32_t)(keys[i] >> 32);
  if (t >= num_tiles) {  // not a key of this frame
    raise_error(kErrCapacity);
    return;
  }
  if (i == 0) {
    ranges[2 * t] = 0;
  } else {
    const uint32_t pt = (uint32_t)(keys[i - 1] >> 32);
    if (pt != t && pt < num_tiles) {
      ranges[2 * pt + 1] = (uint32_t)i;
      ranges[2 * t] = (uint32_t)i;
    }
  }
  if (i == n - 1) ranges[2 * t + 1] = (uint32_t)n;
}

// One CTA: bucket counts per tile, inclusive scan, bucket -> tile map.
// FB does this with perTileBucketCount + cub::DeviceScan + a host copy of the
// total + perBucketRange (render.cu:13-49, 418-434).
// Bucket bookkeeping (FB render.cu:418-433 counts buckets per tile, scans them
// with CUB and copies the total to the host): per tile ceil(n / bs) buckets, their
// inclusive offsets, and the owning tile of every bucket.  Two launches, no
// host read: k_bucket_count scans 1024 tiles per block, k_bucket_fill adds
// the preceding blocks' totals and writes the bucket -> tile table.
__device__ __forceinline__ uint32_t tile_buckets(const uint32_t* __restrict__ ranges, int t, int bs) {
  return (ranges[2 * t + 1] - ranges[2 * t] + (uint32_t)bs - 1) / (uint32_t)bs;
}

__global__ void __launch_bounds__(kScanTiles) k_bucket_count(int T, const uint32_t* __restrict__ ranges, int bs,
                                                             uint32_t* __restrict__ bucket_off,
                                                             uint32_t* __restrict__ block_sums) {
  __shared__ uint32_t s_warp[kScanTiles / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int t = blockIdx.x * kScanTiles + tid;
  const uint32_t nb = t < T ? tile_buckets(ranges, t, bs) : 0u;
  uint32_t incl = nb;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += u;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = s_warp[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += u;
    }
    s_warp[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  incl += warp ? s_warp[warp - 1] : 0u;
  if (t < T) bucket_off[t] = incl;
  if (tid == kScanTiles - 1) block_sums[blockIdx.x] = incl;
}

__global__ void __launch_bounds__(kScanTiles) k_bucket_fill(int T, const uint32_t* __restrict__ ranges, int bs,
                                                            long long max_buckets, uint32_t* __restrict__ bucket_off,
                                                            const uint32_t* __restrict__ block_sums,
                                                            uint32_t* __restrict__ bucket_tile,
                                                            uint32_t* bucket_sum) {
  __shared__ uint32_t s_base;
  const int tid = threadIdx.x;
  if (tid < 32) {
    uint32_t acc = 0;
    for (int j = tid; j < (int)blockIdx.x; j += 32) acc += block_sums[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (tid == 0) {
      s_base = acc;
      if (blockIdx.x == gridDim.x - 1) {
        const uint32_t total = acc + block_sums[blockIdx.x];
        bucket_sum[0] = (uint32_t)min((long long)total, max_buckets);
        bucket_sum[1] = total;
        bucket_sum[2] = 0;  // forward work cursor
        if ((long long)total > max_buckets) raise_error(kErrCapacity);
      }
    }
  }
  __syncthreads();
  const int t = blockIdx.x * kScanTiles + tid;
  if (t >= T) return;
  const uint32_t nb = tile_buckets(ranges, t, bs);
  const uint32_t end = bucket_off[t] + s_base;
  bucket_off[t] = end;
  for (uint32_t j = end - nb; j < end; ++j)
    if ((long long)j < max_buckets) bucket_tile[j] = (uint32_t)t;
}

struct FwdArgs {
  Views views;
  const float* splat;
  const uint32_t* vals;
  const uint32_t* ranges;
  const uint32_t* bucket_tile;
  const uint32_t* bucket_off;
  uint32_t* bucket_sum;
  float4* samples;
  int bs;
};

template <int BX>
__global__ void __launch_bounds__(kFwdWarps * kWarp, 8) k_render_fwd(const FwdArgs a) {
  using M = TileMap<BX>;
  constexpr int BY = kTilePixels / BX;
  __shared__ BucketStage s_stage[kFwdWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  BucketStage& st = s_stage[warp];
  const int B = (int)a.bucket_sum[0];
  for (int b = next_bucket(a.bucket_sum + 2, lane); b < B;) {
    const int b_next = next_bucket(a.bucket_sum + 2, lane);
    const BucketInfo bi = bucket_info(b, a.bucket_tile, a.bucket_off, a.ranges, a.bs);
    const ViewDesc& cam = a.views.v[a.views.of_tile((uint32_t)bi.tile)];
    const int lt = bi.tile - (int)cam.tile_off;  // tile index inside its view
    const int tx0 = (lt % cam.gx) * BX, ty0 = (lt / cam.gx) * BY;
    stage_bucket<BX>(st, a.splat, a.vals + bi.start, bi.n, lane, tx0, ty0);
    float pxc[M::kCols], pyr[M::kRows];
#pragma unroll
    for (int c = 0; c < M::kCols; ++c) pxc[c] = (float)(tx0 + 8 * c + (lane & 7));
#pragma unroll
    for (int r = 0; r < M::kRows; ++r) pyr[r] = (float)(ty0 + 4 * r + (lane >> 3));
    float T[kPxPerThread], Cr[kPxPerThread], Cg[kPxPerThread], Cb[kPxPerThread];
#pragma unroll
    for (int k = 0; k < kPxPerThread; ++k) { T[k] = 1.f; Cr[k] = 0.f; Cg[k] = 0.f; Cb[k] = 0.f; }
    for (int g = 0; g < bi.n; ++g) {
      const uint32_t mask = st.mask[g];
      if (mask == 0) continue;  // alpha < 1/256 on the whole tile
      const float4 pos = st.pos[g];
      const float4 q = st.quad[g];   // A1, P, C1, log2 o
      const float4 c = st.rgb[g];
      float dx[M::kCols];
#pragma unroll
      for (int cc = 0; cc < M::kCols; ++cc) dx[cc] = centre_offset(pos.x, pos.z, pxc[cc]);
#pragma unroll
      for (int r = 0; r < M::kRows; ++r) {
        const uint32_t rm = (mask >> (r * M::kCols)) & ((1u << M::kCols) - 1u);
        if (rm == 0) continue;
        const float dy = centre_offset(pos.y, pos.w, pyr[r]);
        const float f = fmaf(q.z * dy, dy, q.w);  // log2 o + C1 dy^2
#pragma unroll
        for (int cc = 0; cc < M::kCols; ++cc) {
          if (!((rm >> cc) & 1u)) continue;
          const int k = r * M::kCols + cc;
          // alpha = o * exp(-q/2) = 2^(log2 o + A1 (dx + P dy)^2 + C1 dy^2)
          const float w = fmaf(q.y, dy, dx[cc]);
          const float e = fmaf(q.x * w, w, f);
          float al = fminf(kAlphaMax, ex2_approx(e));
          al = al < kAlphaCut ? 0.f : al;
          const float wt = al * T[k];
          Cr[k] = fmaf(c.x, wt, Cr[k]);
          Cg[k] = fmaf(c.y, wt, Cg[k]);
          Cb[k] = fmaf(c.z, wt, Cb[k]);
          T[k] = fmaf(-al, T[k], T[k]);  // T (1 - alpha), rounded once
        }
      }
    }
    __syncwarp();
    float4* out = a.samples + (size_t)b * kTilePixels;
#pragma unroll
    for (int r = 0; r < M::kRows; ++r)
#pragma unroll
      for (int cc = 0; cc < M::kCols; ++cc) {
        const int k = r * M::kCols + cc;
        out[M::pix(r, cc, lane)] = make_float4(Cr[k], Cg[k], Cb[k], T[k]);
      }
    b = b_next;
  }
}

struct MergeArgs {
  Views views;
  const uint32_t* ranges;
  const uint32_t* bucket_off;
  const uint32_t* bucket_sum;
  float4* samples;
  float* out_color;     // per view (3, H, W), view k at 3 * pix_off
  float* pix_color;     // same layout, without background
  int* last_contrib;    // per view (H, W), view k at pix_off
  float* Ts_final;
  uint32_t* max_contrib;
  int bs;
};

// Per pixel: fold the tile's buckets front to back, storing the running
// prefix in place (FB mergeResults, render.cu:285-391).
__global__ void __launch_bounds__(kTilePixels) k_merge(const MergeArgs a) {
  __shared__ uint32_t s_max[kTilePixels / kWarp];
  const int tile = blockIdx.x, p = threadIdx.x;
  const ViewDesc& cam = a.views.v[a.views.of_tile((uint32_t)tile)];
  const int lt = tile - (int)cam.tile_off, bx = a.views.bx, by = a.views.by;
  const int px = (lt % cam.gx) * bx + p % bx, py = (lt / cam.gx) * by + p / bx;
  const bool in = px < cam.W && py < cam.H;
  // bucket_sum[0] is the bucket count clamped to the sample capacity.
  const int cap = (int)a.bucket_sum[0];
  const int first = min(cap, tile ? (int)a.bucket_off[tile - 1] : 0);
  const int last = min(cap, (int)a.bucket_off[tile]);
  const int rs = (int)a.ranges[2 * tile], re = (int)a.ranges[2 * tile + 1];
  float T = 1.f, Cr = 0.f, Cg = 0.f, Cb = 0.f;
  uint32_t contrib = 0;
  if (in) {
    float4* s = a.samples + (size_t)first * kTilePixels + p;
    float4 cur = first < last ? s[0] : make_float4(0.f, 0.f, 0.f, 1.f);
    for (int b = first; b < last; ++b) {
      const float4 nxt = (b + 1 < last) ? s[kTilePixels] : cur;
      Cr = fmaf(T, cur.x, Cr);
      Cg = fmaf(T, cur.y, Cg);
      Cb = fmaf(T, cur.z, Cb);
      T *= cur.w;
      *s = make_float4(Cr, Cg, Cb, T);
      contrib += (uint32_t)min(a.bs, re - (rs + (b - first) * a.bs));
      if (T < kTMin) break;
      cur = nxt;
      s += kTilePixels;
    }
    const size_t HW = (size_t)cam.W * cam.H;
    const size_t pix = (size_t)py * cam.W + px;
    a.last_contrib[cam.pix_off + pix] = (int)contrib;
    a.Ts_final[cam.pix_off + pix] = T;
    float* oc = a.out_color + 3 * (size_t)cam.pix_off;
    float* pc = a.pix_color + 3 * (size_t)cam.pix_off;
    oc[pix] = Cr + T * cam.bg[0];
    oc[HW + pix] = Cg + T * cam.bg[1];
    oc[2 * HW + pix] = Cb + T * cam.bg[2];
    pc[pix] = Cr;
    pc[HW + pix] = Cg;
    pc[2 * HW + pix] = Cb;
  }
  const uint32_t m = __reduce_max_sync(0xffffffffu, contrib);
  if ((p & 31) == 0) s_max[p >> 5] = m;
  __syncthreads();
  if (p == 0) {
    uint32_t mm = 0;
    for (int w = 0; w < kTilePixels / kWarp; ++w) mm = max(mm, s_max[w]);
    a.max_contrib[tile] = mm;
  }
}


}  // namespace
}  // namespace fgs

FGS_DEFINE_ERROR_ACCESSOR(render)

namespace fgs {
fgs_status run_tile_ranges(int64_t n_cap, const int32_t* n_dev, uint32_t tiles, const uint64_t* keys_sorted,
                           uint32_t* ranges, cudaStream_t s) {
  FGS_TRY(cudaMemsetAsync(ranges, 0, sizeof(uint32_t) * 2 * (size_t)tiles, s));
  if (n_cap > 0) {
    KernelTimer kt__(FGS_K_TILE_RANGES, s);
    k_tile_ranges<<<(unsigned)((n_cap + 255) / 256), 256, 0, s>>>(
        reinterpret_cast<const unsigned long long*>(keys_sorted), n_cap, n_dev, tiles, ranges);
    kt__.stop();
    FGS_LAUNCH_CHECK();
  }
  return FGS_OK;
}

fgs_status run_render_fwd(const Views& views, int64_t n_cap, const int32_t* n_dev, int bucket_size,
                          const float* splat, const uint64_t* keys_sorted, const uint32_t* values_sorted,
                          uint32_t* ranges, float* out_color, int32_t* last_contributor, float* Ts_final,
                          const ImageState& im, const SampleState& sm, int64_t max_buckets, cudaStream_t s) {
  fgs_status st = run_tile_ranges(n_cap, n_dev, views.tiles, keys_sorted, ranges, s);
  if (st != FGS_OK) return st;
  {
    KernelTimer kt__(FGS_K_BUCKET_SETUP, s);
    const unsigned nblk = (views.tiles + kScanTiles - 1) / kScanTiles;
    k_bucket_count<<<nblk, kScanTiles, 0, s>>>((int)views.tiles, ranges, bucket_size, im.bucket_off,
                                               im.block_sums);
    k_bucket_fill<<<nblk, kScanTiles, 0, s>>>((int)views.tiles, ranges, bucket_size, max_buckets, im.bucket_off,
                                              im.block_sums, sm.bucket_tile, im.bucket_sum);
    kt__.stop();
  }
  FGS_LAUNCH_CHECK();
  FwdArgs fa{views, splat, values_sorted, ranges, sm.bucket_tile, im.bucket_off, im.bucket_sum, sm.samples,
             bucket_size};
  {
    KernelTimer kt__(FGS_K_RENDER_FWD, s);
    const int nt = kFwdWarps * kWarp;
    if (views.bx == 8) k_render_fwd<8><<<num_sms() * resident_blocks(k_render_fwd<8>, nt, 0), nt, 0, s>>>(fa);
    else if (views.bx == 16) k_render_fwd<16><<<num_sms() * resident_blocks(k_render_fwd<16>, nt, 0), nt, 0, s>>>(fa);
    else k_render_fwd<32><<<num_sms() * resident_blocks(k_render_fwd<32>, nt, 0), nt, 0, s>>>(fa);
    kt__.stop();
  }
  FGS_LAUNCH_CHECK();
  MergeArgs ma{views, ranges, im.bucket_off, im.bucket_sum, sm.samples, out_color, im.pix_color, last_contributor,
               Ts_final, im.max_contrib, bucket_size};
  {
    KernelTimer kt__(FGS_K_MERGE, s);
    k_merge<<<views.tiles, kTilePixels, 0, s>>>(ma);
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
  // Every tile wastes at most one partially filled bucket.
  return (num_rendered + bucket_size - 1) / bucket_size + std::min<int64_t>(T, num_rendered);
}

extern "C" fgs_status fgs_state_bytes(int width, int height, int block_x, int block_y, int64_t max_buckets,
                                      size_t* image_bytes, size_t* sample_bytes) {
  if (width <= 0 || height <= 0 || block_x <= 0 || block_y <= 0 || max_buckets < 0) return FGS_ERR_BAD_ARG;
  const size_t T = (size_t)((width + block_x - 1) / block_x) * ((height + block_y - 1) / block_y);
  if (image_bytes) *image_bytes = carve_image(nullptr, (size_t)width * height, T).bytes;
  if (sample_bytes) *sample_bytes = carve_sample(nullptr, std::max<int64_t>(max_buckets, 1)).bytes;
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
  const SampleState sm = carve_sample(sample_state, std::max<int64_t>(max_buckets, 1));
  if (image_bytes < im.bytes || sample_bytes < sm.bytes) return FGS_ERR_CAPACITY;
  cudaStream_t s = (cudaStream_t)stream;
  const fgs_status st = run_render_fwd(views, num_rendered, nullptr, bucket_size, splat_buffer, keys_sorted,
                                       values_sorted, ranges, out_color, last_contributor, Ts_final, im, sm,
                                       max_buckets, s);
  if (st != FGS_OK) return st;
  if (bucket_sum_host) {
    uint32_t hs[2] = {0, 0};
    FGS_TRY(cudaMemcpyAsync(hs, im.bucket_sum, sizeof(hs), cudaMemcpyDeviceToHost, s));
    FGS_TRY(cudaStreamSynchronize(s));
    *bucket_sum_host = hs[1];
    if ((int64_t)hs[1] > max_buckets) return FGS_ERR_CAPACITY;
  }
  return FGS_OK;
}
