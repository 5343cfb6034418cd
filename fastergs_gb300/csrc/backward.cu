// Backward pass, sm_103a: bucket-parallel composite backward and the fused
// per-Gaussian backward of projection, EWA covariance, SH and scale/rotation.
//
// Restates FB csrc/cuda_rasterizer/backward.cu with these GB300 changes:
//   * a bucket is walked front to back from the merge's prefix (C, T) before
//     the bucket, so transmittance is recomputed by multiplication instead of
//     FB's repeated division T / (1 - alpha) walking back to front; the colour
//     behind a Gaussian is C_final - prefix, exactly FB's res_ar;
//   * a pixel/Gaussian pair with alpha = 0 contributes nothing and is skipped;
//   * the eleven per-Gaussian partial sums of a warp are reduced with a
//     transpose-reduce (16 shuffles instead of 55) and land with one 12-lane
//     reduction store into an interleaved 48-byte gradient record, instead of
//     eleven scalar atomics from one lane;
//   * the preprocess backward is one kernel (FB launches two) that also
//     scatters the record into FB's output tensors and accumulates the
//     densification statistics.
#include <type_traits>

#include "render_common.cuh"

namespace fgs {
namespace {

constexpr int kBwdWarps = 4;
// Preprocess backward: Gaussians per block and blocks per SM (128 registers
// a thread; SH rows and dL/dsh staged in 2 x 24 KB of shared memory a block).
constexpr int kPbwdThreads = 128;
constexpr int kPbwdBlocks = 4;

struct BwdArgs {
  Views views;
  const float* splat;
  const uint32_t* vals;
  const uint32_t* ranges;
  const uint2* bucket_queue;
  const uint4* live;
  const uint32_t* bucket_off;
  uint32_t* bucket_sum;
  const uint32_t* max_contrib;
  float4* samples;           // prefix after each bucket, or per tile in recompute mode
  uint32_t* tile_stage;      // recompute mode: buckets folded into the tile's rebuilt prefix
  const float* pix_color;    // per view (3, H, W) at 3 * pix_off
  const float* Ts_final;     // per view (H, W) at pix_off
  const int* last_contrib;
  const float* dL;           // per view (3, H, W) at 3 * pix_off
  float* grad;               // gradient record per (view, Gaussian) record
  int bs;
};

// Sum 12 per-lane values over the warp by recursive halving with a
// transpose (exchanges of 6, 3, 2, 1 and 1 values).  On return lane l holds
// the total of value (d + 2c) + 3b + 6a, with a, b, c, d bits 4, 3, 2, 1 of
// l; lanes with c = d = 1 hold a zero pad (warp_value_of).
__device__ __forceinline__ float warp_transpose_reduce12(float (&v)[12], int lane) {
  {
    const bool hi = lane & 16;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const float send = hi ? v[j] : v[j + 6];
      const float keep = hi ? v[j + 6] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
  }
  {
    const bool hi = lane & 8;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float send = hi ? v[j] : v[j + 3];
      const float keep = hi ? v[j + 3] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
  }
  {
    const bool hi = lane & 4;
    const float s0 = hi ? v[0] : v[2], k0 = hi ? v[2] : v[0];
    const float s1 = hi ? v[1] : 0.f, k1 = hi ? 0.f : v[1];  // slot 3 is the pad
    v[0] = k0 + __shfl_xor_sync(0xffffffffu, s0, 4);
    v[1] = k1 + __shfl_xor_sync(0xffffffffu, s1, 4);
  }
  const bool hi = lane & 2;
  const float send = hi ? v[0] : v[1];
  const float keep = hi ? v[1] : v[0];
  const float r = keep + __shfl_xor_sync(0xffffffffu, send, 2);
  return r + __shfl_xor_sync(0xffffffffu, r, 1);
}

// The value warp_transpose_reduce12 leaves in `lane`, or -1 for a pad lane.
__device__ __forceinline__ int warp_value_of(int lane) {
  const int a = (lane >> 4) & 1, b = (lane >> 3) & 1, c = (lane >> 2) & 1, d = (lane >> 1) & 1;
  return (c && d) ? -1 : (d + 2 * c) + 3 * b + 6 * a;
}

// The backward's work list in store mode: the forward's queue without the
// buckets that no pixel reaches (past the tile's last contributor; ~3 in 4 at
// C2), each entry holding what the backward needs to start the bucket, so a
// warp pays one prefetched load per bucket instead of a chain of dependent
// reads per queue slot.  Order: the queue's, warp by warp.
__global__ void __launch_bounds__(256) k_live_buckets(uint32_t* bucket_sum, const uint2* __restrict__ queue,
                                                      const uint32_t* __restrict__ bucket_off,
                                                      const uint32_t* __restrict__ ranges,
                                                      const uint32_t* __restrict__ max_contrib, int bs,
                                                      uint4* __restrict__ live) {
  pdl_wait();  // the preceding kernel of the stream is done
  pdl_trigger();
  const int q = blockIdx.x * 256 + threadIdx.x, lane = threadIdx.x & 31;
  const int B = (int)bucket_sum[0];
  bool keep = false;
  uint4 e = make_uint4(0u, 0u, 0u, 0u);
  if (q < B) {
    const BucketInfo bi = bucket_info(queue[q], bucket_off, ranges, bs);
    keep = (uint32_t)(bi.local * bs) < max_contrib[bi.tile];
    e = make_uint4((uint32_t)bi.b, (uint32_t)bi.tile, (uint32_t)bi.start, ((uint32_t)bi.local << 8) | (uint32_t)bi.n);
  }
  const uint32_t m = __ballot_sync(0xffffffffu, keep);
  if (m == 0u) return;  // warp-uniform
  const int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(bucket_sum + 5, (uint32_t)__popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (keep) live[base + __popc(m & lanemask_lt())] = e;
}

// ABS: also sum |dL/dmean2D| per Gaussian (dmean2D.zw, for the
// xyz_gradient_accum_abs statistic); without it those two slots stay zero.
template <int BX, bool RECOMPUTE, bool ABS>
__global__ void __launch_bounds__(kBwdWarps * kWarp, 6) k_render_bwd(const BwdArgs a) {
  pdl_wait();  // the preceding kernel of the stream is done
  pdl_trigger();
  using M = TileMap<BX>;
  constexpr int BY = kTilePixels / BX;
  __shared__ BucketStage s_stage[kBwdWarps];
  // Per pixel (slot k * 32 + lane): dL/dpixel rgb and K, read once per
  // evaluation with one 16-byte load instead of holding 32 registers.
  __shared__ float4 s_lk[kBwdWarps][kTilePixels];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  BucketStage& st = s_stage[warp];
  const int B = (int)a.bucket_sum[RECOMPUTE ? 0 : 5];
  const int vid = warp_value_of(lane);  // value a lane holds after the transpose reduction

  // Store mode: the live-bucket list (k_live_buckets), one 16-byte entry per
  // bucket, the next entry loaded while the current bucket is processed.
  // Recompute mode: the forward's queue order (round by round), so that a
  // tile's bucket k is always handed out after bucket k-1.
  int q = next_bucket(a.bucket_sum + 3, lane), q_next = 0;
  uint4 e_cur = make_uint4(0u, 0u, 0u, 0u), e_next = e_cur;
  if (!RECOMPUTE && q < B) e_cur = a.live[q];
  for (; q < B; q = q_next, e_cur = e_next) {
    q_next = next_bucket(a.bucket_sum + 3, lane);
    if (!RECOMPUTE && q_next < B) e_next = a.live[q_next];
    int b;
    BucketInfo bi;
    if (RECOMPUTE) {
      bi = bucket_info(a.bucket_queue[q], a.bucket_off, a.ranges, a.bs);
      b = bi.b;
    } else {
      b = (int)e_cur.x;
      bi.tile = (int)e_cur.y;
      bi.start = (int)e_cur.z;
      bi.local = (int)(e_cur.w >> 8);
      bi.n = (int)(e_cur.w & 0xffu);
    }
    const uint32_t thres = (uint32_t)(bi.local * a.bs);
    if (RECOMPUTE && thres >= a.max_contrib[bi.tile]) {  // no pixel of the tile reaches this bucket
      q = q_next;
      continue;
    }
    const ViewDesc& cam = a.views.v[a.views.of_tile((uint32_t)bi.tile)];
    const int lt = bi.tile - (int)cam.tile_off;  // tile index inside its view
    const int tx0 = (lt % cam.gx) * BX, ty0 = (lt / cam.gx) * BY;
    const int HW = cam.W * cam.H;
    const float* dL = a.dL + 3 * (size_t)cam.pix_off;
    const float* pcol = a.pix_color + 3 * (size_t)cam.pix_off;
    const float* Tfin = a.Ts_final + cam.pix_off;
    const int* lcon = a.last_contrib + cam.pix_off;
    const float bgr = cam.bg[0], bgg = cam.bg[1], bgb = cam.bg[2];
    // Scale applied after the reduction to the value a lane ends up holding:
    // mean2D x/|x| need ln2 * W/2, y/|y| ln2 * H/2 (NDC), conic -0.5
    // (ln2 * -0.5 log2e), colour 1, opacity ln2 * log2e / o = 1 / o (per Gaussian).
    // Colour (8..10) is accumulated negated.
    const float vscale = (vid == 0 || vid == 2)   ? kLn2 * 0.5f * (float)cam.W
                         : (vid == 1 || vid == 3) ? kLn2 * 0.5f * (float)cam.H
                         : (vid >= 4 && vid <= 7) ? -0.5f
                         : (vid >= 8 && vid <= 10) ? -1.0f
                                                   : 1.0f;
    stage_bucket<BX>(st, a.splat, load_stage_ids(a.vals + bi.start, bi.n, lane), bi.n, lane, tx0, ty0);
    float pxc[M::kCols], pyr[M::kRows];
#pragma unroll
    for (int c = 0; c < M::kCols; ++c) pxc[c] = (float)(tx0 + 8 * c + (lane & 7));
#pragma unroll
    for (int r = 0; r < M::kRows; ++r) pyr[r] = (float)(ty0 + 4 * r + (lane >> 3));

    // Prefix (C, T) before this bucket for the pixels it reaches, and which of
    // them also reach the next bucket.
    float4* slot = a.samples + (size_t)(RECOMPUTE ? bi.tile : b) * kTilePixels;
    const float4* prev = RECOMPUTE ? slot : a.samples + (size_t)(b - 1) * kTilePixels;
    if (RECOMPUTE && bi.local > 0) wait_stage(a.tile_stage + bi.tile, (uint32_t)bi.local, lane);
    float4 pre[kPxPerThread];
    uint32_t alive = 0, cont = 0;
#pragma unroll
    for (int r = 0; r < M::kRows; ++r)
#pragma unroll
      for (int cc = 0; cc < M::kCols; ++cc) {
        const int k = r * M::kCols + cc;
        const int gxp = (int)pxc[cc], gyp = (int)pyr[r];
        pre[k] = make_float4(0.f, 0.f, 0.f, 1.f);
        if (gxp < cam.W && gyp < cam.H) {
          const uint32_t lc = (uint32_t)lcon[gyp * cam.W + gxp];
          if (lc > thres) {
            alive |= 1u << k;
            if (RECOMPUTE && lc > thres + (uint32_t)bi.n) cont |= 1u << k;
            if (bi.local > 0) pre[k] = __ldcg(prev + M::pix(r, cc, lane));
          }
        }
      }
    if (RECOMPUTE) {
      // Rebuild this bucket's prefix for the pixels that go on, exactly as the
      // forward folded it, and hand it to the tile's next bucket before the
      // gradient work starts.
      uint32_t cont_sb = 0;
#pragma unroll
      for (int k = 0; k < kPxPerThread; ++k)
        if (__any_sync(0xffffffffu, (cont >> k) & 1u)) cont_sb |= 1u << k;
      if (cont_sb != 0u) {
        float Tl[kPxPerThread], Crl[kPxPerThread], Cgl[kPxPerThread], Cbl[kPxPerThread];
        composite_bucket<BX>(st, bi.n, cont_sb, pxc, pyr, Tl, Crl, Cgl, Cbl);
#pragma unroll
        for (int r = 0; r < M::kRows; ++r)
#pragma unroll
          for (int cc = 0; cc < M::kCols; ++cc) {
            const int k = r * M::kCols + cc;
            if ((cont >> k) & 1u)
              slot[M::pix(r, cc, lane)] = make_float4(fmaf(pre[k].w, Crl[k], pre[k].x),
                                                      fmaf(pre[k].w, Cgl[k], pre[k].y),
                                                      fmaf(pre[k].w, Cbl[k], pre[k].z), pre[k].w * Tl[k]);
          }
      }
      publish_stage(a.tile_stage + bi.tile, (uint32_t)bi.local + 1u, lane);
    }

    // Per pixel pair j (slots 2j, 2j + 1): transmittance and prefix . dL
    // packed, and in shared memory (dL.r, dL.g | dL.b, K) of both pixels as
    // two float4 so that every pair half lands in a register pair.
    constexpr int kPairs = kPxPerThread / 2;
    f2x T2[kPairs], Pd2[kPairs];
    float4* lk = s_lk[warp];
    {
      float Tk[kPxPerThread], Pk[kPxPerThread], lx[kPxPerThread], ly[kPxPerThread], lz[kPxPerThread],
          kk[kPxPerThread];
#pragma unroll
      for (int r = 0; r < M::kRows; ++r)
#pragma unroll
        for (int cc = 0; cc < M::kCols; ++cc) {
          const int k = r * M::kCols + cc;
          const int gxp = (int)pxc[cc], gyp = (int)pyr[r];
          Tk[k] = 0.f; Pk[k] = 0.f; lx[k] = 0.f; ly[k] = 0.f; lz[k] = 0.f; kk[k] = 0.f;
          if ((alive >> k) & 1u) {
            const int pix = gyp * cam.W + gxp;
            lx[k] = dL[pix];
            ly[k] = dL[HW + pix];
            lz[k] = dL[2 * HW + pix];
            Tk[k] = pre[k].w;
            Pk[k] = pre[k].x * lx[k] + pre[k].y * ly[k] + pre[k].z * lz[k];
            // K = C_final . dL + T_final * (bg . dL): everything behind a
            // Gaussian is K - (prefix up to and including it) . dL.
            kk[k] = pcol[pix] * lx[k] + pcol[HW + pix] * ly[k] + pcol[2 * HW + pix] * lz[k] +
                    Tfin[pix] * (bgr * lx[k] + bgg * ly[k] + bgb * lz[k]);
          }
        }
#pragma unroll
      for (int j = 0; j < kPairs; ++j) {
        T2[j] = f2_pack(Tk[2 * j], Tk[2 * j + 1]);
        Pd2[j] = f2_pack(Pk[2 * j], Pk[2 * j + 1]);
        lk[(2 * j) * kWarp + lane] = make_float4(lx[2 * j], lx[2 * j + 1], ly[2 * j], ly[2 * j + 1]);
        lk[(2 * j + 1) * kWarp + lane] = make_float4(lz[2 * j], lz[2 * j + 1], kk[2 * j], kk[2 * j + 1]);
      }
    }
    // sub-blocks with at least one pixel that this bucket reaches
    uint32_t live_sb = 0;
#pragma unroll
    for (int k = 0; k < kPxPerThread; ++k)
      if (__any_sync(0xffffffffu, (alive >> k) & 1u)) live_sb |= 1u << k;
    if (live_sb == 0) {
      __syncwarp();
      q = q_next;
      continue;
    }

    const f2x one2 = f2_pack(1.f, 1.f);
    for (int g = 0; g < bi.n; ++g) {
      const uint32_t mask = st.mask[g] & live_sb;
      if (mask == 0) continue;  // alpha < 1/256 on every reached sub-block: no contribution
      const float4 pos = st.pos[g];
      const float4 q = st.quad[g];   // A1, P, C1, log2 o
      const float4 c = st.rgb[g];
      const f2x A12 = f2_pack(q.x, q.x), A22 = f2_pack(2.f * q.x, 2.f * q.x), P2 = f2_pack(q.y, q.y);
      const f2x nr2 = f2_pack(-c.x, -c.x), ng2 = f2_pack(-c.y, -c.y), nb2 = f2_pack(-c.z, -c.z);
      const float wfrac = fmaf(q.y, pos.w, pos.z);  // P fy + fx (shear_offset)
      const f2x wf2 = f2_pack(wfrac, wfrac);
      float ix[M::kCols];
#pragma unroll
      for (int cc = 0; cc < M::kCols; ++cc) ix[cc] = pos.x - pxc[cc];  // exact
      // Packed accumulators (the two halves are summed after the pixel loop):
      // mean x, y; conic moments w^2, w dy, dy^2; -colour; opacity.
      const f2x z2 = f2_pack(0.f, 0.f);
      f2x V0 = z2, V1 = z2, V4 = z2, V5 = z2, V7 = z2, V8 = z2, V9 = z2, V10 = z2, V11 = z2;
      float v2 = 0.f, v3 = 0.f;
      bool any = false;
      auto pair_step = [&](const int j, auto track) {
        const int k0 = 2 * j, k1 = 2 * j + 1;
        const int r0 = k0 / M::kCols, c0 = k0 % M::kCols, r1 = k1 / M::kCols, c1 = k1 % M::kCols;
        const float iy0 = pos.y - pyr[r0], iy1 = r1 == r0 ? iy0 : pos.y - pyr[r1];  // exact
        const float dy0 = iy0 + pos.w;
        const float dy1 = r1 == r0 ? dy0 : iy1 + pos.w;
        const float f0 = fmaf(q.z * dy0, dy0, q.w);
        const float f1 = r1 == r0 ? f0 : fmaf(q.z * dy1, dy1, q.w);
        const f2x dy2 = f2_pack(dy0, dy1);
        const f2x w2 = f2_add(f2_fma(P2, f2_pack(iy0, iy1), f2_pack(ix[c0], ix[c1])), wf2);  // as the forward
        const f2x e2 = f2_fma(f2_mul(A12, w2), w2, f2_pack(f0, f1));
        float e0, e1;
        f2_unpack(e2, e0, e1);
        // -alpha, 0 below the 1/255 cut (pixels this bucket does not reach
        // have T = dL = K = 0 and contribute nothing either way)
        float n0 = fmaxf(-kAlphaMax, -ex2_approx(e0)), n1 = fmaxf(-kAlphaMax, -ex2_approx(e1));
        n0 = n0 > -kAlphaCut ? 0.f : n0;
        n1 = n1 > -kAlphaCut ? 0.f : n1;
        if constexpr (decltype(track)::value) any |= (n0 != 0.f) | (n1 != 0.f);
        const f2x na2 = f2_pack(n0, n1);
        const float4 la = lk[(2 * j) * kWarp + lane], lb = lk[(2 * j + 1) * kWarp + lane];
        const f2x Lx2 = f2_pack(la.x, la.y), Ly2 = f2_pack(la.z, la.w), Lz2 = f2_pack(lb.x, lb.y),
                  K2 = f2_pack(lb.z, lb.w);
        const f2x nwt2 = f2_mul(na2, T2[j]);                                   // -alpha T
        const f2x ncd2 = f2_fma(nr2, Lx2, f2_fma(ng2, Ly2, f2_mul(nb2, Lz2)));  // -c . dL
        Pd2[j] = f2_fma(nwt2, ncd2, Pd2[j]);
        float o0, o1;
        f2_unpack(f2_add(one2, na2), o0, o1);  // 1 - alpha >= 0.01
        const f2x inv2 = f2_pack(rcp_approx(o0), rcp_approx(o1));
        // -dL/dalpha = T (-c . dL) + (K - Pd) / (1 - alpha)
        const f2x nd2 = f2_fma(inv2, f2_sub(K2, Pd2[j]), f2_mul(T2[j], ncd2));
        T2[j] = f2_fma(na2, T2[j], T2[j]);
        V8 = f2_fma(nwt2, Lx2, V8);
        V9 = f2_fma(nwt2, Ly2, V9);
        V10 = f2_fma(nwt2, Lz2, V10);
        const f2x dp2 = f2_mul(nd2, na2);  // dL/dexponent / ln2
        // d exponent / d(centre x) = 2 A1 w, d / d(centre y) = 2 A1 P w + 2 C1 dy
        if constexpr (ABS) {  // per-pixel terms: their absolute values are summed too
          const f2x gw2 = f2_mul(A22, w2);
          const f2x tx2 = f2_mul(dp2, gw2);
          const f2x ty2 = f2_mul(dp2, f2_fma(gw2, P2, f2_pack(2.f * q.z * dy0, 2.f * q.z * dy1)));
          V0 = f2_add(V0, tx2);
          V1 = f2_add(V1, ty2);
          float tx0, tx1, ty0, ty1;
          f2_unpack(tx2, tx0, tx1);
          f2_unpack(ty2, ty0, ty1);
          v2 += fabsf(tx0) + fabsf(tx1);
          v3 += fabsf(ty0) + fabsf(ty1);
          V4 = f2_fma(dp2, f2_mul(w2, w2), V4);
          V5 = f2_fma(f2_mul(dp2, w2), dy2, V5);
          V7 = f2_fma(f2_mul(dp2, dy2), dy2, V7);
        } else {
          // Both mean terms are linear in sum(dp w) and sum(dp dy) (scaled after
          // the loop), the products the conic moments below need anyway.
          const f2x u2 = f2_mul(dp2, w2);
          const f2x t2 = f2_mul(dp2, dy2);
          V0 = f2_add(V0, u2);
          V1 = f2_add(V1, t2);
          V4 = f2_fma(u2, w2, V4);
          V5 = f2_fma(u2, dy2, V5);
          V7 = f2_fma(t2, dy2, V7);
        }
        // (V4, V5, V7: conic-gradient moments in the exponent's own frame
        // (w, dy), w = dx + P dy.  In pixel coordinates a thin footprint's
        // cross-axis gradient is a small difference of large sums; here each
        // frame axis is summed on its own.)
        V11 = f2_add(V11, dp2);
      };
      // Every pixel pair has a sub-block the Gaussian reaches (the common case
      // for large footprints): the four pair chains run without per-pair
      // branches, so they interleave; otherwise pairs without one are skipped.
      if (((mask | (mask >> 1)) & 0x55u) == 0x55u) {
#pragma unroll
        for (int j = 0; j < kPairs; ++j) pair_step(j, std::false_type{});
        // no per-pixel contribution test here: a lane whose alphas were all cut
        // holds exact zeros, so the reduction below then only adds zeros
        any = true;
      } else {
#pragma unroll
        for (int j = 0; j < kPairs; ++j)
          if (((mask >> (2 * j)) & 3u) != 0u) pair_step(j, std::true_type{});
      }
      if (__any_sync(0xffffffffu, any)) {
        float v[12], a0, a1;
        f2_unpack(V0, a0, a1); v[0] = a0 + a1;
        f2_unpack(V1, a0, a1); v[1] = a0 + a1;
        if constexpr (!ABS) {  // from sum(dp w), sum(dp dy): 2 A1 sum(dp w), P (that) + 2 C1 sum(dp dy)
          v[0] *= 2.f * q.x;
          v[1] = fmaf(q.y, v[0], 2.f * q.z * v[1]);
        }
        v[2] = v2;
        v[3] = v3;
        f2_unpack(V4, a0, a1); v[4] = a0 + a1;
        f2_unpack(V5, a0, a1); v[5] = a0 + a1;
        v[6] = 0.f;
        f2_unpack(V7, a0, a1); v[7] = a0 + a1;
        f2_unpack(V8, a0, a1); v[8] = a0 + a1;   // -dL/dcolour
        f2_unpack(V9, a0, a1); v[9] = a0 + a1;
        f2_unpack(V10, a0, a1); v[10] = a0 + a1;
        f2_unpack(V11, a0, a1); v[11] = a0 + a1;
        const float tot = warp_transpose_reduce12(v, lane);
        if (!(lane & 1) && vid >= 0 && vid != 6 && (ABS || (vid != 2 && vid != 3))) {
          const float s = (vid == 11) ? 1.0f / ex2_approx(q.w) : vscale;
          atomicAdd(a.grad + (size_t)__float_as_uint(c.w) * FGS_GRAD_STRIDE + vid, tot * s);
        }
      }
    }
    __syncwarp();
    q = q_next;
  }
}

// One SH basis term: d colour / d coefficient = B, d B / d direction = (bx, by, bz).
// out receives B * drgb (assigned for the first contributing view, added after).
__device__ __forceinline__ void sh_term(float B, float bx, float by, float bz, const float* co, float* out,
                                        float3 drgb, float3& ddir, bool add) {
  out[0] = (add ? out[0] : 0.f) + B * drgb.x;
  out[1] = (add ? out[1] : 0.f) + B * drgb.y;
  out[2] = (add ? out[2] : 0.f) + B * drgb.z;
  const float dot = co[0] * drgb.x + co[1] * drgb.y + co[2] * drgb.z;
  ddir.x = fmaf(bx, dot, ddir.x);
  ddir.y = fmaf(by, dot, ddir.y);
  ddir.z = fmaf(bz, dot, ddir.z);
}

__device__ __forceinline__ float adam_lr(const fgs_adam_fused& ad, int g) {
  return ad.lr ? ad.lr[g] : ad.lr_value[g];
}

// One thread per Gaussian; loops over the views and sums their gradients
// (FB backward.cu:250-539, 892-918 for one view).
// One Gaussian: co / gsh are its SH row and its dL/dsh row (shared memory
// when staged, else global); gsh starts at zero and is accumulated over views.
// Returns whether some view saw the Gaussian (radius > 0).
// Per-Gaussian sums carried from the geometry part of the backward to its SH
// part and outputs.
struct PbwdAcc {
  float m3[3], gc[6], gs[3], gdc[3];
  float dR[3][3];  // dL/dR of the raw quaternion's rotation, summed over views
  float4 gco_sum;
  bool seen;
};

// A Gaussian that no view saw (radius 0 everywhere) has no pairs, so its
// gradient records were zeroed and never added to: every gradient is zero,
// as FB leaves it (its backward returns early for radius 0).  Its outputs are
// written as zeros without reading its parameters or records.
template <bool ADAM, bool GEOM, bool SHFIN>
__device__ __forceinline__ bool pbwd_unseen(const PbwdArgs& a, int i) {
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  if constexpr (GEOM) {
    for (int vi = 0; vi < a.views.V; ++vi) {
      const size_t rid = (size_t)vi * a.P + i;
      if (a.dmean2D) reinterpret_cast<float4*>(a.dmean2D)[rid] = z4;
      if (a.dconic) reinterpret_cast<float4*>(a.dconic)[rid] = z4;
    }
  }
  if constexpr (SHFIN && !ADAM) {  // the fused Adam step leaves unseen rows alone
    if (a.dcolor) {
      a.dcolor[3 * (size_t)i] = 0.f; a.dcolor[3 * (size_t)i + 1] = 0.f; a.dcolor[3 * (size_t)i + 2] = 0.f;
    }
    a.dopac[i] = 0.f;
    a.dmean3D[3 * (size_t)i] = 0.f; a.dmean3D[3 * (size_t)i + 1] = 0.f; a.dmean3D[3 * (size_t)i + 2] = 0.f;
    if (a.dcov3D) {
#pragma unroll
      for (int k = 0; k < 6; ++k) a.dcov3D[6 * (size_t)i + k] = 0.f;
    }
    a.ddc[3 * (size_t)i] = 0.f; a.ddc[3 * (size_t)i + 1] = 0.f; a.ddc[3 * (size_t)i + 2] = 0.f;
    a.dscale[3 * (size_t)i] = 0.f; a.dscale[3 * (size_t)i + 1] = 0.f; a.dscale[3 * (size_t)i + 2] = 0.f;
    reinterpret_cast<float4*>(a.drot)[i] = z4;
  }
  return false;
}

// The backward of one Gaussian over every view, in two parts that can run on
// either side of a block barrier: GEOM (covariance, projection, densification
// statistics; zeroes acc first) and SHFIN (SH, then the rotation and the
// outputs or the fused Adam step).  The staged kernel runs the geometry while
// its SH rows are still being copied into shared memory.  vis: some view saw
// the Gaussian (else pbwd_unseen).
template <bool ADAM, bool GEOM, bool SHFIN>
__device__ __forceinline__ bool pbwd_part(const PbwdArgs& a, int i, bool vis, const float* co, float* gsh,
                                          PbwdAcc& acc) {
  if constexpr (GEOM) acc = PbwdAcc{};
  if (!vis) return pbwd_unseen<ADAM, GEOM, SHFIN>(a, i);
  bool& seen = acc.seen;
  float(&m3)[3] = acc.m3;
  float(&gc)[6] = acc.gc;
  float(&gs)[3] = acc.gs;
  float(&gdc)[3] = acc.gdc;
  float4& gco_sum = acc.gco_sum;
  float gq[4] = {0.f, 0.f, 0.f, 0.f};
  const float3 p = make_float3(a.means[3 * (size_t)i], a.means[3 * (size_t)i + 1], a.means[3 * (size_t)i + 2]);
  // --- rotation of the raw quaternion (FB backward.cu:407-430)
  const float4 q = reinterpret_cast<const float4*>(a.rots)[i];
  const float qr = q.x, qx = q.y, qy = q.z, qz = q.w;
  float R[3][3];
  R[0][0] = 1.f - 2.f * (qy * qy + qz * qz); R[0][1] = 2.f * (qx * qy - qr * qz); R[0][2] = 2.f * (qx * qz + qr * qy);
  R[1][0] = 2.f * (qx * qy + qr * qz); R[1][1] = 1.f - 2.f * (qx * qx + qz * qz); R[1][2] = 2.f * (qy * qz - qr * qx);
  R[2][0] = 2.f * (qx * qz - qr * qy); R[2][1] = 2.f * (qy * qz + qr * qx); R[2][2] = 1.f - 2.f * (qx * qx + qy * qy);
  float(&dR)[3][3] = acc.dR;

  for (int vi = 0; vi < a.views.V; ++vi) {
    const ViewDesc& cam = a.views.v[vi];
    const size_t rid = (size_t)vi * a.P + i;
    const float4* gr = reinterpret_cast<const float4*>(a.grad + rid * FGS_GRAD_STRIDE);
    const float4 gm2 = gr[0], gcn = gr[1], gco = gr[2];
    const int radius = a.radii[rid];
    if constexpr (GEOM) {
    // gcn: -1/2 x the conic-gradient moments sum dp w^2, dp w dy, dp dy^2 in
    // the (w = dx + P dy, dy) frame of the record's exponent.  In pixel
    // coordinates dL/dconic (off-diagonal halved, as FB stores it) is
    // G = Ms S Ms^T with Ms = [[1, -P], [0, 1]].
    const float Pc = radius > 0 ? a.splat[rid * 32 + F_CHOL + 1] : 0.f;
    const float sww = gcn.x, swy = gcn.y, syy = gcn.w;
    const float gz = syy, gy = fmaf(-Pc, syy, swy), gx = fmaf(-Pc, gy, fmaf(-Pc, swy, sww));
    if (a.dmean2D) reinterpret_cast<float4*>(a.dmean2D)[rid] = gm2;
    if (a.dconic) reinterpret_cast<float4*>(a.dconic)[rid] = make_float4(gx, gy, 0.f, gz);
    gco_sum.x += gco.x; gco_sum.y += gco.y; gco_sum.z += gco.z; gco_sum.w += gco.w;
    if (!(radius > 0)) continue;
    seen = true;
    const float sv[3] = {cam.smod * a.scales[3 * (size_t)i], cam.smod * a.scales[3 * (size_t)i + 1],
                         cam.smod * a.scales[3 * (size_t)i + 2]};
    const float s2[3] = {sv[0] * sv[0], sv[1] * sv[1], sv[2] * sv[2]};
    // --- conic -> cov2D -> cov3D / mean (FB backward.cu:250-403)
    const float3 t = xform_point3(cam.view, p);
    const float limx = 1.3f * cam.tanx, limy = 1.3f * cam.tany;
    const float txtz = t.x / t.z, tytz = t.y / t.z;
    const float tx = fminf(limx, fmaxf(-limx, txtz)) * t.z;
    const float ty = fminf(limy, fmaxf(-limy, tytz)) * t.z;
    const float xm = (txtz < -limx || txtz > limx) ? 0.f : 1.f;
    const float ym = (tytz < -limy || tytz > limy) ? 0.f : 1.f;
    const float iz = 1.f / t.z, iz2 = iz * iz, iz3 = iz2 * iz;
    const float j00 = cam.fx * iz, j02 = -cam.fx * tx * iz2, j11 = cam.fy * iz, j12 = -cam.fy * ty * iz2;
    const float* V = cam.view;
    float M0[3], M1[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      M0[b] = j00 * V[b * 4 + 0] + j02 * V[b * 4 + 2];
      M1[b] = j11 * V[b * 4 + 1] + j12 * V[b * 4 + 2];
    }
    const ScreenCov sc2 = screen_cov(M0, M1, R, s2);
    const float idet = 1.f / sc2.det;
    const float ia = sc2.c * idet, ib = -sc2.b * idet, ic = sc2.a * idet;  // C = Sigma2^-1 (the conic)
    // FB divides by den^2 + 1e-7 instead of den^2 (backward.cu:304); keep that factor.
    const float rr = sc2.det * sc2.det / (sc2.det * sc2.det + 0.0000001f);
    // dL/dSigma2 = rr * E with E = -C Gm C.  FB forms E and then projects it on
    // each principal axis N_k (backward.cu:310-347, 445-454), which cancels with
    // the square of the footprint's condition number; here every axis term is
    // formed from v_k = C N_k instead: N_k^T E N_k = -v_k^T Gm v_k.
    float dM0[3] = {0.f, 0.f, 0.f}, dM1[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float v0 = ia * sc2.N0[k] + ib * sc2.N1[k];
      const float v1 = ib * sc2.N0[k] + ic * sc2.N1[k];
      // G v and v^T G v through the moment frame: u = v1 - P v0 is v's
      // second coordinate there, so no large pixel-frame terms cancel.
      const float u = fmaf(-Pc, v0, v1);
      const float h0 = fmaf(sww, v0, swy * u), h1 = fmaf(swy, v0, syy * u);
      const float g0 = fmaf(-Pc, h1, h0), g1 = h1;
      gs[k] += -2.f * sv[k] * rr * fmaf(v0, h0, u * h1);  // w.r.t. the modified scale, as FB returns it
      const float y0 = ia * g0 + ib * g1, y1 = ib * g0 + ic * g1;
      const float f = -2.f * s2[k] * rr;
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        dR[b][k] = fmaf(f, M0[b] * y0 + M1[b] * y1, dR[b][k]);
        dM0[b] = fmaf(f * y0, R[b][k], dM0[b]);
        dM1[b] = fmaf(f * y1, R[b][k], dM1[b]);
      }
    }
    {  // dL/dcov3D in FB's storage (diagonal once, off-diagonal doubled)
      const float c00 = ia * gx + ib * gy, c01 = ia * gy + ib * gz, c10 = ib * gx + ic * gy, c11 = ib * gy + ic * gz;
      const float E00 = -rr * (c00 * ia + c01 * ib), E01 = -rr * (c00 * ib + c01 * ic),
                  E11 = -rr * (c10 * ib + c11 * ic);
      auto G = [&](int r, int c) {
        return M0[r] * M0[c] * E00 + (M0[r] * M1[c] + M1[r] * M0[c]) * E01 + M1[r] * M1[c] * E11;
      };
      gc[0] += G(0, 0); gc[1] += 2.f * G(0, 1); gc[2] += 2.f * G(0, 2);
      gc[3] += G(1, 1); gc[4] += 2.f * G(1, 2); gc[5] += G(2, 2);
    }
    // dL/dJ[a][k] = sum_b dM[a][b] * Rw[k][b], Rw[k][b] = V[b*4 + k]
    const float dJ00 = dM0[0] * V[0] + dM0[1] * V[4] + dM0[2] * V[8];
    const float dJ02 = dM0[0] * V[2] + dM0[1] * V[6] + dM0[2] * V[10];
    const float dJ11 = dM1[0] * V[1] + dM1[1] * V[5] + dM1[2] * V[9];
    const float dJ12 = dM1[0] * V[2] + dM1[1] * V[6] + dM1[2] * V[10];
    const float dtx = xm * -cam.fx * iz2 * dJ02;
    const float dty = ym * -cam.fy * iz2 * dJ12;
    const float dtz = -cam.fx * iz2 * dJ00 - cam.fy * iz2 * dJ11 + 2.f * cam.fx * tx * iz3 * dJ02 +
                      2.f * cam.fy * ty * iz3 * dJ12;
#pragma unroll
    for (int k = 0; k < 3; ++k) m3[k] += V[k * 4 + 0] * dtx + V[k * 4 + 1] * dty + V[k * 4 + 2] * dtz;
    // --- screen-space mean (FB backward.cu:504-526)
    const float4 hp = xform_point4(cam.proj, p);
    const float mw = 1.f / (hp.w + 0.0000001f);
    const float* Pm = cam.proj;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float jx = Pm[4 * k] * mw - Pm[4 * k + 3] * hp.x * mw * mw;
      const float jy = Pm[4 * k + 1] * mw - Pm[4 * k + 3] * hp.y * mw * mw;
      m3[k] += jx * gm2.x + jy * gm2.y;
    }
    } else {  // SH part only: the views that saw the Gaussian
      if (!(radius > 0)) continue;
    }
    // --- SH (FB backward.cu:121-245), only when SH coefficients were given
    if (SHFIN && a.shs) {
      const float* rec = a.splat + rid * 32;
      const float3 drgb = make_float3(gco.x * (1.f - rec[F_CLAMP]), gco.y * (1.f - rec[F_CLAMP + 1]),
                                      gco.z * (1.f - rec[F_CLAMP + 2]));
      const float vx = p.x - cam.campos[0], vy = p.y - cam.campos[1], vz = p.z - cam.campos[2];
      const float n2 = vx * vx + vy * vy + vz * vz, inv_n = rsqrtf(n2);
      const float x = vx * inv_n, y = vy * inv_n, z = vz * inv_n;
      const float c0 = 0.28209479177387814f;
      gdc[0] += c0 * drgb.x; gdc[1] += c0 * drgb.y; gdc[2] += c0 * drgb.z;
      const bool add = true;  // gsh starts at zero
      float3 dd = make_float3(0.f, 0.f, 0.f);
      if (a.D > 0) {
        const float c1 = 0.4886025119029199f;
        sh_term(-c1 * y, 0.f, -c1, 0.f, co + 0, gsh + 0, drgb, dd, add);
        sh_term(c1 * z, 0.f, 0.f, c1, co + 3, gsh + 3, drgb, dd, add);
        sh_term(-c1 * x, -c1, 0.f, 0.f, co + 6, gsh + 6, drgb, dd, add);
        if (a.D > 1) {
          const float k2a = 1.0925484305920792f, k2b = 0.31539156525252005f, k2c = 0.5462742152960396f;
          const float xx = x * x, yy = y * y, zz = z * z;
          sh_term(k2a * x * y, k2a * y, k2a * x, 0.f, co + 9, gsh + 9, drgb, dd, add);
          sh_term(-k2a * y * z, 0.f, -k2a * z, -k2a * y, co + 12, gsh + 12, drgb, dd, add);
          sh_term(k2b * (2.f * zz - xx - yy), -2.f * k2b * x, -2.f * k2b * y, 4.f * k2b * z, co + 15, gsh + 15,
                  drgb, dd, add);
          sh_term(-k2a * x * z, -k2a * z, 0.f, -k2a * x, co + 18, gsh + 18, drgb, dd, add);
          sh_term(k2c * (xx - yy), 2.f * k2c * x, -2.f * k2c * y, 0.f, co + 21, gsh + 21, drgb, dd, add);
          if (a.D > 2) {
            const float ka = 0.5900435899266435f, kb = 2.890611442640554f, kc = 0.4570457994644658f,
                        kd = 0.3731763325901154f, ke = 1.445305721320277f;
            sh_term(-ka * y * (3.f * xx - yy), -ka * 6.f * x * y, -ka * (3.f * xx - 3.f * yy), 0.f, co + 24,
                    gsh + 24, drgb, dd, add);
            sh_term(kb * x * y * z, kb * y * z, kb * x * z, kb * x * y, co + 27, gsh + 27, drgb, dd, add);
            sh_term(-kc * y * (4.f * zz - xx - yy), kc * 2.f * x * y, -kc * (4.f * zz - xx - 3.f * yy),
                    -kc * 8.f * y * z, co + 30, gsh + 30, drgb, dd, add);
            sh_term(kd * z * (2.f * zz - 3.f * xx - 3.f * yy), -kd * 6.f * x * z, -kd * 6.f * y * z,
                    kd * (6.f * zz - 3.f * xx - 3.f * yy), co + 33, gsh + 33, drgb, dd, add);
            sh_term(-kc * x * (4.f * zz - xx - yy), -kc * (4.f * zz - 3.f * xx - yy), kc * 2.f * x * y,
                    -kc * 8.f * x * z, co + 36, gsh + 36, drgb, dd, add);
            sh_term(ke * z * (xx - yy), ke * 2.f * x * z, -ke * 2.f * y * z, ke * (xx - yy), co + 39, gsh + 39,
                    drgb, dd, add);
            sh_term(-ka * x * (xx - 3.f * yy), -ka * (3.f * xx - 3.f * yy), ka * 6.f * x * y, 0.f, co + 42,
                    gsh + 42, drgb, dd, add);
          }
        }
      }
      // d(v / |v|)/dv applied to the direction gradient
      const float vd = vx * dd.x + vy * dd.y + vz * dd.z;
      const float inv3 = inv_n * inv_n * inv_n;
      m3[0] += (dd.x * n2 - vx * vd) * inv3;
      m3[1] += (dd.y * n2 - vy * vd) * inv3;
      m3[2] += (dd.z * n2 - vz * vd) * inv3;
    }
    // --- densification statistics (FB backward.cu:892-918), once per view
    if (GEOM && a.accum) {
      if (a.denom) a.denom[i] += 1.f;
      if (a.max_radii) a.max_radii[i] = fmaxf(a.max_radii[i], (float)radius);
      a.accum[i] += sqrt_approx(gm2.x * gm2.x + gm2.y * gm2.y);
      if (a.accum_abs) a.accum_abs[i] += sqrt_approx(gm2.z * gm2.z + gm2.w * gm2.w);
    }
  }
  if constexpr (!SHFIN) return seen;
  // --- rotation (FB backward.cu:460-482): dL/dq from dL/dR of the raw quaternion
  gq[0] = 2.f * qz * (dR[1][0] - dR[0][1]) + 2.f * qy * (dR[0][2] - dR[2][0]) + 2.f * qx * (dR[2][1] - dR[1][2]);
  gq[1] = 2.f * qy * (dR[0][1] + dR[1][0]) + 2.f * qz * (dR[0][2] + dR[2][0]) + 2.f * qr * (dR[2][1] - dR[1][2]) -
          4.f * qx * (dR[1][1] + dR[2][2]);
  gq[2] = 2.f * qx * (dR[0][1] + dR[1][0]) + 2.f * qr * (dR[0][2] - dR[2][0]) + 2.f * qz * (dR[1][2] + dR[2][1]) -
          4.f * qy * (dR[0][0] + dR[2][2]);
  gq[3] = 2.f * qr * (dR[1][0] - dR[0][1]) + 2.f * qx * (dR[0][2] + dR[2][0]) + 2.f * qy * (dR[1][2] + dR[2][1]) -
          4.f * qz * (dR[0][0] + dR[1][1]);
  if constexpr (ADAM) {
    // --- fused sparse Adam (FB adam.cu:26-37 on the autograd gradients of the
    // raw parameters): only Gaussians some view saw take a step.  Every
    // operand is loaded before the first store so the loads overlap.
    if (!seen) return false;
    const fgs_adam_fused& ad = a.adam;
    constexpr int kE = 14;  // xyz 3, f_dc 3, opacity 1, scaling 3, rotation 4
    constexpr int kGroup[kE] = {FGS_ADAM_XYZ, FGS_ADAM_XYZ, FGS_ADAM_XYZ, FGS_ADAM_F_DC, FGS_ADAM_F_DC,
                                FGS_ADAM_F_DC, FGS_ADAM_OPACITY, FGS_ADAM_SCALING, FGS_ADAM_SCALING,
                                FGS_ADAM_SCALING, FGS_ADAM_ROTATION, FGS_ADAM_ROTATION, FGS_ADAM_ROTATION,
                                FGS_ADAM_ROTATION};
    constexpr int kWidth[kE] = {3, 3, 3, 3, 3, 3, 1, 3, 3, 3, 4, 4, 4, 4};
    constexpr int kCol[kE] = {0, 1, 2, 0, 1, 2, 0, 0, 1, 2, 0, 1, 2, 3};
    float p[kE], m1[kE], m2[kE], g[kE];
#pragma unroll
    for (int e = 0; e < kE; ++e) {
      p[e] = m1[e] = m2[e] = 0.f;
      if (const float* prm = ad.param[kGroup[e]]) {
        const size_t off = (size_t)kWidth[e] * i + kCol[e];
        p[e] = prm[off];
        m1[e] = ad.exp_avg[kGroup[e]][off];
        m2[e] = ad.exp_avg_sq[kGroup[e]][off];
      }
    }
    const bool sig = ad.param[FGS_ADAM_OPACITY] && ad.opacity_act == FGS_ACT_SIGMOID;
    const float y = sig ? a.opac[i] : 0.f;
    const bool ex = ad.param[FGS_ADAM_SCALING] && ad.scaling_act == FGS_ACT_EXP;
    const float e0 = ex ? a.scales[3 * (size_t)i] : 1.f, e1 = ex ? a.scales[3 * (size_t)i + 1] : 1.f,
                e2 = ex ? a.scales[3 * (size_t)i + 2] : 1.f;
    g[0] = m3[0]; g[1] = m3[1]; g[2] = m3[2];
    g[3] = gdc[0]; g[4] = gdc[1]; g[5] = gdc[2];
    g[6] = sig ? gco_sum.w * (1.f - y) * y : gco_sum.w;  // sigmoid'(x) = (1 - y) y, in autograd's order
    g[7] = ex ? gs[0] * e0 : gs[0];                        // exp'(x) = exp(x)
    g[8] = ex ? gs[1] * e1 : gs[1];
    g[9] = ex ? gs[2] * e2 : gs[2];
    g[10] = gq[0]; g[11] = gq[1]; g[12] = gq[2]; g[13] = gq[3];
    if (ad.param[FGS_ADAM_ROTATION] && ad.rotation_act == FGS_ACT_NORMALIZE) {
      // q = x / max(|x|, 1e-12): dL/dx = g / d - x (g . x) / d^3 (the norm's
      // term only where |x| > 1e-12, as the clamp passes it); x = raw row
      const float x0 = p[10], x1 = p[11], x2 = p[12], x3 = p[13];
      const float nrm = sqrtf(x0 * x0 + x1 * x1 + x2 * x2 + x3 * x3);
      const float d = fmaxf(nrm, 1e-12f);
      const float gx = gq[0] * x0 + gq[1] * x1 + gq[2] * x2 + gq[3] * x3;
      const float c = nrm > 1e-12f ? gx / (d * d) / d : 0.f;
      g[10] = gq[0] / d - x0 * c;
      g[11] = gq[1] / d - x1 * c;
      g[12] = gq[2] / d - x2 * c;
      g[13] = gq[3] / d - x3 * c;
    }
#pragma unroll
    for (int e = 0; e < kE; ++e) {
      if (float* prm = ad.param[kGroup[e]]) {
        adam_reg(p[e], m1[e], m2[e], g[e], adam_lr(ad, kGroup[e]), ad.b1, ad.b2, ad.eps[kGroup[e]]);
        const size_t off = (size_t)kWidth[e] * i + kCol[e];
        prm[off] = p[e];
        ad.exp_avg[kGroup[e]][off] = m1[e];
        ad.exp_avg_sq[kGroup[e]][off] = m2[e];
      }
    }
    return true;
  }
  // --- outputs (zeros where no view saw the Gaussian, as FB leaves them);
  // dcolor and dcov3D are optional (only precomputed colours / covariances need them)
  if (a.dcolor) {
    a.dcolor[3 * (size_t)i] = gco_sum.x;
    a.dcolor[3 * (size_t)i + 1] = gco_sum.y;
    a.dcolor[3 * (size_t)i + 2] = gco_sum.z;
  }
  a.dopac[i] = gco_sum.w;
  float* gm = a.dmean3D + 3 * (size_t)i;
  gm[0] = m3[0]; gm[1] = m3[1]; gm[2] = m3[2];
  if (a.dcov3D) {
#pragma unroll
    for (int k = 0; k < 6; ++k) a.dcov3D[6 * (size_t)i + k] = gc[k];
  }
  a.ddc[3 * (size_t)i] = gdc[0]; a.ddc[3 * (size_t)i + 1] = gdc[1]; a.ddc[3 * (size_t)i + 2] = gdc[2];
  a.dscale[3 * (size_t)i] = gs[0]; a.dscale[3 * (size_t)i + 1] = gs[1]; a.dscale[3 * (size_t)i + 2] = gs[2];
  reinterpret_cast<float4*>(a.drot)[i] = make_float4(gq[0], gq[1], gq[2], gq[3]);
  return seen;
}

template <bool ADAM>
__device__ __forceinline__ bool pbwd_gaussian(const PbwdArgs& a, int i, bool vis, const float* co, float* gsh) {
  PbwdAcc acc;
  return pbwd_part<ADAM, true, true>(a, i, vis, co, gsh, acc);
}

// Whether some view saw Gaussian i (radius > 0).  The views' radii are read
// as independent loads (no early exit), so many views cost one latency.
__device__ __forceinline__ bool pbwd_visible(const PbwdArgs& a, int i) {
  bool vis = false;
#pragma unroll 4
  for (int vi = 0; vi < a.views.V; ++vi) vis |= a.radii[(size_t)vi * a.P + i] > 0;
  return vis;
}

// f_rest rows of one block of Gaussians, [first, first + n), row floats each,
// with their summed gradients in shared memory (s_g): the Adam step on the
// rows of Gaussians some view saw, as float4 over the block's contiguous span
// (kRestUnroll float4 per array in flight per thread; a float4 spans at most
// two rows as row >= 3) when the arrays are 16-byte aligned there, else
// element by element.  When the rasterizer's SH input is the f_rest tensor
// itself, the parameter values come from the staged copy (s_co) instead of a
// second read.
constexpr int kRestUnroll = 4;
__device__ __forceinline__ void adam_rest_rows(const PbwdArgs& a, int first, int n, int row, const float* s_co,
                                               const float* s_g, const uint8_t* s_seen) {
  const fgs_adam_fused& ad = a.adam;
  const float lr = adam_lr(ad, FGS_ADAM_F_REST), eps = ad.eps[FGS_ADAM_F_REST], b1 = ad.b1, b2 = ad.b2;
  const size_t base = (size_t)first * row;
  float* prm = ad.param[FGS_ADAM_F_REST] + base;
  float* pm1 = ad.exp_avg[FGS_ADAM_F_REST] + base;
  float* pm2 = ad.exp_avg_sq[FGS_ADAM_F_REST] + base;
  const bool staged = a.shs == ad.param[FGS_ADAM_F_REST];
  const int total = n * row;
  const bool vec = row >= 3 &&
                   ((reinterpret_cast<uintptr_t>(prm) | reinterpret_cast<uintptr_t>(pm1) |
                     reinterpret_cast<uintptr_t>(pm2)) & 15) == 0;
  int done = 0;
  if (vec) {
    const int n4 = total >> 2;
    float4* P4 = reinterpret_cast<float4*>(prm);
    float4* A4 = reinterpret_cast<float4*>(pm1);
    float4* B4 = reinterpret_cast<float4*>(pm2);
    const float4* C4 = reinterpret_cast<const float4*>(s_co);
    const float4* G4 = reinterpret_cast<const float4*>(s_g);
    // Row of element j: floor((j + 1/2) / row) in FP32.  j < kPbwdThreads row and
    // 3 <= row <= 48, so the product is off by less than 5e-4 while the exact
    // quotient stays at least 1 / (2 row) > 0.01 away from an integer
    // (tests/test_capi_cpu.py checks every row and j).
    const float inv_row = 1.f / (float)row;
    for (int q0 = threadIdx.x; q0 < n4; q0 += kPbwdThreads * kRestUnroll) {
      float4 pv[kRestUnroll], av[kRestUnroll], bv[kRestUnroll];
      int r0[kRestUnroll];
      bool s0[kRestUnroll], s1[kRestUnroll];
#pragma unroll
      for (int u = 0; u < kRestUnroll; ++u) {
        const int q = q0 + kPbwdThreads * u, j = 4 * q;
        r0[u] = (int)(((float)j + 0.5f) * inv_row);
        const int r3 = (int)(((float)j + 3.5f) * inv_row);
        s0[u] = q < n4 && s_seen[r0[u]] != 0;
        s1[u] = q < n4 && s_seen[r3] != 0;
        if (s0[u] || s1[u]) {
          pv[u] = staged ? C4[q] : P4[q];
          av[u] = A4[q];
          bv[u] = B4[q];
        }
      }
#pragma unroll
      for (int u = 0; u < kRestUnroll; ++u) {
        if (!(s0[u] || s1[u])) continue;
        const int q = q0 + kPbwdThreads * u, j = 4 * q;
        const int split = (r0[u] + 1) * row - j;  // elements [0, split) belong to row r0
        const float4 gv = G4[q];
        float* pp = &pv[u].x;
        float* pa = &av[u].x;
        float* pb = &bv[u].x;
        const float gg[4] = {gv.x, gv.y, gv.z, gv.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {  // branch-free: step all four, keep the seen rows' results
          float p = pp[e], ma = pa[e], mb = pb[e];
          adam_reg(p, ma, mb, gg[e], lr, b1, b2, eps);
          const bool on = e < split ? s0[u] : s1[u];
          pp[e] = on ? p : pp[e];
          pa[e] = on ? ma : pa[e];
          pb[e] = on ? mb : pb[e];
        }
        P4[q] = pv[u];
        A4[q] = av[u];
        B4[q] = bv[u];
      }
    }
    done = n4 << 2;
  }
  for (int j = done + threadIdx.x; j < total; j += kPbwdThreads)
    if (s_seen[j / row]) adam_step(prm, pm1, pm2, j, s_g[j], lr, b1, b2, eps);
}

// ADAM: the sparse Adam step fused in place of the gradient outputs.
template <bool ADAM>
__global__ void __launch_bounds__(kPbwdThreads, kPbwdBlocks) k_preprocess_bwd(const PbwdArgs a) {
  pdl_wait();  // the preceding kernel of the stream is done
  pdl_trigger();
  // sh_staged: [kPbwdThreads x M x 3] SH rows, then as many dL/dsh accumulators
  extern __shared__ __align__(16) float s_pb[];
  __shared__ uint8_t s_seen[kPbwdThreads];
  const int first = blockIdx.x * kPbwdThreads, n = min(kPbwdThreads, a.P - first), row = a.M * 3;
  const int i = first + threadIdx.x;
  if (a.sh_staged) {
    float* s_co = s_pb;
    float* s_g = s_pb + kPbwdThreads * row;
    const bool vis = i < a.P && pbwd_visible(a, i);
    bool seen;
    if (a.views.V == 1) {
      // one view: only the SH rows of Gaussians it saw are read (at 1M
      // Gaussians in one 1297x840 view, about a third), so only those are
      // copied, and they arrive while the geometry part runs (with many
      // views the geometry alone outlasts the copy, a second walk over the
      // views would cost more than the overlap gains, and nearly every row
      // is seen by some view)
      s_seen[threadIdx.x] = vis ? 1 : 0;
      __syncthreads();
      block_copy_rows_to_smem_async(s_co, a.shs, (size_t)first * row, n, row, s_seen);
      for (int j = threadIdx.x; j < n * row; j += kPbwdThreads) s_g[j] = 0.f;
      PbwdAcc acc;
      const bool active = i < a.P;
      if (active) pbwd_part<ADAM, true, false>(a, i, vis, nullptr, nullptr, acc);
      cp_async_wait_all();
      __syncthreads();
      seen = active && pbwd_part<ADAM, false, true>(a, i, vis, s_co + threadIdx.x * row, s_g + threadIdx.x * row,
                                                    acc);
    } else {
      block_copy_rows_to_smem(s_co, a.shs, (size_t)first * row, n, row, nullptr);
      for (int j = threadIdx.x; j < n * row; j += kPbwdThreads) s_g[j] = 0.f;
      __syncthreads();
      seen = i < a.P && pbwd_gaussian<ADAM>(a, i, vis, s_co + threadIdx.x * row, s_g + threadIdx.x * row);
    }
    s_seen[threadIdx.x] = seen ? 1 : 0;
    __syncthreads();
    if constexpr (!ADAM) {
      block_copy_from_smem(a.dsh, (size_t)first * row, s_g, n * row);
    } else {
      if (a.adam.param[FGS_ADAM_F_REST]) adam_rest_rows(a, first, n, row, s_co, s_g, s_seen);
    }
    return;
  }
  if (i >= a.P) return;
  float* gsh = a.dsh ? a.dsh + (size_t)i * row : nullptr;
  if (gsh)
    for (int k = 0; k < row; ++k) gsh[k] = 0.f;
  pbwd_gaussian<ADAM>(a, i, pbwd_visible(a, i), a.shs ? a.shs + (size_t)i * row : nullptr, gsh);
}

__global__ void __launch_bounds__(256) k_densify(int P, const int* radii, const float4* dm2, float* accum,
                                                 float* accum_abs, float* max_radii, float* denom) {
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= P || !(radii[i] > 0)) return;
  const float4 g = dm2[i];
  if (denom) denom[i] += 1.f;
  if (max_radii) max_radii[i] = fmaxf(max_radii[i], (float)radii[i]);
  if (accum) accum[i] += sqrt_approx(g.x * g.x + g.y * g.y);
  if (accum_abs) accum_abs[i] += sqrt_approx(g.z * g.z + g.w * g.w);
}

}  // namespace
}  // namespace fgs

FGS_DEFINE_ERROR_ACCESSOR(backward)

namespace fgs {
fgs_status run_render_bwd(const Views& views, int64_t records, int bucket_size, const uint32_t* values_sorted,
                          const uint32_t* ranges, const float* splat, const float* Ts_final,
                          const int32_t* last_contributor, const ImageState& im, const SampleState& sm,
                          const float* dL_dpixels, float* grad_record, bool recompute, bool abs_grad,
                          cudaStream_t s) {
  // the gradient records, and the backward work cursor and live-list count
  // (words 3 and 5 of the image-state header): reset on every call, one launch
  {
    const fgs_status z = zero_async(grad_record, sizeof(float) * FGS_GRAD_STRIDE * (size_t)records, s,
                                    im.bucket_sum + 3, 3 * sizeof(uint32_t));
    if (z != FGS_OK) return z;
  }
  // recompute mode rebuilds every tile's prefix from the start
  if (recompute) FGS_TRY(cudaMemsetAsync(im.tile_stage, 0, sizeof(uint32_t) * views.tiles, s));
  const int sub = sub_bucket_size(bucket_size);
  if (!recompute) {
    KernelTimer kt__(FGS_K_BWD_LIST, s);
    const unsigned blocks = (unsigned)((std::max<int64_t>(sm.max_buckets, 1) + 255) / 256);
    (void)launch_pdl(k_live_buckets, dim3(blocks), dim3(256), 0, s, im.bucket_sum, sm.bucket_queue, im.bucket_off,
                     ranges, im.max_contrib, sub, sm.live);
    kt__.stop();
    FGS_LAUNCH_CHECK();
  }
  BwdArgs a{views, splat, values_sorted, ranges, sm.bucket_queue, sm.live, im.bucket_off,
            im.bucket_sum, im.max_contrib, sm.samples, im.tile_stage, im.pix_color, Ts_final, last_contributor,
            dL_dpixels, grad_record, sub};
  {
    KernelTimer kt__(FGS_K_RENDER_BWD, s);
    const int nt = kBwdWarps * kWarp;
    auto launch = [&](auto kernel) {
      (void)launch_pdl(kernel, dim3(num_sms() * resident_blocks(kernel, nt, 0)), dim3(nt), 0, s, a);
    };
    auto by_tile = [&](auto rc, auto ab) {
      constexpr bool R = decltype(rc)::value, A = decltype(ab)::value;
      if (views.bx == 8) launch(k_render_bwd<8, R, A>);
      else if (views.bx == 16) launch(k_render_bwd<16, R, A>);
      else launch(k_render_bwd<32, R, A>);
    };
    using T_ = std::true_type;
    using F_ = std::false_type;
    if (recompute) {
      if (abs_grad) by_tile(T_{}, T_{});
      else by_tile(T_{}, F_{});
    } else {
      if (abs_grad) by_tile(F_{}, T_{});
      else by_tile(F_{}, F_{});
    }
    kt__.stop();
  }
  FGS_LAUNCH_CHECK();
  return FGS_OK;
}

fgs_status run_preprocess_bwd(PbwdArgs& a, cudaStream_t s) {
  a.sh_staged = (a.shs && (a.dsh || a.adam_on) && a.M >= 1 && a.M <= kMaxStagedCoeffs) ? 1 : 0;
  // the fused step keeps dL/dsh only in shared memory
  if (a.adam_on && a.shs && a.D > 0 && !a.sh_staged) return FGS_ERR_BAD_ARG;
  const int dyn = a.sh_staged ? 2 * kPbwdThreads * a.M * 3 * (int)sizeof(float) : 0;
  const void* kern = a.adam_on ? reinterpret_cast<const void*>(&k_preprocess_bwd<true>)
                               : reinterpret_cast<const void*>(&k_preprocess_bwd<false>);
  if (dyn) FGS_TRY(allow_dyn_smem(kern, 2 * kPbwdThreads * kMaxStagedCoeffs * 12));
  KernelTimer kt__(FGS_K_PREPROCESS_BWD, s);
  const unsigned blocks = (unsigned)((a.P + kPbwdThreads - 1) / kPbwdThreads);
  if (a.adam_on) (void)launch_pdl(k_preprocess_bwd<true>, dim3(blocks), dim3(kPbwdThreads), dyn, s, a);
  else (void)launch_pdl(k_preprocess_bwd<false>, dim3(blocks), dim3(kPbwdThreads), dyn, s, a);
  kt__.stop();
  FGS_LAUNCH_CHECK();
  return FGS_OK;
}
}  // namespace fgs

using namespace fgs;

extern "C" fgs_status fgs_render_bwd(int P, int width, int height, int block_x, int block_y, int bucket_size,
                                     const uint32_t* values_sorted, const uint32_t* ranges, const float* bg,
                                     const float* splat_buffer, const float* Ts_final,
                                     const int32_t* last_contributor, const void* image_state,
                                     const void* sample_state, int64_t max_buckets, const float* dL_dpixels,
                                     float* grad_record, int flags, void* stream) {
  if (P < 0 || width <= 0 || height <= 0 || !tile_shape_ok(block_x, block_y) || bucket_size < 1 ||
      bucket_size > kMaxBucket || max_buckets < 0)
    return FGS_ERR_BAD_ARG;
  if (P == 0) return FGS_OK;
  if (!ranges || !bg || !splat_buffer || !Ts_final || !last_contributor || !image_state || !sample_state ||
      !dL_dpixels || !grad_record || !values_sorted)
    return FGS_ERR_BAD_ARG;
  if (((uintptr_t)grad_record & 15) || ((uintptr_t)splat_buffer & 15)) return FGS_ERR_BAD_ARG;
  const Views views = single_view(width, height, block_x, block_y, nullptr, nullptr, nullptr, bg, 1.f, 1.f, 1.f, 1.f);
  const ImageState im = carve_image(const_cast<void*>(image_state), (size_t)width * height, views.tiles);
  const int64_t mb = max_buckets > 0 ? max_buckets : 1;
  const SampleState sm = carve_sample(const_cast<void*>(sample_state), mb, mb);
  return run_render_bwd(views, P, bucket_size, values_sorted, ranges, splat_buffer, Ts_final, last_contributor, im,
                        sm, dL_dpixels, grad_record, false, (flags & FGS_BWD_NO_ABS) == 0, (cudaStream_t)stream);
}

extern "C" fgs_status fgs_preprocess_bwd(
    int P, int D, int M, const float* means3D, const int32_t* radii, const float* dc, const float* shs,
    const float* splat_buffer, const float* scales, const float* rotations, float scale_modifier,
    const float* viewmatrix, const float* projmatrix, int width, int height, float tan_fovx, float tan_fovy,
    const float* campos, const float* grad_record, float* dL_dmean2D, float* dL_dconic, float* dL_dopacity,
    float* dL_dcolor, float* dL_dmean3D, float* dL_dcov3D, float* dL_ddc, float* dL_dsh, float* dL_dscale,
    float* dL_drot, float* xyz_gradient_accum, float* xyz_gradient_accum_abs, float* max_radii, float* denom,
    void* stream) {
  if (P < 0 || D < 0 || D > 3 || M < 0 || width <= 0 || height <= 0) return FGS_ERR_BAD_ARG;
  if (P == 0) return FGS_OK;
  if (!means3D || !radii || !splat_buffer || !scales || !rotations || !viewmatrix || !projmatrix || !grad_record ||
      !dL_dopacity || !dL_dmean3D || !dL_ddc || !dL_dscale || !dL_drot)
    return FGS_ERR_BAD_ARG;
  if (shs && (!dc || !campos || (D > 0 && M < (D + 1) * (D + 1) - 1) || !dL_dsh)) return FGS_ERR_BAD_ARG;
  if (((uintptr_t)grad_record & 15) || ((uintptr_t)dL_dmean2D & 15) || ((uintptr_t)dL_dconic & 15) ||
      ((uintptr_t)rotations & 15) || ((uintptr_t)dL_drot & 15))
    return FGS_ERR_BAD_ARG;
  PbwdArgs a;
  a.views = single_view(width, height, 16, 16, viewmatrix, projmatrix, campos, nullptr, tan_fovx, tan_fovy, 1.f,
                        scale_modifier);
  a.P = P; a.D = D; a.M = M;
  a.means = means3D; a.radii = radii; a.dc = dc; a.shs = shs; a.splat = splat_buffer;
  a.scales = scales; a.rots = rotations; a.grad = grad_record;
  a.dmean2D = dL_dmean2D; a.dconic = dL_dconic; a.dopac = dL_dopacity; a.dcolor = dL_dcolor;
  a.dmean3D = dL_dmean3D; a.dcov3D = dL_dcov3D; a.ddc = dL_ddc; a.dsh = (M > 0) ? dL_dsh : nullptr;
  a.dscale = dL_dscale; a.drot = dL_drot;
  a.accum = xyz_gradient_accum; a.accum_abs = xyz_gradient_accum_abs; a.max_radii = max_radii; a.denom = denom;
  return run_preprocess_bwd(a, (cudaStream_t)stream);
}

bool fgs::adam_args_ok(const fgs_adam_fused* ad, const float* shs, const float* opacities) {
  if (!ad) return false;
  for (int g = 0; g < FGS_ADAM_GROUPS; ++g)
    if (ad->param[g] && (!ad->exp_avg[g] || !ad->exp_avg_sq[g])) return false;
  if (ad->opacity_act != FGS_ACT_IDENTITY && ad->opacity_act != FGS_ACT_SIGMOID) return false;
  if (ad->scaling_act != FGS_ACT_IDENTITY && ad->scaling_act != FGS_ACT_EXP) return false;
  if (ad->rotation_act != FGS_ACT_IDENTITY && ad->rotation_act != FGS_ACT_NORMALIZE) return false;
  if (ad->param[FGS_ADAM_OPACITY] && ad->opacity_act == FGS_ACT_SIGMOID && !opacities) return false;
  if (ad->param[FGS_ADAM_ROTATION] && ((uintptr_t)ad->param[FGS_ADAM_ROTATION] & 15)) return false;
  if (ad->param[FGS_ADAM_F_REST] && !shs) return false;
  return true;
}

extern "C" fgs_status fgs_preprocess_bwd_adam(
    int P, int D, int M, const float* means3D, const int32_t* radii, const float* shs, const float* splat_buffer,
    const float* opacities, const float* scales, const float* rotations, float scale_modifier,
    const float* viewmatrix, const float* projmatrix, int width, int height, float tan_fovx, float tan_fovy,
    const float* campos, const float* grad_record, const fgs_adam_fused* adam, float* xyz_gradient_accum,
    float* xyz_gradient_accum_abs, float* max_radii, float* denom, void* stream) {
  if (P < 0 || D < 0 || D > 3 || M < 0 || width <= 0 || height <= 0) return FGS_ERR_BAD_ARG;
  if (P == 0) return FGS_OK;
  if (!means3D || !radii || !splat_buffer || !scales || !rotations || !viewmatrix || !projmatrix || !grad_record ||
      !adam_args_ok(adam, shs, opacities))
    return FGS_ERR_BAD_ARG;
  if (shs && (!campos || (D > 0 && M < (D + 1) * (D + 1) - 1))) return FGS_ERR_BAD_ARG;
  if (((uintptr_t)grad_record & 15) || ((uintptr_t)rotations & 15)) return FGS_ERR_BAD_ARG;
  PbwdArgs a;
  a.views = single_view(width, height, 16, 16, viewmatrix, projmatrix, campos, nullptr, tan_fovx, tan_fovy, 1.f,
                        scale_modifier);
  a.P = P; a.D = D; a.M = M;
  a.means = means3D; a.radii = radii; a.dc = nullptr; a.shs = shs; a.splat = splat_buffer;
  a.scales = scales; a.rots = rotations; a.grad = grad_record;
  a.dmean2D = nullptr; a.dconic = nullptr; a.dopac = nullptr; a.dcolor = nullptr;
  a.dmean3D = nullptr; a.dcov3D = nullptr; a.ddc = nullptr; a.dsh = nullptr; a.dscale = nullptr; a.drot = nullptr;
  a.accum = xyz_gradient_accum; a.accum_abs = xyz_gradient_accum_abs; a.max_radii = max_radii; a.denom = denom;
  a.adam_on = 1; a.opac = opacities; a.adam = *adam;
  return run_preprocess_bwd(a, (cudaStream_t)stream);
}

extern "C" fgs_status fgs_densify_stats(int P, const int32_t* radii, const float* dL_dmean2D,
                                        float* xyz_gradient_accum, float* xyz_gradient_accum_abs,
                                        float* max_radii, float* denom, void* stream) {
  if (P < 0) return FGS_ERR_BAD_ARG;
  if (P == 0) return FGS_OK;
  if (!radii || !dL_dmean2D || ((uintptr_t)dL_dmean2D & 15)) return FGS_ERR_BAD_ARG;
  k_densify<<<(P + 255) / 256, 256, 0, (cudaStream_t)stream>>>(P, radii, reinterpret_cast<const float4*>(dL_dmean2D),
                                                              xyz_gradient_accum, xyz_gradient_accum_abs, max_radii,
                                                              denom);
  FGS_LAUNCH_CHECK();
  return FGS_OK;
}
