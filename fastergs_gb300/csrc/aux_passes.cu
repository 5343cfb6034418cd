// Auxiliary passes over the sorted tile lists, sm_103a: the importance pass
// (FB csrc/cuda_rasterizer/render_simp.cu) and the depth pass
// (FB csrc/cuda_rasterizer/render_depth.cu) that Mini-Splatting-style
// pipelines use for pruning and depth-based re-initialisation.  Both are
// sequential per tile / per pixel in FB and stay so here (their stopping
// rules depend on the order); they reuse the splat records, the sorted lists
// and the exponent form of the compositing kernels.
#include <algorithm>

#include "render_common.cuh"

namespace fgs {
namespace {

// Importance pass: one warp per 16x16 tile (8 pixels per lane), Gaussians in
// list order.  Per Gaussian: weights alpha T summed over the tile's pixels and
// the number of pixels with alpha >= 1/255 (FB pixel_shader,
// render_simp.cu:35-63); per pixel the Gaussian of largest weight.  The tile
// stops after a pair of Gaussians once every pixel of the tile has T < 1e-4
// (FB checks after each pair -- a lone first Gaussian when the count is odd,
// render_simp.cu:120-236 -- and never stops a tile that overlaps the image
// border, whose outside pixels keep T = 1).
__global__ void __launch_bounds__(kWarp) k_render_simp(int P, int W, int H, int gx, const float* __restrict__ splat,
                                                       const uint32_t* __restrict__ vals,
                                                       const uint32_t* __restrict__ ranges,
                                                       float* __restrict__ accum_weights,
                                                       int* __restrict__ accum_count,
                                                       float* __restrict__ accum_max_count) {
  using M = TileMap<16>;
  __shared__ BucketStage st;
  const int tile = blockIdx.x, lane = threadIdx.x;
  const int tx0 = (tile % gx) * 16, ty0 = (tile / gx) * 16;
  const int rs = (int)ranges[2 * tile], re = (int)ranges[2 * tile + 1], n = re - rs;
  float pxc[M::kCols], pyr[M::kRows];
#pragma unroll
  for (int c = 0; c < M::kCols; ++c) pxc[c] = (float)(tx0 + 8 * c + (lane & 7));
#pragma unroll
  for (int r = 0; r < M::kRows; ++r) pyr[r] = (float)(ty0 + 4 * r + (lane >> 3));
  float T[kPxPerThread], wmax[kPxPerThread];
  int imax[kPxPerThread];
  uint32_t in_img = 0;
#pragma unroll
  for (int r = 0; r < M::kRows; ++r)
#pragma unroll
    for (int cc = 0; cc < M::kCols; ++cc) {
      const int k = r * M::kCols + cc;
      T[k] = 1.f; wmax[k] = 0.f; imax[k] = -1;
      if ((int)pxc[cc] < W && (int)pyr[r] < H) in_img |= 1u << k;
    }
  const int odd = n & 1;
  bool stop = false;
  for (int base = 0; base < n && !stop; base += kSubBucket) {
    const int cnt = min(kSubBucket, n - base);
    stage_bucket<16>(st, splat, load_stage_ids(vals + rs + base, cnt, lane), cnt, lane, tx0, ty0);
    for (int g = 0; g < cnt; ++g) {
      const int i = base + g;  // position in the tile's list
      const uint32_t mask = st.mask[g];
      float wsum = 0.f;
      int wcnt = 0;
      const uint32_t id = __float_as_uint(st.rgb[g].w);
      if (mask != 0u) {
        const float4 pos = st.pos[g];
        const float4 q4 = st.quad[g];
#pragma unroll
        for (int r = 0; r < M::kRows; ++r)
#pragma unroll
          for (int cc = 0; cc < M::kCols; ++cc) {
            const int k = r * M::kCols + cc;
            if (!((mask >> k) & 1u) || !((in_img >> k) & 1u)) continue;
            const float dy = centre_offset(pos.y, pos.w, pyr[r]);
            const float w = shear_offset(q4.y, pos.y - pyr[r], pos.x - pxc[cc], fmaf(q4.y, pos.w, pos.z));
            const float e = fmaf(q4.x * w, w, fmaf(q4.z * dy, dy, q4.w));
            const float al = fminf(kAlphaMax, ex2_approx(e));
            if (al < kAlphaCut) continue;
            const float wt = al * T[k];
            T[k] -= wt;
            wsum += wt;
            wcnt += 1;
            if (wmax[k] < wt) { wmax[k] = wt; imax[k] = (int)id; }
          }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
        wcnt += __shfl_xor_sync(0xffffffffu, wcnt, o);
      }
      if (lane == 0 && id < (uint32_t)P) {
        atomicAdd(accum_weights + id, wsum);
        atomicAdd(accum_count + id, wcnt);
      }
      if (i >= odd && ((i - odd) & 1)) {  // end of a pair: does the whole tile stop?
        bool done = true;
#pragma unroll
        for (int k = 0; k < kPxPerThread; ++k) done = done && ((in_img >> k) & 1u) && T[k] < kTMin;
        if (__all_sync(0xffffffffu, done)) { stop = true; break; }
      }
    }
    __syncwarp();
  }
#pragma unroll
  for (int k = 0; k < kPxPerThread; ++k)
    if (imax[k] >= 0) atomicAdd(accum_max_count + imax[k], 1.f);
}

// 4x4 inverse (column-major) in FP64 by cofactors.
__device__ void invert4(const float* m, float* out) {
  double a[16], inv[16];
  for (int i = 0; i < 16; ++i) a[i] = m[i];
  inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] +
           a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
  inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] -
           a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
  inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] +
           a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
  inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] -
            a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
  inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] -
           a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
  inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] +
           a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
  inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] -
           a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
  inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] +
            a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
  inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] +
           a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
  inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] -
           a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
  inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] +
            a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
  inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] -
            a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
  inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] -
           a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
  inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] +
           a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
  inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] -
            a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
  inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] +
            a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
  const double det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
  const double s = det != 0.0 ? 1.0 / det : 0.0;
  for (int i = 0; i < 16; ++i) out[i] = (float)(inv[i] * s);
}

constexpr int kDepthThreads = 256;

// Depth pass: one thread per pixel, the tile's list in batches of 256
// (FB render_depthCUDA, render_depth.cu:97-327).  Per pixel: the ray from
// the camera through the pixel's NDC point on the far plane mapped by the
// inverse projection (not divided by w, as FB does); Gaussians in order with
// alpha < 1/255 skipped, a stop before the one that would take T below 1e-4,
// and those whose 3-sigma ellipsoid's closest point lies behind the camera
// skipped without changing T.  The Gaussian of largest weight alpha T gives
// the depth, the world point, the discriminant and the index.
__global__ void __launch_bounds__(kDepthThreads) k_render_depth(
    int W, int H, int gx, const float* __restrict__ splat, const uint32_t* __restrict__ vals,
    const uint32_t* __restrict__ ranges, const float* __restrict__ means3D, const float* __restrict__ scales,
    const float* __restrict__ rotations, const float* __restrict__ projmatrix, const float* __restrict__ campos,
    float* __restrict__ out_pts, float* __restrict__ out_depth, float* __restrict__ accum_alpha,
    int* __restrict__ gidx, float* __restrict__ discriminants) {
  __shared__ float s_inv[16];
  __shared__ float4 s_pos[kDepthThreads], s_quad[kDepthThreads], s_rot[kDepthThreads];
  __shared__ float s_geo[kDepthThreads][6];  // mean xyz, 3-sigma scale xyz
  __shared__ int s_id[kDepthThreads];
  const int tile = blockIdx.x, t = threadIdx.x;
  if (t == 0) invert4(projmatrix, s_inv);
  const int px = (tile % gx) * 16 + (t & 15), py = (tile / gx) * 16 + (t >> 4);
  const bool inside = px < W && py < H;
  bool done = !inside;
  __syncthreads();
  // ray (FB render_depth.cu:160-188)
  const float ox = campos[0], oy = campos[1], oz = campos[2];
  const float nx = ((2.f * px + 1.f) / W - 1.f) * 1.0000001f, ny = ((2.f * py + 1.f) / H - 1.f) * 1.0000001f;
  const float nz = (float)((100.0 - 100.0 * 0.01) / (100.0 - 0.01));
  const float* m = s_inv;
  const float rx = m[0] * nx + m[4] * ny + m[8] * nz + m[12] - ox;
  const float ry = m[1] * nx + m[5] * ny + m[9] * nz + m[13] - oy;
  const float rz = m[2] * nx + m[6] * ny + m[10] * nz + m[14] - oz;
  const float rlen = sqrtf(rx * rx + ry * ry + rz * rz);
  const float dnx = rx / rlen, dny = ry / rlen, dnz = rz / rlen;

  const int rs = (int)ranges[2 * tile], re = (int)ranges[2 * tile + 1];
  float T = 1.f, wmax = 0.f, dmax = 0.f, discmax = 0.f, prx = 0.f, pry = 0.f, prz = 0.f;
  int imax = 0;
  for (int base = rs; base < re; base += kDepthThreads) {
    if (__syncthreads_count(done) == kDepthThreads) break;
    const int j = base + t;
    if (j < re) {
      const uint32_t id = vals[j];
      const float4* rec = reinterpret_cast<const float4*>(splat + (size_t)id * 32);
      const float4 a = __ldg(rec), b = __ldg(rec + 1), c = __ldg(rec + 2);
      s_pos[t] = make_float4(floorf(a.x), floorf(a.y), c.z, c.w);
      s_quad[t] = make_float4(b.z, b.w, c.x, c.y);
      s_rot[t] = *reinterpret_cast<const float4*>(rotations + 4 * (size_t)id);
      for (int k = 0; k < 3; ++k) {
        s_geo[t][k] = means3D[3 * (size_t)id + k];
        s_geo[t][3 + k] = scales[3 * (size_t)id + k] * 3.0f;
      }
      s_id[t] = (int)id;
    }
    __syncthreads();
    const int cnt = min(kDepthThreads, re - base);
    for (int g = 0; !done && g < cnt; ++g) {
      const float4 pos = s_pos[g], q4 = s_quad[g];
      const float dy = centre_offset(pos.y, pos.w, (float)py);
      const float w = shear_offset(q4.y, pos.y - (float)py, pos.x - (float)px, fmaf(q4.y, pos.w, pos.z));
      const float e = fmaf(q4.x * w, w, fmaf(q4.z * dy, dy, q4.w));
      const float al = fminf(kAlphaMax, ex2_approx(e));
      if (al < kAlphaCut) continue;
      const float test_T = T * (1.f - al);
      if (test_T < kTMin) { done = true; continue; }
      // closest approach of the ray to the Gaussian's 3-sigma ellipsoid, in
      // its frame: R^T (o - mean) and R^T d (R from the raw quaternion)
      const float4 q = s_rot[g];
      const float qr = q.x, qx = q.y, qy = q.z, qz = q.w;
      const float R00 = 1.f - 2.f * (qy * qy + qz * qz), R01 = 2.f * (qx * qy - qr * qz), R02 = 2.f * (qx * qz + qr * qy);
      const float R10 = 2.f * (qx * qy + qr * qz), R11 = 1.f - 2.f * (qx * qx + qz * qz), R12 = 2.f * (qy * qz - qr * qx);
      const float R20 = 2.f * (qx * qz - qr * qy), R21 = 2.f * (qy * qz + qr * qx), R22 = 1.f - 2.f * (qx * qx + qy * qy);
      const float tx = ox - s_geo[g][0], ty = oy - s_geo[g][1], tz = oz - s_geo[g][2];
      const float sx = s_geo[g][3], sy = s_geo[g][4], sz = s_geo[g][5];
      const float lo0 = (R00 * tx + R10 * ty + R20 * tz) / sx, lo1 = (R01 * tx + R11 * ty + R21 * tz) / sy,
                  lo2 = (R02 * tx + R12 * ty + R22 * tz) / sz;
      const float ld0 = (R00 * dnx + R10 * dny + R20 * dnz) / sx, ld1 = (R01 * dnx + R11 * dny + R21 * dnz) / sy,
                  ld2 = (R02 * dnx + R12 * dny + R22 * dnz) / sz;
      const float qa = ld0 * ld0 + ld1 * ld1 + ld2 * ld2;
      const float qb = 2.f * (ld0 * lo0 + ld1 * lo1 + ld2 * lo2);
      const float tmin = -qb / 2.f / qa;
      const float depth = tmin / rlen;
      if (depth < 0.f) continue;
      const float wt = al * T;
      if (wmax < wt) {
        wmax = wt;
        dmax = depth;
        // b^2 - 4ac, which FB forms directly and which cancels in FP32 when
        // the ray passes near the ellipsoid, by Lagrange's identity:
        // (d.o)^2 - |d|^2 |o|^2 = -|d x o|^2, so b^2 - 4ac = 4 (|d|^2 - |d x o|^2)
        const float x0 = ld1 * lo2 - ld2 * lo1, x1 = ld2 * lo0 - ld0 * lo2, x2 = ld0 * lo1 - ld1 * lo0;
        discmax = 4.f * (qa - (x0 * x0 + x1 * x1 + x2 * x2));
        imax = s_id[g];
        prx = ox + tmin * dnx; pry = oy + tmin * dny; prz = oz + tmin * dnz;
      }
      T = test_T;
    }
    __syncthreads();
  }
  if (inside) {
    const size_t HW = (size_t)W * H, pix = (size_t)py * W + px;
    out_pts[pix] = prx;
    out_pts[HW + pix] = pry;
    out_pts[2 * HW + pix] = prz;
    out_depth[pix] = dmax;
    accum_alpha[pix] = T;
    discriminants[pix] = discmax;
    gidx[pix] = imax;
  }
}

}  // namespace
}  // namespace fgs

FGS_DEFINE_ERROR_ACCESSOR(aux)

using namespace fgs;

extern "C" fgs_status fgs_render_simp(int P, int64_t num_rendered, int width, int height, const float* splat_buffer,
                                      const uint64_t* keys_sorted, const uint32_t* values_sorted, uint32_t* ranges,
                                      float* accum_weights, int32_t* accum_count, float* accum_max_count,
                                      void* stream) {
  if (P < 0 || num_rendered < 0 || width <= 0 || height <= 0 || !ranges ||
      (num_rendered > 0 && (!keys_sorted || !values_sorted || !splat_buffer)))
    return FGS_ERR_BAD_ARG;
  if (P > 0 && (!accum_weights || !accum_count || !accum_max_count)) return FGS_ERR_BAD_ARG;
  if (((uintptr_t)splat_buffer & 15)) return FGS_ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int gx = (width + 15) / 16, gy = (height + 15) / 16;
  if (P > 0) {
    FGS_TRY(cudaMemsetAsync(accum_weights, 0, sizeof(float) * P, s));
    FGS_TRY(cudaMemsetAsync(accum_count, 0, sizeof(int32_t) * P, s));
    FGS_TRY(cudaMemsetAsync(accum_max_count, 0, sizeof(float) * P, s));
  }
  fgs_status st = run_tile_ranges(num_rendered, nullptr, (uint32_t)(gx * gy), keys_sorted, ranges, s);
  if (st != FGS_OK) return st;
  KernelTimer kt__(FGS_K_SIMP, s);
  k_render_simp<<<gx * gy, kWarp, 0, s>>>(P, width, height, gx, splat_buffer, values_sorted, ranges, accum_weights,
                                          accum_count, accum_max_count);
  kt__.stop();
  FGS_LAUNCH_CHECK();
  return FGS_OK;
}

extern "C" fgs_status fgs_render_depth(int P, int64_t num_rendered, int width, int height, const float* splat_buffer,
                                       const uint64_t* keys_sorted, const uint32_t* values_sorted, uint32_t* ranges,
                                       const float* means3D, const float* scales, const float* rotations,
                                       const float* projmatrix, const float* campos, float* out_pts,
                                       float* out_depth, float* accum_alpha, int32_t* gidx, float* discriminants,
                                       void* stream) {
  if (P < 0 || num_rendered < 0 || width <= 0 || height <= 0 || !ranges || !projmatrix || !campos || !out_pts ||
      !out_depth || !accum_alpha || !gidx || !discriminants)
    return FGS_ERR_BAD_ARG;
  if (num_rendered > 0 && (!keys_sorted || !values_sorted || !splat_buffer || !means3D || !scales || !rotations))
    return FGS_ERR_BAD_ARG;
  if (((uintptr_t)splat_buffer & 15) || ((uintptr_t)rotations & 15)) return FGS_ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int gx = (width + 15) / 16, gy = (height + 15) / 16;
  fgs_status st = run_tile_ranges(num_rendered, nullptr, (uint32_t)(gx * gy), keys_sorted, ranges, s);
  if (st != FGS_OK) return st;
  KernelTimer kt__(FGS_K_DEPTH, s);
  k_render_depth<<<gx * gy, kDepthThreads, 0, s>>>(width, height, gx, splat_buffer, values_sorted, ranges, means3D,
                                                    scales, rotations, projmatrix, campos, out_pts, out_depth,
                                                    accum_alpha, gidx, discriminants);
  kt__.stop();
  FGS_LAUNCH_CHECK();
  return FGS_OK;
}
