// Per-Gaussian preprocess and (tile | depth, Gaussian) key emission, sm_103a.
//
// Restates FB csrc/cuda_rasterizer/preprocess.cu (projection, EWA covariance,
// SH colour, tile rectangle, ellipse/tile test, lane-packed emission of small
// Gaussians, 128-tile sub-tasks for large ones) with a GB300 layout:
//   * one CTA of 2 warps handles 64 consecutive Gaussians, one per thread;
//   * the warp's small Gaussians are flattened into one candidate list
//     (exclusive scan of rect areas) and 32 candidates are tested per step, so
//     every lane does useful work whatever the footprint mix;
//   * hits are staged per warp in shared memory and flushed with one atomic
//     per ~100 pairs instead of one per 32 candidates;
//   * large Gaussians queue (id, first tile) sub-tasks that a persistent
//     second kernel drains; the task count never travels to the host.
#include "internal.cuh"

namespace fgs {
namespace {

// Gaussians per preprocess block: 64 at 16 blocks per SM (64 registers, 32
// warps per SM); at 1M Gaussians in a 1297x840 view 0.109 ms, against 0.111
// with 128 at 8 per SM, 0.117 with 256 at 4 and 0.126 with 256 at 3.
constexpr int kPreThreads = 64;
constexpr int kPreWarps = kPreThreads / kWarp;
constexpr int kStage = 128;  // staged pairs per warp before a flush

// Ellipse chord test along one tile edge (FB preprocess.cu:168-177): does the
// quadratic A u^2 + B u + C = 0 have a root interval meeting [l - d, r - d]?
__device__ __forceinline__ bool chord_hits(float A, float B, float C, float d, float l, float r) {
  const float disc = B * B - 4.0f * A * C;
  const float t1 = (l - d) * (2.0f * A) + B;
  const float t2 = (r - d) * (2.0f * A) + B;
  return disc >= 0.0f && (t1 <= 0.0f || t1 * t1 <= disc) && (t2 >= 0.0f || t2 * t2 <= disc);
}

// Does the level set conic(d) = 2*power touch the pixel block whose top-left
// pixel centre is (px0, py0)?  Centre-inside test plus a chord test against
// the nearest vertical and nearest horizontal edge (FB preprocess.cu:179-218).
__device__ __forceinline__ bool tile_hit(int px0, int py0, int bx, int by, float2 c, float4 cp) {
  const float x0 = (float)px0, x1 = (float)(px0 + bx - 1);
  const float y0 = (float)py0, y1 = (float)(py0 + by - 1);
  if (c.x >= x0 && c.x <= x1 && c.y >= y0 && c.y <= y1) return true;
  const float w = 2.0f * cp.w;
  const float dx = c.x - ((c.x * 2.0f < x0 + x1) ? x0 : x1);
  if (chord_hits(cp.z, -2.0f * cp.y * dx, cp.x * dx * dx - w, c.y, y0, y1)) return true;
  const float dy = c.y - ((c.y * 2.0f < y0 + y1) ? y0 : y1);
  return chord_hits(cp.x, -2.0f * cp.y * dy, cp.z * dy * dy - w, c.x, x0, x1);
}

struct WarpStage {
  unsigned long long* key;
  uint32_t* val;
  int n;
};

__device__ __forceinline__ void stage_flush(WarpStage& st, const PreArgs& a, int lane) {
  __syncwarp();
  if (st.n == 0) return;
  unsigned int base = 0;
  if (lane == 0) base = atomicAdd(a.curr, (unsigned int)st.n);
  base = __shfl_sync(0xffffffffu, base, 0);
  bool over = false;
  for (int j = lane; j < st.n; j += kWarp) {
    const long long dst = (long long)base + j;
    if (dst < a.cap) {
      a.keys[dst] = st.key[j];
      a.vals[dst] = st.val[j];
    } else {
      over = true;
    }
  }
  if (__any_sync(0xffffffffu, over) && lane == 0) raise_error(kErrCapacity);
  st.n = 0;
  __syncwarp();
}

__device__ __forceinline__ void stage_push(WarpStage& st, const PreArgs& a, int lane, bool hit,
                                           unsigned long long key, uint32_t id) {
  const uint32_t m = __ballot_sync(0xffffffffu, hit);
  if (m == 0) return;
  const int cnt = __popc(m);
  if (st.n + cnt > kStage) stage_flush(st, a, lane);
  if (hit) {
    const int pos = st.n + __popc(m & lanemask_lt());
    st.key[pos] = key;
    st.val[pos] = id;
  }
  st.n += cnt;
}

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 ld3(const float* p) { return f3(p[0], p[1], p[2]); }

// SH colour at the unit view direction (FB preprocess.cu:119-166).
__device__ __forceinline__ float3 sh_colour(int D, float x, float y, float z, const float* dc, const float* sh,
                                            float* clamp) {
  float3 r = 0.28209479177387814f * ld3(dc);
  if (D > 0) {
    const float c1 = 0.4886025119029199f;
    r = r + (-c1 * y) * ld3(sh + 0) + (c1 * z) * ld3(sh + 3) + (-c1 * x) * ld3(sh + 6);
    if (D > 1) {
      const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
      r = r + (1.0925484305920792f * xy) * ld3(sh + 9) + (-1.0925484305920792f * yz) * ld3(sh + 12) +
          (0.31539156525252005f * (2.0f * zz - xx - yy)) * ld3(sh + 15) +
          (-1.0925484305920792f * xz) * ld3(sh + 18) + (0.5462742152960396f * (xx - yy)) * ld3(sh + 21);
      if (D > 2) {
        r = r + (-0.5900435899266435f * y * (3.0f * xx - yy)) * ld3(sh + 24) +
            (2.890611442640554f * xy * z) * ld3(sh + 27) +
            (-0.4570457994644658f * y * (4.0f * zz - xx - yy)) * ld3(sh + 30) +
            (0.3731763325901154f * z * (2.0f * zz - 3.0f * xx - 3.0f * yy)) * ld3(sh + 33) +
            (-0.4570457994644658f * x * (4.0f * zz - xx - yy)) * ld3(sh + 36) +
            (1.445305721320277f * z * (xx - yy)) * ld3(sh + 39) +
            (-0.5900435899266435f * x * (xx - 3.0f * yy)) * ld3(sh + 42);
      }
    }
  }
  r = r + f3(0.5f, 0.5f, 0.5f);
  clamp[0] = r.x < 0.0f ? 1.0f : 0.0f;
  clamp[1] = r.y < 0.0f ? 1.0f : 0.0f;
  clamp[2] = r.z < 0.0f ? 1.0f : 0.0f;
  return f3(fmaxf(r.x, 0.0f), fmaxf(r.y, 0.0f), fmaxf(r.z, 0.0f));
}

__global__ void __launch_bounds__(kPreThreads, 16) k_preprocess(const PreArgs a) {
  pdl_wait();  // the preceding kernel of the stream is done
  pdl_trigger();
  __shared__ float2 s_xy[kPreWarps][kWarp];
  __shared__ float4 s_cp[kPreWarps][kWarp];    // conic a, b, c, power
  __shared__ int4 s_geo[kPreWarps][kWarp];     // rect min x, min y, width, candidate start
  __shared__ float s_inv_w[kPreWarps][kWarp];  // 1 / rect width
  __shared__ uint32_t s_depth[kPreWarps][kWarp];
  __shared__ unsigned long long s_key[kPreWarps][kStage];
  __shared__ uint32_t s_val[kPreWarps][kStage];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // Block b covers Gaussians [(b / V) * kPreThreads, +kPreThreads) of view b % V: the views of
  // one Gaussian chunk run back to back, so its parameters come from L2 after
  // the first view instead of being re-read from HBM per view.
  const int vi = (int)(blockIdx.x % (unsigned)a.views.V);
  const int chunk = (int)(blockIdx.x / (unsigned)a.views.V);
  const int i = chunk * kPreThreads + threadIdx.x;

  const ViewDesc& cam = a.views.v[vi];
  const int bx = a.views.bx, by = a.views.by;
  const size_t rbase = (size_t)vi * a.P;  // first record of this view

  bool valid = false;
  int area = 0, tw = 0;
  int2 rmin = make_int2(0, 0), rmax = make_int2(0, 0);
  float2 xy = make_float2(0.f, 0.f);
  float4 cp = make_float4(0.f, 0.f, 0.f, 0.f);
  float depth = 0.f;

  if (i < a.P) {
    float radius = 0.0f;
    float rec[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) rec[k] = 0.0f;
    do {
      if (a.culling && a.culling[i]) break;
      const float3 p = ld3(a.means + 3 * (size_t)i);
      const float3 t = xform_point3(cam.view, p);
      if (t.z <= 0.2f) break;                        // near cull (FB preprocess.cu:456)
      const float o = a.opac[i];
      if (255.0f * o < 1.0f) break;                  // opacity cull (FB preprocess.cu:459)
      // Projection to pixels in float-float.  FB projects in FP32 and converts
      // NDC to pixels in double (preprocess.cu:463-465, 494); an FP32 pixel
      // position near 1000 px is only good to 6e-5 px, which would dominate
      // the image error, so the homogeneous coordinates are summed from exact
      // products, divided and scaled in float-float (the value FP64 gives, to
      // ~1e-12 relative) and the position's fraction is kept.
      const float* Pm = cam.proj;
      auto row = [&](int r) {
        ff acc = ff_prod(Pm[r], p.x);
        acc = ff_add(acc, ff_prod(Pm[4 + r], p.y));
        acc = ff_add(acc, ff_prod(Pm[8 + r], p.z));
        return ff_add_f(acc, Pm[12 + r]);
      };
      const ff hx = row(0), hy = row(1), hw = row(3);
      constexpr float kEpsHi = 1e-7f;
      constexpr float kEpsLo = (float)(1e-7 - (double)kEpsHi);
      const ff wden = ff_add(hw, ff{kEpsHi, kEpsLo});  // p_w + 1e-7 (FB preprocess.cu:464)
      auto to_px = [&](ff h, int n) {  // ((h / w + 1) * n - 1) / 2
        ff t = ff_add_f(ff_div(h, wden), 1.0f);
        t = ff_add_f(ff_mul_f(t, (float)n), -1.0f);
        return ff{0.5f * t.hi, 0.5f * t.lo};
      };
      const ff X = to_px(hx, cam.W), Y = to_px(hy, cam.H);

      // 3D covariance R diag(s^2) R^T from the raw quaternion (FB preprocess.cu:364-400).
      const float4 q = *reinterpret_cast<const float4*>(a.rots + 4 * (size_t)i);
      const float qr = q.x, qx = q.y, qy = q.z, qz = q.w;
      float R[3][3];
      R[0][0] = 1.f - 2.f * (qy * qy + qz * qz); R[0][1] = 2.f * (qx * qy - qr * qz); R[0][2] = 2.f * (qx * qz + qr * qy);
      R[1][0] = 2.f * (qx * qy + qr * qz); R[1][1] = 1.f - 2.f * (qx * qx + qz * qz); R[1][2] = 2.f * (qy * qz - qr * qx);
      R[2][0] = 2.f * (qx * qz - qr * qy); R[2][1] = 2.f * (qy * qz + qr * qx); R[2][2] = 1.f - 2.f * (qx * qx + qy * qy);
      const float sx = cam.smod * a.scales[3 * (size_t)i], sy = cam.smod * a.scales[3 * (size_t)i + 1],
                  sz = cam.smod * a.scales[3 * (size_t)i + 2];
      const float s2[3] = {sx * sx, sy * sy, sz * sz};
      float S[6];
      {
        int k = 0;
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = r; c < 3; ++c) S[k++] = R[r][0] * s2[0] * R[c][0] + R[r][1] * s2[1] * R[c][1] + R[r][2] * s2[2] * R[c][2];
      }
      // EWA screen covariance (FB preprocess.cu:79-117).
      const float limx = 1.3f * cam.tanx, limy = 1.3f * cam.tany;
      const float tx = fminf(limx, fmaxf(-limx, t.x / t.z)) * t.z;
      const float ty = fminf(limy, fmaxf(-limy, t.y / t.z)) * t.z;
      const float j00 = cam.fx / t.z, j02 = -(cam.fx * tx) / (t.z * t.z);
      const float j11 = cam.fy / t.z, j12 = -(cam.fy * ty) / (t.z * t.z);
      const float* V = cam.view;
      // M = J * Rw, Rw[k][b] = V[b*4 + k]
      float M0[3], M1[3];
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        M0[b] = j00 * V[b * 4 + 0] + j02 * V[b * 4 + 2];
        M1[b] = j11 * V[b * 4 + 1] + j12 * V[b * 4 + 2];
      }
      const ScreenCov sc2 = screen_cov(M0, M1, R, s2);
      const float ca = sc2.a, cb = sc2.b, cc = sc2.c, det = sc2.det;
      const float det_inv = 1.0f / det;
      const float3 conic = f3(cc * det_inv, -cb * det_inv, ca * det_inv);
      // Reported radius (FB preprocess.cu:480-485).  FB compares with the
      // double 3.33 and stores the result in a float, so the extent, the
      // product and its ceiling are all FP32 (for o <= 1 the square root is
      // at most sqrt(2 ln 255) = 3.329, below the bound).
      const float mid = 0.5f * (ca + cc);
      const float extent = fminf(3.33f, sqrtf(2.0f * logf(o * 255.0f)));
      // mid^2 - det written as ((a - c)/2)^2 + b^2, which does not cancel
      const float hd = 0.5f * (ca - cc);
      const float lambda = mid + sqrtf(fmaxf(0.01f, hd * hd + cb * cb));
      radius = ceilf(extent * sqrtf(lambda));
      // Tile rectangle of the 1/256 level set (FB preprocess.cu:488-497).
      const float log2o = lg2_approx(o);
      const float power = (kLn2 * 8.0f + kLn2 * log2o) * cam.mult;
      const int wpx = (int)(1.414214f * sqrt_approx(ca * power) + 1.0f);
      const int hpx = (int)(1.414214f * sqrt_approx(cc * power) + 1.0f);
      xy = make_float2(X.hi, Y.hi);
      rmin.x = min(cam.gx, max(0, (int)((xy.x - wpx) / (float)bx)));
      rmin.y = min(cam.gy, max(0, (int)((xy.y - hpx) / (float)by)));
      rmax.x = min(cam.gx, max(0, (int)((xy.x + wpx) / (float)bx) + 1));
      rmax.y = min(cam.gy, max(0, (int)((xy.y + hpx) / (float)by) + 1));
      tw = rmax.x - rmin.x;
      area = tw * (rmax.y - rmin.y);
      if (area <= 0) break;
      valid = true;
      cp = make_float4(conic.x, conic.y, conic.z, power);
      depth = t.z;

      float3 rgb;
      if (a.colors) {
        rgb = ld3(a.colors + 3 * (size_t)i);
      } else {
        const float3 cpos = ld3(cam.campos);
        float dxv = p.x - cpos.x, dyv = p.y - cpos.y, dzv = p.z - cpos.z;
        const float inv = 1.0f / sqrtf(dxv * dxv + dyv * dyv + dzv * dzv);
        // each thread reads its own contiguous SH row; consecutive loads hit the same L1 lines
        rgb = sh_colour(a.D, dxv * inv, dyv * inv, dzv * inv, a.dc + 3 * (size_t)i,
                        a.shs ? a.shs + (size_t)i * a.M * 3 : nullptr, rec + F_CLAMP);
      }
      rec[F_XY] = xy.x; rec[F_XY + 1] = xy.y;
      rec[F_RGB] = rgb.x; rec[F_RGB + 1] = rgb.y; rec[F_RGB + 2] = rgb.z;
      rec[F_DEPTH] = t.z;
      // Exponent of alpha in the cancellation-free form
      // log2 o + A1 (dx + P dy)^2 + C1 dy^2 (equal to FB's con_o form).
      rec[F_CHOL] = (-0.5f * kLog2e) * conic.x;
      rec[F_CHOL + 1] = -cb / cc;
      rec[F_CHOL + 2] = (-0.5f * kLog2e) / cc;
      rec[F_LOG2O] = log2o;
      // X - floor(X.hi): the first difference is exact (a fraction of X.hi)
      rec[F_FRAC] = __fadd_rn(__fsub_rn(X.hi, floorf(X.hi)), X.lo);
      rec[F_FRAC + 1] = __fadd_rn(__fsub_rn(Y.hi, floorf(Y.hi)), Y.lo);
      rec[F_RMIN] = __int_as_float(rmin.x); rec[F_RMIN + 1] = __int_as_float(rmin.y);
      rec[F_RMAX] = __int_as_float(rmax.x); rec[F_RMAX + 1] = __int_as_float(rmax.y);
      rec[F_CONIC] = conic.x; rec[F_CONIC + 1] = conic.y; rec[F_CONIC + 2] = conic.z;
      rec[F_POWER] = power;
      rec[F_PVIEW] = t.x; rec[F_PVIEW + 1] = t.y; rec[F_PVIEW + 2] = t.z;
#pragma unroll
      for (int k = 0; k < 6; ++k) rec[F_COV3D + k] = S[k];
    } while (false);
    a.radii[rbase + i] = valid ? (int)radius : 0;
    if (valid) {
      float4* dst = reinterpret_cast<float4*>(a.splat + (rbase + i) * 32);
#pragma unroll
      for (int k = 0; k < 8; ++k) dst[k] = make_float4(rec[4 * k], rec[4 * k + 1], rec[4 * k + 2], rec[4 * k + 3]);
    }
  }

  // Large footprints: queue large_tiles-tile sub-tasks (FB preprocess.cu:723-745
  // uses 128).
  const int LT = a.large_tiles;
  const bool small = valid && area < LT;
  if (valid && !small) {
    const int n = (area + LT - 1) / LT;
    const int base = atomicAdd(&a.counters[0], n);
    for (int j = 0; j < n; ++j) {
      const long long t = (long long)base + j;
      if (t < a.task_cap) {
        a.tasks[2 * t] = (uint32_t)(rbase + i);
        a.tasks[2 * t + 1] = (uint32_t)(j * LT);
      } else {
        raise_error(kErrCapacity);
      }
    }
  }

  // Small footprints (area < LT <= 256 tiles, so the row of candidate `local`
  // is row_of(local, 1 / width), exact for local < 256 width): flatten the
  // warp's (Gaussian, tile) candidates and test
  // 32 x packet at a time, packet consecutive candidates per lane (the lane
  // packing of FB preprocess.cu:536-696, which tests one per lane): a lane
  // finds the owner of its first candidate and walks on from there.
  const int cnt = small ? area : 0;
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < kWarp; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  s_xy[warp][lane] = xy;
  s_cp[warp][lane] = cp;
  s_geo[warp][lane] = make_int4(rmin.x, rmin.y, tw, incl - cnt);
  s_inv_w[warp][lane] = tw > 0 ? 1.0f / (float)tw : 0.f;
  s_depth[warp][lane] = __float_as_uint(depth);
  __syncwarp();

  WarpStage st{s_key[warp], s_val[warp], 0};
  const int warp_first = chunk * kPreThreads + warp * kWarp;
  const int pk = a.packet;
  if (pk == 1) {  // one candidate per lane (FB's packing): no owner walk
    for (int base = 0; base < total; base += kWarp) {
      const int c = base + lane;
      bool hit = false;
      unsigned long long key = 0;
      uint32_t gid = 0;
      if (c < total) {
        int lo = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
          if (s_geo[warp][lo + step].w <= c) lo += step;
        const int4 g = s_geo[warp][lo];
        const int local = c - g.w;
        const int ty = row_of(local, s_inv_w[warp][lo]), tx = local - ty * g.z;
        const int x = g.x + tx, y = g.y + ty;
        hit = tile_hit(x * bx, y * by, bx, by, s_xy[warp][lo], s_cp[warp][lo]);
        key = ((unsigned long long)(cam.tile_off + (uint32_t)(y * cam.gx + x)) << 32) | s_depth[warp][lo];
        gid = (uint32_t)(rbase + warp_first + lo);
      }
      stage_push(st, a, lane, hit, key, gid);
    }
    stage_flush(st, a, lane);
    return;
  }
  for (int base = 0; base < total; base += kWarp * pk) {
    const int c0 = base + lane * pk;
    // Owner = last lane whose candidate start is <= c (steps sum to 31, so
    // lo + step never leaves the warp); lanes with no candidates share the
    // start of the next lane and are passed over.
    int lo = 0;
    if (c0 < total) {
#pragma unroll
      for (int step = 16; step > 0; step >>= 1)
        if (s_geo[warp][lo + step].w <= c0) lo += step;
    }
    for (int j = 0; j < pk; ++j) {  // warp-uniform trip count
      const int c = c0 + j;
      bool hit = false;
      unsigned long long key = 0;
      uint32_t gid = 0;
      if (c < total) {
        while (lo < kWarp - 1 && s_geo[warp][lo + 1].w <= c) ++lo;
        const int4 g = s_geo[warp][lo];
        const int local = c - g.w;
        const int ty = row_of(local, s_inv_w[warp][lo]), tx = local - ty * g.z;
        const int x = g.x + tx, y = g.y + ty;
        hit = tile_hit(x * bx, y * by, bx, by, s_xy[warp][lo], s_cp[warp][lo]);
        key = ((unsigned long long)(cam.tile_off + (uint32_t)(y * cam.gx + x)) << 32) | s_depth[warp][lo];
        gid = (uint32_t)(rbase + warp_first + lo);
      }
      stage_push(st, a, lane, hit, key, gid);
    }
  }
  stage_flush(st, a, lane);
}

// Drains the large-Gaussian sub-task queue: one warp per 128-tile sub-task,
// persistent grid (FB preprocess.cu:749-895 uses a work-stealing cursor and a
// host read of the task count; here the count stays on the device).
__global__ void __launch_bounds__(kPreThreads) k_preprocess_large(const PreArgs a) {
  pdl_wait();  // the preceding kernel of the stream is done
  pdl_trigger();
  __shared__ unsigned long long s_key[kPreWarps][kStage];
  __shared__ uint32_t s_val[kPreWarps][kStage];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long ntask = min((long long)a.counters[0], a.task_cap);
  const int gw = blockIdx.x * kPreWarps + warp, nw = gridDim.x * kPreWarps;
  WarpStage st{s_key[warp], s_val[warp], 0};
  for (long long t = gw; t < ntask; t += nw) {
    const uint32_t id = a.tasks[2 * t], off = a.tasks[2 * t + 1];  // record index, first tile
    const ViewDesc& cam = a.views.v[id / (uint32_t)a.P];
    const int bx = a.views.bx, by = a.views.by;
    const float* r = a.splat + (size_t)id * 32;
    const float2 xy = make_float2(r[F_XY], r[F_XY + 1]);
    const uint32_t depth = __float_as_uint(r[F_DEPTH]);
    const int rx0 = __float_as_int(r[F_RMIN]), ry0 = __float_as_int(r[F_RMIN + 1]);
    const int rx1 = __float_as_int(r[F_RMAX]), ry1 = __float_as_int(r[F_RMAX + 1]);
    const float4 cp = make_float4(r[F_CONIC], r[F_CONIC + 1], r[F_CONIC + 2], r[F_POWER]);
    const int w = rx1 - rx0, area = w * (ry1 - ry0);
    const int end = min((int)off + a.large_tiles, area);
#pragma unroll 1
    for (int k = 0; k < a.large_tiles / kWarp; ++k) {
      const int c = (int)off + k * kWarp + lane;
      bool hit = false;
      unsigned long long key = 0;
      if (c < end) {
        const int ty = c / w, tx = c - ty * w;
        const int x = rx0 + tx, y = ry0 + ty;
        hit = tile_hit(x * bx, y * by, bx, by, xy, cp);
        key = ((unsigned long long)(cam.tile_off + (uint32_t)(y * cam.gx + x)) << 32) | depth;
      }
      stage_push(st, a, lane, hit, key, id);
    }
  }
  stage_flush(st, a, lane);
}

}  // namespace
}  // namespace fgs

FGS_DEFINE_ERROR_ACCESSOR(preprocess)

namespace fgs {
// Launches preprocess + large-Gaussian emission for every view of a.views
// (grid.y = view).  Shared by the plain and the batched entry points.
fgs_status run_preprocess(PreArgs& a, cudaStream_t s) {
  {
    const fgs_status z = zero_async(a.counters, FGS_COUNTER_WORDS * sizeof(int32_t), s);
    if (z != FGS_OK) return z;
  }
  {
    KernelTimer kt__(FGS_K_PREPROCESS, s);
    const unsigned blocks = (unsigned)((a.P + kPreThreads - 1) / kPreThreads) * (unsigned)a.views.V;
    (void)launch_pdl(k_preprocess, dim3(blocks), dim3(kPreThreads), 0, s, a);
    kt__.stop();
  }
  FGS_LAUNCH_CHECK();
  {
    KernelTimer kt__(FGS_K_PREPROCESS_LARGE, s);
    (void)launch_pdl(k_preprocess_large, dim3(num_sms() * (1024 / kPreThreads)), dim3(kPreThreads), 0, s, a);
    kt__.stop();
  }
  FGS_LAUNCH_CHECK();
  return FGS_OK;
}
}  // namespace fgs

extern "C" fgs_status fgs_preprocess(
    int P, int D, int M, const float* means3D, const float* colors_precomp, const float* dc, const float* shs,
    const float* opacities, const float* scales, const float* rotations, float scale_modifier, int width,
    int height, int block_x, int block_y, const float* campos, const float* viewmatrix, const float* projmatrix,
    float tan_fovx, float tan_fovy, float zfar, float znear, float mult, const uint8_t* culling,
    float* splat_buffer, int64_t splat_rows, uint64_t* keys_unsorted, uint32_t* values_unsorted,
    int64_t pair_capacity, uint32_t* task_scratch, int64_t task_scratch_words, int32_t* curr_offset,
    int32_t* counters, int32_t* radii, void* stream) {
  (void)zfar;
  (void)znear;
  using namespace fgs;
  if (P < 0 || D < 0 || D > 3 || width <= 0 || height <= 0 || block_x <= 0 || block_y <= 0) return FGS_ERR_BAD_ARG;
  if (P == 0) return FGS_OK;
  if (!means3D || !opacities || !scales || !rotations || !viewmatrix || !projmatrix || !splat_buffer ||
      !keys_unsorted || !values_unsorted || !curr_offset || !counters || !radii || !task_scratch)
    return FGS_ERR_BAD_ARG;
  if (!colors_precomp) {
    if (!dc || !campos) return FGS_ERR_BAD_ARG;
    if (D > 0 && (!shs || M < (D + 1) * (D + 1) - 1)) return FGS_ERR_BAD_ARG;
  }
  if (((uintptr_t)rotations & 15) || ((uintptr_t)splat_buffer & 15) || ((uintptr_t)keys_unsorted & 7))
    return FGS_ERR_BAD_ARG;
  if ((int64_t)P > splat_rows) return FGS_ERR_CAPACITY;
  PreArgs a;
  a.views = single_view(width, height, block_x, block_y, viewmatrix, projmatrix, campos, nullptr, tan_fovx, tan_fovy,
                        mult, scale_modifier);
  a.P = P; a.D = D; a.M = M;
  a.means = means3D; a.colors = colors_precomp; a.dc = dc; a.shs = shs; a.opac = opacities;
  a.scales = scales; a.rots = rotations; a.culling = culling; a.splat = splat_buffer;
  a.keys = reinterpret_cast<unsigned long long*>(keys_unsorted); a.vals = values_unsorted;
  a.cap = pair_capacity; a.tasks = task_scratch; a.task_cap = task_scratch_words / 2;
  a.curr = reinterpret_cast<unsigned int*>(curr_offset); a.counters = counters; a.radii = radii;
  a.large_tiles = kLargeTiles;
  a.packet = kPacket;
  return run_preprocess(a, (cudaStream_t)stream);
}
