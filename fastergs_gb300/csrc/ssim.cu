// SSIM and the training loss right after the image, sm_103a.
//
// Restates the fused-ssim extension FasterGS's backbones train with
// (gs_submodules/fused-ssim/ssim.cu, fused_ssim/__init__.py; called as
// fast_ssim(image, gt) in taming-3dgs/train_faster.py:123 and
// FastGS/train_faster.py:107), which computes the SSIM of 3DGS
// (3DGS/utils/loss_utils.py:33-63): 11-tap Gaussian window (sigma 1.5), zero
// padding, C1 = 0.01^2, C2 = 0.03^2,
//   m = (2 mu1 mu2 + C1)(2 s12 + C2) / ((mu1^2 + mu2^2 + C1)(s1 + s2 + C2)),
// with the map's partial derivatives w.r.t. mu1, E[x^2] and E[xy] for the
// backward dL/dx = G * (g dm/dmu1) + 2 x G * (g dm/dE[x^2]) + y G * (g dm/dE[xy]).
//
// GB300 layout: one CTA of 256 threads per 32x32 output tile of one plane;
// the plane region the tile needs (zero outside the image) is staged in
// shared memory once and every window sum is separable (horizontal pass into
// shared memory, vertical pass), each thread sliding a register window over
// K consecutive outputs so that one shared-memory load feeds K FMAs.
//
// fgs_l1_dssim fuses the whole loss of the training loop,
//   L = (1 - lambda) mean|x - y| + lambda (1 - mean m),
// and its gradient: a tile stages x and y with a 10-pixel halo, forms the
// map's partials on the tile plus a 5-pixel halo (scaled by dL/dm = -lambda/N),
// convolves them back and adds the L1 term, so the image and the target are
// read once and dL/dx is written once; per-tile partial sums of m and |x - y|
// are reduced by a second, one-block kernel (deterministic).
#include <cmath>

#include "internal.cuh"

namespace fgs {
namespace {

constexpr int kT = 32;          // output tile edge
constexpr int kRad = 5;         // window radius (11 taps)
constexpr int kTaps = 2 * kRad + 1;
constexpr int kSsimThreads = 256;

struct Taps {
  float w[kTaps];
};

// N x N regions of two planes whose top-left is (y0, x0), zero outside the
// image, into da / db (row stride N): four elements of each per thread and
// round, all eight loads issued before the shared-memory stores.
template <int N>
__device__ __forceinline__ void stage_two(float* __restrict__ da, float* __restrict__ db,
                                          const float* __restrict__ pa, const float* __restrict__ pb, int H, int W,
                                          int y0, int x0) {
  constexpr int kU = 4;
  for (int base = threadIdx.x; base < N * N; base += kU * kSsimThreads) {
    float va[kU], vb[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int i = base + u * kSsimThreads;
      const int r = i / N, c = i - r * N;
      const int y = y0 + r, x = x0 + c;
      const bool in = i < N * N && y >= 0 && y < H && x >= 0 && x < W;
      const size_t at = in ? (size_t)y * W + x : 0;
      va[u] = in ? __ldg(pa + at) : 0.f;
      vb[u] = in ? __ldg(pb + at) : 0.f;
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int i = base + u * kSsimThreads;
      if (i < N * N) {
        da[i] = va[u];
        db[i] = vb[u];
      }
    }
  }
}

// Horizontal window sums of the five moments x, y, x^2, y^2, xy of two staged
// regions (row stride ld_in): out[q][r * ld_out + c] for c < cols_out (a
// multiple of K), r < rows.
template <int K>
__device__ __forceinline__ void hpass_moments(const float* sx, const float* sy, int ld_in, float* out, int plane_out,
                                              int ld_out, int rows, int cols_out, const Taps& w) {
  const int segs = cols_out / K;
  for (int it = threadIdx.x; it < rows * segs; it += kSsimThreads) {
    const int r = it / segs, c0 = (it - r * segs) * K;
    float a[K][5];
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
      for (int q = 0; q < 5; ++q) a[k][q] = 0.f;
    const float* px = sx + r * ld_in + c0;
    const float* py = sy + r * ld_in + c0;
#pragma unroll
    for (int j = 0; j < K + kTaps - 1; ++j) {
      const float x = px[j], y = py[j];
      const float xx = x * x, yy = y * y, xy = x * y;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int t = j - k;
        if (t >= 0 && t < kTaps) {
          a[k][0] = fmaf(w.w[t], x, a[k][0]);
          a[k][1] = fmaf(w.w[t], y, a[k][1]);
          a[k][2] = fmaf(w.w[t], xx, a[k][2]);
          a[k][3] = fmaf(w.w[t], yy, a[k][3]);
          a[k][4] = fmaf(w.w[t], xy, a[k][4]);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
      for (int q = 0; q < 5; ++q) out[q * plane_out + r * ld_out + c0 + k] = a[k][q];
  }
}

// Horizontal window sums of NQ staged maps (map q at in + q * plane_in).
template <int K, int NQ>
__device__ __forceinline__ void hpass(const float* in, int plane_in, int ld_in, float* out, int plane_out, int ld_out,
                                      int rows, int cols_out, const Taps& w) {
  const int segs = cols_out / K;
  for (int it = threadIdx.x; it < rows * segs; it += kSsimThreads) {
    const int r = it / segs, c0 = (it - r * segs) * K;
    float a[K][NQ];
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
      for (int q = 0; q < NQ; ++q) a[k][q] = 0.f;
#pragma unroll
    for (int j = 0; j < K + kTaps - 1; ++j) {
      float v[NQ];
#pragma unroll
      for (int q = 0; q < NQ; ++q) v[q] = in[q * plane_in + r * ld_in + c0 + j];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int t = j - k;
        if (t >= 0 && t < kTaps) {
#pragma unroll
          for (int q = 0; q < NQ; ++q) a[k][q] = fmaf(w.w[t], v[q], a[k][q]);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
      for (int q = 0; q < NQ; ++q) out[q * plane_out + r * ld_out + c0 + k] = a[k][q];
  }
}

// Vertical window sums of NQ maps for output column c, rows [r0, r0 + K):
// res[k][q] = sum_t w[t] in[q][(r0 + k + t) * ld + c].
template <int K, int NQ>
__device__ __forceinline__ void vsums(const float* in, int plane_in, int ld, int r0, int c, const Taps& w,
                                      float (&res)[K][NQ]) {
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int q = 0; q < NQ; ++q) res[k][q] = 0.f;
#pragma unroll
  for (int j = 0; j < K + kTaps - 1; ++j) {
    float v[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) v[q] = in[q * plane_in + (r0 + j) * ld + c];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const int t = j - k;
      if (t >= 0 && t < kTaps) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) res[k][q] = fmaf(w.w[t], v[q], res[k][q]);
      }
    }
  }
}

// SSIM value and its partials from the five window moments (3DGS
// loss_utils.py:47-60; fused-ssim ssim.cu:262-283).
struct SsimPoint {
  float m, d_mu1, d_e11, d_e12;
};
__device__ __forceinline__ SsimPoint ssim_point(const float (&mo)[5], float C1, float C2) {
  const float mu1 = mo[0], mu2 = mo[1];
  const float mu1_sq = mu1 * mu1, mu2_sq = mu2 * mu2, mu12 = mu1 * mu2;
  const float s1 = mo[2] - mu1_sq, s2 = mo[3] - mu2_sq, s12 = mo[4] - mu12;
  const float Cn = 2.f * mu12 + C1, Dn = 2.f * s12 + C2;
  const float A = mu1_sq + mu2_sq + C1, B = s1 + s2 + C2;
  const float iAB = 1.f / (A * B);
  SsimPoint p;
  p.m = Cn * Dn * iAB;
  // dm/dmu1 through C, D (s12 = E[xy] - mu1 mu2), A and B (s1 = E[x^2] - mu1^2)
  p.d_mu1 = 2.f * iAB * (mu2 * Dn - mu2 * Cn - mu1 * p.m * B + mu1 * p.m * A);
  p.d_e11 = -p.m / B;        // dm/dE[x^2] = -C D / (A B^2)
  p.d_e12 = 2.f * Cn * iAB;  // dm/dE[xy] = 2 C / (A B)
  return p;
}

// ---------------------------------------------------------------------------
// Map and partials (fused-ssim forward, train=True when dm_* are given).
constexpr int kFwdRows = kT + 2 * kRad;  // 42: tile plus halo
struct FwdShared {
  float sx[kFwdRows * kFwdRows], sy[kFwdRows * kFwdRows];
  float h[5 * kFwdRows * kT];
};

__global__ void __launch_bounds__(kSsimThreads) k_ssim_fwd(int H, int W, float C1, float C2, const float* img1,
                                                           const float* img2, float* map, float* d_mu1,
                                                           float* d_e11, float* d_e12, Taps w) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  FwdShared& sh = *reinterpret_cast<FwdShared*>(s_raw);
  const int x0 = blockIdx.x * kT, y0 = blockIdx.y * kT;
  const size_t poff = (size_t)blockIdx.z * H * W;
  stage_two<kFwdRows>(sh.sx, sh.sy, img1 + poff, img2 + poff, H, W, y0 - kRad, x0 - kRad);
  __syncthreads();
  hpass_moments<4>(sh.sx, sh.sy, kFwdRows, sh.h, kFwdRows * kT, kT, kFwdRows, kT, w);
  __syncthreads();
  // vertical: column c, 4 rows per thread (32 columns x 8 segments = 256)
  const int c = threadIdx.x & 31, r0 = (threadIdx.x >> 5) * 4;
  float mo[4][5];
  vsums<4, 5>(sh.h, kFwdRows * kT, kT, r0, c, w, mo);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int y = y0 + r0 + k, x = x0 + c;
    if (y < H && x < W) {
      const SsimPoint p = ssim_point(mo[k], C1, C2);
      const size_t i = poff + (size_t)y * W + x;
      map[i] = p.m;
      if (d_mu1) {
        d_mu1[i] = p.d_mu1;
        d_e11[i] = p.d_e11;
        d_e12[i] = p.d_e12;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// dL/dimg1 from dL/dmap and the partial maps (fused-ssim backward).
struct BwdShared {
  float p[3 * kFwdRows * kFwdRows];
  float h[3 * kFwdRows * kT];
};

__global__ void __launch_bounds__(kSsimThreads) k_ssim_bwd(int H, int W, const float* img1, const float* img2,
                                                           const float* dL_dmap, const float* d_mu1,
                                                           const float* d_e11, const float* d_e12, float* dL_dimg1,
                                                           Taps w) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  BwdShared& sh = *reinterpret_cast<BwdShared*>(s_raw);
  const int x0 = blockIdx.x * kT, y0 = blockIdx.y * kT;
  const size_t poff = (size_t)blockIdx.z * H * W;
  constexpr int kP = kFwdRows * kFwdRows;
  for (int i = threadIdx.x; i < kP; i += kSsimThreads) {
    const int r = i / kFwdRows, cc = i - r * kFwdRows;
    const int y = y0 - kRad + r, x = x0 - kRad + cc;
    float a = 0.f, b = 0.f, e = 0.f;
    if (y >= 0 && y < H && x >= 0 && x < W) {
      const size_t j = poff + (size_t)y * W + x;
      const float g = __ldg(dL_dmap + j);
      a = g * __ldg(d_mu1 + j);
      b = g * __ldg(d_e11 + j);
      e = g * __ldg(d_e12 + j);
    }
    sh.p[i] = a;
    sh.p[kP + i] = b;
    sh.p[2 * kP + i] = e;
  }
  __syncthreads();
  hpass<4, 3>(sh.p, kP, kFwdRows, sh.h, kFwdRows * kT, kT, kFwdRows, kT, w);
  __syncthreads();
  const int c = threadIdx.x & 31, r0 = (threadIdx.x >> 5) * 4;
  float s[4][3];
  vsums<4, 3>(sh.h, kFwdRows * kT, kT, r0, c, w, s);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int y = y0 + r0 + k, x = x0 + c;
    if (y < H && x < W) {
      const size_t i = poff + (size_t)y * W + x;
      dL_dimg1[i] = s[k][0] + 2.f * __ldg(img1 + i) * s[k][1] + __ldg(img2 + i) * s[k][2];
    }
  }
}

// ---------------------------------------------------------------------------
// Fused loss: (1 - lambda) mean|x - y| + lambda (1 - mean SSIM) and dL/dx.
constexpr int kInRows = kT + 4 * kRad;  // 52: tile plus the partials' halo plus the window's
struct LossShared {
  union {
    struct {
      float sx[kInRows * kInRows], sy[kInRows * kInRows];
    } in;
    float p[3 * kFwdRows * kFwdRows];  // partials, once the inputs are consumed
  } a;
  union {
    float h1[5 * kInRows * kFwdRows];  // horizontal moments over the staged rows
    float h2[3 * kFwdRows * kT];       // horizontal sums of the partials
  } b;
  float red[2][kSsimThreads / 32];
};

__global__ void __launch_bounds__(kSsimThreads) k_l1_dssim(int H, int W, float C1, float C2, float lambda,
                                                           float inv_n, const float* img, const float* gt,
                                                           float* dL_dimg, float* block_sums, Taps w) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  LossShared& sh = *reinterpret_cast<LossShared*>(s_raw);
  const int x0 = blockIdx.x * kT, y0 = blockIdx.y * kT;
  const size_t poff = (size_t)blockIdx.z * H * W;
  const float* px = img + poff;
  const float* py = gt + poff;
  stage_two<kInRows>(sh.a.in.sx, sh.a.in.sy, px, py, H, W, y0 - 2 * kRad, x0 - 2 * kRad);
  __syncthreads();
  // moments for the tile plus a 5-pixel halo: 52 staged rows x 42 columns
  hpass_moments<6>(sh.a.in.sx, sh.a.in.sy, kInRows, sh.b.h1, kInRows * kFwdRows, kFwdRows, kInRows, kFwdRows, w);
  __syncthreads();
  // vertical: 42 columns x 7 segments of 6 rows; the partials, scaled by
  // dL/dm = -lambda / N and zero outside the image, replace the inputs
  constexpr int kP = kFwdRows * kFwdRows;
  float msum = 0.f;
  float mo[6][5];
  SsimPoint pt[6];
  bool in_img[6];
  for (int it = threadIdx.x; it < kFwdRows * 7; it += kSsimThreads) {
    const int cc = it % kFwdRows, r0 = (it / kFwdRows) * 6;
    vsums<6, 5>(sh.b.h1, kInRows * kFwdRows, kFwdRows, r0, cc, w, mo);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const int y = y0 - kRad + r0 + k, x = x0 - kRad + cc;
      in_img[k] = y >= 0 && y < H && x >= 0 && x < W;
      pt[k] = ssim_point(mo[k], C1, C2);
      // the tile's own pixels count towards the mean
      if (in_img[k] && r0 + k >= kRad && r0 + k < kRad + kT && cc >= kRad && cc < kRad + kT) msum += pt[k].m;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      mo[k][0] = in_img[k] ? -lambda * inv_n * pt[k].d_mu1 : 0.f;
      mo[k][1] = in_img[k] ? -lambda * inv_n * pt[k].d_e11 : 0.f;
      mo[k][2] = in_img[k] ? -lambda * inv_n * pt[k].d_e12 : 0.f;
    }
    // the staged inputs were last read by hpass_moments, before the barrier
    // above, so the partials can take their place
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const int i = (r0 + k) * kFwdRows + cc;
      sh.a.p[i] = mo[k][0];
      sh.a.p[kP + i] = mo[k][1];
      sh.a.p[2 * kP + i] = mo[k][2];
    }
  }
  __syncthreads();
  hpass<4, 3>(sh.a.p, kP, kFwdRows, sh.b.h2, kFwdRows * kT, kT, kFwdRows, kT, w);
  __syncthreads();
  const int c = threadIdx.x & 31, r0 = (threadIdx.x >> 5) * 4;
  float s[4][3];
  vsums<4, 3>(sh.b.h2, kFwdRows * kT, kT, r0, c, w, s);
  float l1 = 0.f;
  const float wl1 = (1.f - lambda) * inv_n;
  float xv[4], yv[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {  // loads first, then the stores
    const int y = y0 + r0 + k, x = x0 + c;
    const bool in = y < H && x < W;
    const size_t i = in ? (size_t)y * W + x : 0;
    xv[k] = in ? __ldg(px + i) : 0.f;
    yv[k] = in ? __ldg(py + i) : 0.f;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int y = y0 + r0 + k, x = x0 + c;
    if (y < H && x < W) {
      const float d = xv[k] - yv[k];
      l1 += fabsf(d);
      const float sg = d > 0.f ? 1.f : (d < 0.f ? -1.f : 0.f);  // d|d|/dd as torch.abs (0 at 0)
      dL_dimg[poff + (size_t)y * W + x] = s[k][0] + 2.f * xv[k] * s[k][1] + yv[k] * s[k][2] + wl1 * sg;
    }
  }
  // per-tile sums of m and |x - y|
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    msum += __shfl_xor_sync(0xffffffffu, msum, o);
    l1 += __shfl_xor_sync(0xffffffffu, l1, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sh.red[0][threadIdx.x >> 5] = msum;
    sh.red[1][threadIdx.x >> 5] = l1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.f, b = 0.f;
    for (int j = 0; j < kSsimThreads / 32; ++j) {
      a += sh.red[0][j];
      b += sh.red[1][j];
    }
    const size_t blk = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    block_sums[2 * blk] = a;
    block_sums[2 * blk + 1] = b;
  }
}

// loss = (1 - lambda) * (sum |x - y|) / N + lambda * (1 - (sum m) / N), one block,
// fixed order (deterministic).
__global__ void __launch_bounds__(1024) k_loss_reduce(const float* block_sums, long long nblk, float lambda,
                                                      float inv_n, float* loss, float* ssim_mean) {
  __shared__ double s_m[32], s_l[32];
  double m = 0.0, l = 0.0;
  for (long long j = threadIdx.x; j < nblk; j += 1024) {
    m += (double)block_sums[2 * j];
    l += (double)block_sums[2 * j + 1];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    m += __shfl_xor_sync(0xffffffffu, m, o);
    l += __shfl_xor_sync(0xffffffffu, l, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s_m[threadIdx.x >> 5] = m;
    s_l[threadIdx.x >> 5] = l;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int j = 0; j < 32; ++j) {
      a += s_m[j];
      b += s_l[j];
    }
    const double mean_m = a * (double)inv_n, mean_l1 = b * (double)inv_n;
    if (ssim_mean) *ssim_mean = (float)mean_m;
    *loss = (float)((1.0 - (double)lambda) * mean_l1 + (double)lambda * (1.0 - mean_m));
  }
}

Taps window_taps() {
  // Normalised Gaussian of sigma 1.5 over 11 taps (3DGS loss_utils.py:23-25),
  // formed in double and rounded once.
  double g[kTaps], sum = 0.0;
  for (int t = 0; t < kTaps; ++t) {
    const double d = (double)(t - kRad);
    g[t] = std::exp(-d * d / (2.0 * 1.5 * 1.5));
    sum += g[t];
  }
  Taps w;
  for (int t = 0; t < kTaps; ++t) w.w[t] = (float)(g[t] / sum);
  return w;
}

bool planes_ok(int planes, int H, int W) {
  return planes > 0 && H > 0 && W > 0 && planes <= 65535 && (int64_t)planes * H * W < ((int64_t)1 << 40);
}

}  // namespace
}  // namespace fgs

using namespace fgs;

extern "C" size_t fgs_l1_dssim_scratch_bytes(int planes, int H, int W) {
  if (!planes_ok(planes, H, W)) return 0;
  const size_t nblk = (size_t)planes * ((H + kT - 1) / kT) * ((W + kT - 1) / kT);
  return 2 * sizeof(float) * nblk;
}

extern "C" fgs_status fgs_ssim_fwd(int planes, int H, int W, float C1, float C2, const float* img1, const float* img2,
                                   float* ssim_map, float* dm_dmu1, float* dm_dsigma1_sq, float* dm_dsigma12,
                                   void* stream) {
  if (!planes_ok(planes, H, W) || !img1 || !img2 || !ssim_map) return FGS_ERR_BAD_ARG;
  const bool partials = dm_dmu1 || dm_dsigma1_sq || dm_dsigma12;
  if (partials && (!dm_dmu1 || !dm_dsigma1_sq || !dm_dsigma12)) return FGS_ERR_BAD_ARG;
  const int smem = (int)sizeof(FwdShared);
  FGS_TRY(allow_dyn_smem(reinterpret_cast<const void*>(&k_ssim_fwd), smem));
  const dim3 grid((W + kT - 1) / kT, (H + kT - 1) / kT, planes);
  k_ssim_fwd<<<grid, kSsimThreads, smem, (cudaStream_t)stream>>>(H, W, C1, C2, img1, img2, ssim_map, dm_dmu1,
                                                                   dm_dsigma1_sq, dm_dsigma12, window_taps());
  FGS_LAUNCH_CHECK();
  return FGS_OK;
}

extern "C" fgs_status fgs_ssim_bwd(int planes, int H, int W, const float* img1, const float* img2,
                                   const float* dL_dmap, const float* dm_dmu1, const float* dm_dsigma1_sq,
                                   const float* dm_dsigma12, float* dL_dimg1, void* stream) {
  if (!planes_ok(planes, H, W) || !img1 || !img2 || !dL_dmap || !dm_dmu1 || !dm_dsigma1_sq || !dm_dsigma12 ||
      !dL_dimg1)
    return FGS_ERR_BAD_ARG;
  const int smem = (int)sizeof(BwdShared);
  FGS_TRY(allow_dyn_smem(reinterpret_cast<const void*>(&k_ssim_bwd), smem));
  const dim3 grid((W + kT - 1) / kT, (H + kT - 1) / kT, planes);
  k_ssim_bwd<<<grid, kSsimThreads, smem, (cudaStream_t)stream>>>(H, W, img1, img2, dL_dmap, dm_dmu1, dm_dsigma1_sq,
                                                                   dm_dsigma12, dL_dimg1, window_taps());
  FGS_LAUNCH_CHECK();
  return FGS_OK;
}

extern "C" fgs_status fgs_l1_dssim(int planes, int H, int W, float lambda, const float* img, const float* gt,
                                   void* scratch, size_t scratch_bytes, float* loss, float* ssim_mean,
                                   float* dL_dimg, void* stream) {
  if (!planes_ok(planes, H, W) || !img || !gt || !scratch || !loss || !dL_dimg) return FGS_ERR_BAD_ARG;
  if (((uintptr_t)scratch & 7) != 0) return FGS_ERR_BAD_ARG;
  if (scratch_bytes < fgs_l1_dssim_scratch_bytes(planes, H, W)) return FGS_ERR_CAPACITY;
  const int smem = (int)sizeof(LossShared);
  FGS_TRY(allow_dyn_smem(reinterpret_cast<const void*>(&k_l1_dssim), smem));
  const dim3 grid((W + kT - 1) / kT, (H + kT - 1) / kT, planes);
  const long long nblk = (long long)grid.x * grid.y * grid.z;
  const float inv_n = (float)(1.0 / ((double)planes * H * W));
  float* sums = static_cast<float*>(scratch);
  cudaStream_t s = (cudaStream_t)stream;
  const float C1 = (float)(0.01 * 0.01), C2 = (float)(0.03 * 0.03);  // fused_ssim/__init__.py:46-47
  KernelTimer kt__(FGS_K_LOSS, s);
  k_l1_dssim<<<grid, kSsimThreads, smem, s>>>(H, W, C1, C2, lambda, inv_n, img, gt, dL_dimg, sums, window_taps());
  kt__.stop();
  FGS_LAUNCH_CHECK();
  k_loss_reduce<<<1, 1024, 0, s>>>(sums, nblk, lambda, inv_n, loss, ssim_mean);
  FGS_LAUNCH_CHECK();
  return FGS_OK;
}
