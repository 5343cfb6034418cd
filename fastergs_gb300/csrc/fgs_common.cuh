// Shared device helpers of the sm_103a rasterizer.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

#include "../../include/fgs.h"

namespace fgs {

// Splat record: 32 floats (128 bytes) per Gaussian.  It holds every field of
// FB's record (rasterizer_imp.h:27-38) but orders them so the 12 floats the
// compositing kernels read come first (three 16-byte loads, two sectors), and
// it stores the footprint in a form that keeps full FP32 accuracy:
//   * the exponent of alpha is log2(o) + A1 (dx + P dy)^2 + C1 dy^2, a sum of
//     non-positive terms (FB's a dx^2 + 2b dx dy + c dy^2 cancels for thin,
//     elongated footprints);
//   * the pixel position is floor(x) + fx with fx taken from an FP64
//     projection, so dx = (floor(x) - px) + fx is exact to ~1e-7 px (an FP32
//     x near 1000 px is only good to 6e-5 px).
enum : int {
  F_XY = 0,       // pixel x, y (FP32, as FB stores them)
  F_RGB = 2,      // r, g, b
  F_DEPTH = 5,    // view depth (key source)
  F_CHOL = 6,     // A1 = -0.5 log2e conic_a, P = conic_b / conic_a, C1 = -0.5 log2e / cov_c
  F_LOG2O = 9,    // log2 opacity
  F_FRAC = 10,    // x - floor(float(x)), y - floor(float(y)) from the FP64 projection
  F_RMIN = 12,    // tile rect min (int bits)
  F_RMAX = 14,    // tile rect max (int bits)
  F_CONIC = 16,   // conic a, b, c
  F_POWER = 19,   // ln(256 opacity) * mult
  F_CLAMP = 20,   // SH clamp flags (1.0 = clamped)
  F_COV3D = 23,   // upper triangle of the 3D covariance
  F_PVIEW = 29,   // view-space position
};

constexpr int kWarp = 32;
// Gaussians whose tile rect reaches this many tiles take the split path
// (FB rasterizer_imp.h:40-41: large_threshold / large_split_tile_count).
constexpr int kLargeTiles = 128;
// Candidate tiles of small footprints each lane tests per step of the
// preprocess's flattened candidate list in the plain entry points (the
// autotuner's packet for the batched ones).
constexpr int kPacket = 1;

constexpr float kLn2 = 0.69314718055994531f;
constexpr float kLog2e = 1.44269504088896341f;
constexpr float kAlphaCut = 1.0f / 255.0f;
constexpr float kAlphaMax = 0.99f;
constexpr float kTMin = 1e-4f;

// Error word bits (fgs_device_errors).
constexpr int kErrTimeout = 1;
constexpr int kErrCapacity = 2;

// Upper bound on polling iterations of any device-side wait.
constexpr int kSpinLimit = 1 << 22;

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// Float-float arithmetic: a value is hi + lo with |lo| <= ulp(hi) / 2, good to
// about 44 bits.  Built from the error-free transforms TwoSum (Knuth, TAOCP
// vol. 2, 4.2.2) and the FMA product (Dekker 1971 with a fused multiply-add).
// Explicit _rn intrinsics keep the compiler from contracting the transforms.
// On sm_103 FP64 issues at a small fraction of the FP32 rate, so this is the
// cheap way to get pixel positions far below FP32 resolution.
struct ff {
  float hi, lo;
};
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ ff ff_fast_sum(float a, float b) {  // needs |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff ff_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const ff s = ff_two_sum(a.hi, b.hi);
  return ff_fast_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ ff ff_add_f(ff a, float b) {
  const ff s = ff_two_sum(a.hi, b);
  return ff_fast_sum(s.hi, __fadd_rn(s.lo, a.lo));
}
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
  const ff p = ff_prod(a.hi, b);
  return ff_fast_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}
// a / b: quotient of the leading parts, then one correction from the exact
// remainder a - q1 b.
__device__ __forceinline__ ff ff_div(ff a, ff b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const ff p = ff_prod(q1, b.hi);
  float r = __fsub_rn(a.hi, p.hi);
  r = __fsub_rn(r, p.lo);
  r = __fadd_rn(r, a.lo);
  r = __fmaf_rn(-q1, b.lo, r);
  return ff_fast_sum(q1, __fdiv_rn(r, b.hi));
}

// Packed FP32 pairs (sm_100+ f32x2 arithmetic): one instruction does the
// work of two scalar ones with identical per-element IEEE rounding, which
// halves the issue slots of the compositing kernels' FMA-heavy inner loops.
typedef unsigned long long f2x;
__device__ __forceinline__ f2x f2_pack(float lo, float hi) {
  f2x r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2_unpack(f2x v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2x f2_fma(f2x a, f2x b, f2x c) {
  f2x d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2x f2_mul(f2x a, f2x b) {
  f2x d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2x f2_add(f2x a, f2x b) {
  f2x d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2x f2_sub(f2x a, f2x b) {
  f2x d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// Programmatic dependent launch (sm_90+).  Kernels of the path start with
// pdl_wait(), which returns once the preceding kernel in the stream has
// completed and its writes are visible (immediately for a kernel launched
// without the attribute), then pdl_trigger(), which lets the next kernel's
// launch begin while this one's blocks run.  launch_pdl() launches with the
// attribute, so a kernel's launch and prologue overlap its predecessor's last
// wave instead of following its completion.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args&&... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}
// Vector reduction into global memory (sm_90+): one instruction, 16 bytes.
__device__ __forceinline__ void red_add_v4(float* addr, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b), "f"(c), "f"(d)
               : "memory");
}
__device__ __forceinline__ uint32_t ld_volatile_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_volatile_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Row of element j of a span of rows `row` elements wide, in FP32 from the
// correctly rounded inv_row = 1 / row: floor((j + 1/2) inv_row), equal to
// j / row for j < 256 row with 3 <= row <= 48 (SH rows) and for j < 256 with
// 1 <= row <= 255 (tile rectangles); tests/test_capi_cpu.py checks every row
// and j of both ranges.
__device__ __forceinline__ int row_of(int j, float inv_row) { return (int)(((float)j + 0.5f) * inv_row); }

// Block-cooperative copy into shared memory (16-byte aligned dst) of the rows
// of `nrows` consecutive rows, `row` floats each, that start at src + first
// and whose keep flag is set, with 16-byte loads when the source allows:
// turns per-thread strided reads of a Gaussian's coefficient row (180 bytes
// apart at SH degree 3) into coalesced ones, and skips the rows that are not
// needed (the floats of a skipped row are left as they were; a 16-byte piece
// shared with a kept row is copied).  No barrier; the caller syncs.
// Asynchronous form (cp.async, 16 bytes at a time, L2 only): issues the copy
// and returns; the caller does other work, then cp.async.wait_group 0 and a
// block barrier before reading dst.  An unaligned source or tail is copied
// synchronously.
__device__ __forceinline__ void block_copy_rows_to_smem_async(float* dst, const float* src, size_t first,
                                                              int nrows, int row, const uint8_t* keep) {
  const float* s = src + first;
  const int n = nrows * row;
  const float inv_row = 1.f / (float)row;
  int done = 0;
  if ((reinterpret_cast<uintptr_t>(s) & 15) == 0 && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
    const int n4 = n >> 2;
    for (int j = threadIdx.x; j < n4; j += blockDim.x) {
      if (!(keep[row_of(4 * j, inv_row)] | keep[row_of(4 * j + 3, inv_row)])) continue;
      const uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst + 4 * j));
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(s + 4 * j) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    done = 4 * n4;
  }
  for (int j = done + threadIdx.x; j < n; j += blockDim.x)
    if (keep[row_of(j, inv_row)]) dst[j] = __ldg(s + j);
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Synchronous form of block_copy_rows_to_smem_async; keep == nullptr copies every row.
__device__ __forceinline__ void block_copy_rows_to_smem(float* dst, const float* src, size_t first, int nrows,
                                                        int row, const uint8_t* keep) {
  const float* s = src + first;
  const int n = nrows * row;
  const float inv_row = 1.f / (float)row;
  int done = 0;
  if ((reinterpret_cast<uintptr_t>(s) & 15) == 0) {
    const int n4 = n >> 2;
    for (int j = threadIdx.x; j < n4; j += blockDim.x)
      if (!keep || (keep[row_of(4 * j, inv_row)] | keep[row_of(4 * j + 3, inv_row)]))
        reinterpret_cast<float4*>(dst)[j] = __ldg(reinterpret_cast<const float4*>(s) + j);
    done = 4 * n4;
  }
  for (int j = done + threadIdx.x; j < n; j += blockDim.x)
    if (!keep || keep[row_of(j, inv_row)]) dst[j] = __ldg(s + j);
}
// The reverse: n floats from shared memory to dst + first.
__device__ __forceinline__ void block_copy_from_smem(float* dst, size_t first, const float* src, int n) {
  float* d = dst + first;
  if ((reinterpret_cast<uintptr_t>(d) & 15) == 0) {
    const int n4 = n >> 2;
    for (int j = threadIdx.x; j < n4; j += blockDim.x)
      reinterpret_cast<float4*>(d)[j] = reinterpret_cast<const float4*>(src)[j];
    for (int j = 4 * n4 + threadIdx.x; j < n; j += blockDim.x) d[j] = src[j];
  } else {
    for (int j = threadIdx.x; j < n; j += blockDim.x) d[j] = src[j];
  }
}
// Largest SH coefficient count per Gaussian that is staged in shared memory.
constexpr int kMaxStagedCoeffs = 16;

// One element of FB's masked Adam step (adam.cu:27-36); lr carries the bias
// compensation.  Shared by the plain and the fused update so both round alike.
// The moments are FB's to the bit; the step -lr m / (sqrt(v) + eps) uses the
// hardware square root and reciprocal (relative error about 2^-22 of a step
// of size ~lr) instead of the IEEE-rounded sequences, which cost the fused
// preprocess backward a large share of its instructions.
__device__ __forceinline__ void adam_reg(float& param, float& m1, float& m2, float g, float lr, float b1, float b2,
                                         float eps) {
  const float a = b1 * m1 + (1.0f - b1) * g;
  const float b = b2 * m2 + (1.0f - b2) * g * g;
  param += (-lr * a) * rcp_approx(sqrt_approx(b) + eps);
  m1 = a;
  m2 = b;
}
__device__ __forceinline__ void adam_step(float* param, float* m1, float* m2, size_t k, float g, float lr, float b1,
                                          float b2, float eps) {
  float p = param[k], a = m1[k], b = m2[k];
  adam_reg(p, a, b, g, lr, b1, b2, eps);
  param[k] = p;
  m1[k] = a;
  m2[k] = b;
}

// Column-major 4x4 transforms, as the 3DGS matrices are laid out.
__device__ __forceinline__ float3 xform_point3(const float* m, float3 p) {
  return make_float3(m[0] * p.x + m[4] * p.y + m[8] * p.z + m[12], m[1] * p.x + m[5] * p.y + m[9] * p.z + m[13],
                     m[2] * p.x + m[6] * p.y + m[10] * p.z + m[14]);
}
__device__ __forceinline__ float4 xform_point4(const float* m, float3 p) {
  return make_float4(m[0] * p.x + m[4] * p.y + m[8] * p.z + m[12], m[1] * p.x + m[5] * p.y + m[9] * p.z + m[13],
                     m[2] * p.x + m[6] * p.y + m[10] * p.z + m[14], m[3] * p.x + m[7] * p.y + m[11] * p.z + m[15]);
}

// Cameras of one frame batch.  The plain (single-view) entry points use one
// view; the batched entry points render up to kMaxViews cameras of different
// resolutions in one launch per stage.  Tiles of all views share one global
// tile index space (view k owns tiles [tile_off, tile_off + gx*gy)) so that a
// single sort orders every view's pairs, and per-pixel arrays of all views are
// concatenated (view k starts at pixel pix_off).  Passed to kernels by value.
constexpr int kMaxViews = 32;
struct ViewDesc {
  const float* view;    // 4x4 column-major world -> view (device)
  const float* proj;    // 4x4 column-major full projection (device)
  const float* campos;  // 3 (device)
  const float* bg;      // 3 (device), compositing only
  float tanx, tany, fx, fy, mult, smod;
  int W, H, gx, gy;
  uint32_t tile_off, pix_off;
};
struct Views {
  int V, bx, by;
  uint32_t tiles;  // total tiles of all views
  ViewDesc v[kMaxViews];
  // view owning global tile t
  __device__ __forceinline__ int of_tile(uint32_t t) const {
    int k = 0;
    for (int j = 1; j < V; ++j)
      if (v[j].tile_off <= t) k = j;
    return k;
  }
};
inline void set_view(ViewDesc& d, int W, int H, int bx, int by, const float* view, const float* proj,
                     const float* campos, const float* bg, float tanx, float tany, float mult, float smod) {
  d.view = view; d.proj = proj; d.campos = campos; d.bg = bg;
  d.tanx = tanx; d.tany = tany; d.fx = W / (2.0f * tanx); d.fy = H / (2.0f * tany);
  d.mult = mult; d.smod = smod;
  d.W = W; d.H = H; d.gx = (W + bx - 1) / bx; d.gy = (H + by - 1) / by;
  d.tile_off = 0; d.pix_off = 0;
}
// One-view table for the plain entry points.
inline Views single_view(int W, int H, int bx, int by, const float* view, const float* proj, const float* campos,
                         const float* bg, float tanx, float tany, float mult, float smod) {
  Views vs;
  vs.V = 1; vs.bx = bx; vs.by = by;
  set_view(vs.v[0], W, H, bx, by, view, proj, campos, bg, tanx, tany, mult, smod);
  vs.tiles = (uint32_t)(vs.v[0].gx * vs.v[0].gy);
  return vs;
}

// Kahan's 2x2 determinant a*d - b*c with one rounding of the cancelling part.
__device__ __forceinline__ float det2_kahan(float a, float b, float c, float d) {
  const float w = b * c;
  const float e = fmaf(-b, c, w);
  const float f = fmaf(a, d, -w);
  return f + e;
}

// Screen covariance of a 3D Gaussian Sigma = R diag(s2) R^T seen through the
// 2x3 EWA Jacobian M:  Sigma2 = N diag(s2) N^T + 0.3 I with N = M R.  The
// determinant is the Cauchy-Binet sum of squared 2x2 minors plus the
// low-pass terms, all non-negative, so it keeps full FP32 accuracy for thin,
// elongated footprints where a*c - b*b cancels (the relative error of the
// latter grows with the footprint's condition number).
struct ScreenCov {
  float a, b, c, det;   // a, c include the 0.3 low-pass
  float N0[3], N1[3];   // rows of M R
};
__device__ __forceinline__ ScreenCov screen_cov(const float M0[3], const float M1[3], const float R[3][3],
                                                const float s2[3]) {
  ScreenCov r;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    r.N0[k] = M0[0] * R[0][k] + M0[1] * R[1][k] + M0[2] * R[2][k];
    r.N1[k] = M1[0] * R[0][k] + M1[1] * R[1][k] + M1[2] * R[2][k];
  }
  const float ap = s2[0] * r.N0[0] * r.N0[0] + s2[1] * r.N0[1] * r.N0[1] + s2[2] * r.N0[2] * r.N0[2];
  const float cp = s2[0] * r.N1[0] * r.N1[0] + s2[1] * r.N1[1] * r.N1[1] + s2[2] * r.N1[2] * r.N1[2];
  r.b = s2[0] * r.N0[0] * r.N1[0] + s2[1] * r.N0[1] * r.N1[1] + s2[2] * r.N0[2] * r.N1[2];
  const float m01 = det2_kahan(r.N0[0], r.N0[1], r.N1[0], r.N1[1]);
  const float m02 = det2_kahan(r.N0[0], r.N0[2], r.N1[0], r.N1[2]);
  const float m12 = det2_kahan(r.N0[1], r.N0[2], r.N1[1], r.N1[2]);
  const float detp = s2[0] * s2[1] * m01 * m01 + s2[0] * s2[2] * m02 * m02 + s2[1] * s2[2] * m12 * m12;
  r.a = ap + 0.3f;
  r.c = cp + 0.3f;
  r.det = detp + 0.3f * (ap + cp) + 0.09f;
  return r;
}

// Device error word; one per translation unit (no relocatable device code),
// each unit exposes it through FGS_DEFINE_ERROR_ACCESSOR.
static __device__ int g_error_word;
__device__ __forceinline__ void raise_error(int bits) { atomicOr(&g_error_word, bits); }

// Host helpers.
int num_sms();
// Device address of each translation unit's error word (looked up once).
int* error_word_preprocess();
int* error_word_sort();
int* error_word_render();
int* error_word_backward();
int* error_word_aux();
// Optional per-kernel event timing (fgs_kernel_timer).  Usage around a launch:
//   KernelTimer kt(FGS_K_RENDER_FWD, stream); launch...; kt.stop();
// `kernels`: how many kernel launches the timed region holds.
void timer_begin(int id, cudaStream_t s);
void timer_end(int id, cudaStream_t s, int kernels);
struct KernelTimer {
  int id;
  cudaStream_t s;
  int kernels;
  KernelTimer(int id_, cudaStream_t s_, int kernels_ = 1) : id(id_), s(s_), kernels(kernels_) { timer_begin(id, s); }
  void stop() { timer_end(id, s, kernels); }
};
// Opts a kernel into `bytes` of dynamic shared memory on the current device,
// once per (kernel, device); the first launch happens before any capture.
cudaError_t allow_dyn_smem(const void* kernel, int bytes);
inline int tile_bits(uint32_t tiles) {
  int b = 0;
  while (b < 32 && (1u << b) < tiles) ++b;
  return b;
}

}  // namespace fgs

#define FGS_TRY(expr)                                 \
  do {                                                \
    cudaError_t e__ = (expr);                         \
    if (e__ != cudaSuccess) return FGS_ERR_CUDA;      \
  } while (0)

#define FGS_LAUNCH_CHECK()                            \
  do {                                                \
    cudaError_t e__ = cudaGetLastError();             \
    if (e__ != cudaSuccess) return FGS_ERR_CUDA;      \
  } while (0)

#define FGS_DEFINE_ERROR_ACCESSOR(name)                                     \
  namespace fgs {                                                          \
  int* error_word_##name() {                                               \
    void* p = nullptr;                                                     \
    return cudaGetSymbolAddress(&p, g_error_word) == cudaSuccess           \
               ? static_cast<int*>(p)                                      \
               : nullptr;                                                  \
  }                                                                        \
  }
