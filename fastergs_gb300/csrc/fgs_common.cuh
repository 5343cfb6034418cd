// Shared device helpers of the sm_103a rasterizer.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fgs.h"

namespace fgs {

// Splat record field offsets: one 32-float (128-byte) record per Gaussian,
// the same field map as FB (rasterizer_imp.h:27-38) so records are
// interchangeable between the two implementations.
enum : int {
  F_XY = 0,       // pixel x, y
  F_RGBD = 2,     // r, g, b, view depth
  F_CONO = 6,     // (-0.5 log2e a, -log2e b, -0.5 log2e c, log2 opacity)
  F_RMIN = 10,    // tile rect min (int bits)
  F_RMAX = 12,    // tile rect max (int bits)
  F_CONIC = 14,   // conic a, b, c
  F_PVIEW = 17,   // view-space position
  F_POWER = 20,   // ln(256 opacity) * mult
  F_CLAMP = 22,   // SH clamp flags (1.0 = clamped)
  F_COV3D = 25,   // upper triangle of the 3D covariance
};

constexpr int kWarp = 32;
// Gaussians whose tile rect reaches this many tiles take the split path
// (FB rasterizer_imp.h:40-41: large_threshold / large_split_tile_count).
constexpr int kLargeTiles = 128;

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
__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
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

// Column-major 4x4 transforms, as the 3DGS matrices are laid out.
__device__ __forceinline__ float3 xform_point3(const float* m, float3 p) {
  return make_float3(m[0] * p.x + m[4] * p.y + m[8] * p.z + m[12], m[1] * p.x + m[5] * p.y + m[9] * p.z + m[13],
                     m[2] * p.x + m[6] * p.y + m[10] * p.z + m[14]);
}
__device__ __forceinline__ float4 xform_point4(const float* m, float3 p) {
  return make_float4(m[0] * p.x + m[4] * p.y + m[8] * p.z + m[12], m[1] * p.x + m[5] * p.y + m[9] * p.z + m[13],
                     m[2] * p.x + m[6] * p.y + m[10] * p.z + m[14], m[3] * p.x + m[7] * p.y + m[11] * p.z + m[15]);
}

// Device error word; one per translation unit (no relocatable device code),
// each unit exposes it through FGS_DEFINE_ERROR_ACCESSOR.
static __device__ int g_error_word;
__device__ __forceinline__ void raise_error(int bits) { atomicOr(&g_error_word, bits); }

// Host helpers.
int num_sms();
cudaError_t errors_preprocess(int* out, bool clear, cudaStream_t s);
cudaError_t errors_sort(int* out, bool clear, cudaStream_t s);
cudaError_t errors_render(int* out, bool clear, cudaStream_t s);
cudaError_t errors_backward(int* out, bool clear, cudaStream_t s);
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

#define FGS_DEFINE_ERROR_ACCESSOR(name)                                                        \
  namespace fgs {                                                                             \
  cudaError_t errors_##name(int* out, bool clear, cudaStream_t s) {                           \
    int v = 0;                                                                                \
    cudaError_t e = cudaMemcpyFromSymbolAsync(&v, g_error_word, sizeof(int), 0,               \
                                              cudaMemcpyDeviceToHost, s);                     \
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);                                       \
    if (e == cudaSuccess && clear && v) {                                                     \
      const int z = 0;                                                                        \
      e = cudaMemcpyToSymbolAsync(g_error_word, &z, sizeof(int), 0, cudaMemcpyHostToDevice, s); \
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);                                     \
    }                                                                                         \
    *out |= v;                                                                                \
    return e;                                                                                 \
  }                                                                                           \
  }
