// Library-wide C entry points: status strings, device error word, SM count
// cache, and the masked Adam step.
#include <mutex>

#include "fgs_common.cuh"

namespace fgs {

int num_sms() {
  // Cached per device; cudaDeviceGetAttribute is cheap but not free.
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (cache[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
    cache[dev] = n;
  }
  return cache[dev];
}

namespace {
// Masked Adam over N rows of M values (FB adam.cu:9-38).
__global__ void __launch_bounds__(256) k_adam(float* __restrict__ param, const float* __restrict__ grad,
                                              float* __restrict__ m1, float* __restrict__ m2,
                                              const uint8_t* __restrict__ visible, float lr, float b1, float b2,
                                              float eps, uint32_t N, uint32_t M) {
  const uint64_t p = blockIdx.x * 256ull + threadIdx.x;
  const uint64_t row = p / M;
  if (row >= N) return;
  if (!visible[row]) return;
  const float g = grad[p];
  const float a = b1 * m1[p] + (1.0f - b1) * g;
  const float b = b2 * m2[p] + (1.0f - b2) * g * g;
  param[p] += -lr * a / (sqrtf(b) + eps);
  m1[p] = a;
  m2[p] = b;
}
}  // namespace

}  // namespace fgs

extern "C" const char* fgs_status_string(int status) {
  switch (status) {
    case FGS_OK: return "ok";
    case FGS_ERR_BAD_ARG: return "bad argument (null, misaligned, or inconsistent sizes)";
    case FGS_ERR_CAPACITY: return "a caller-provided buffer is too small";
    case FGS_ERR_CUDA: return "CUDA runtime error";
    case FGS_ERR_TIMEOUT: return "a bounded device-side wait expired";
    case FGS_ERR_UNSUPPORTED: return "not supported by this build";
    default: return "unknown status";
  }
}

extern "C" const char* fgs_version(void) { return "fgs 0.1 sm_103a"; }

extern "C" fgs_status fgs_device_errors(int* flags, int clear, void* stream) {
  if (!flags) return FGS_ERR_BAD_ARG;
  *flags = 0;
  cudaStream_t s = (cudaStream_t)stream;
  const bool c = clear != 0;
  FGS_TRY(fgs::errors_preprocess(flags, c, s));
  FGS_TRY(fgs::errors_sort(flags, c, s));
  FGS_TRY(fgs::errors_render(flags, c, s));
  FGS_TRY(fgs::errors_backward(flags, c, s));
  return FGS_OK;
}

extern "C" fgs_status fgs_adam_update(float* param, const float* grad, float* exp_avg, float* exp_avg_sq,
                                      const uint8_t* visible, float lr, float b1, float b2, float eps, uint32_t N,
                                      uint32_t M, void* stream) {
  if (M == 0) return FGS_ERR_BAD_ARG;
  const uint64_t cnt = (uint64_t)N * M;
  if (cnt == 0) return FGS_OK;
  if (!param || !grad || !exp_avg || !exp_avg_sq || !visible) return FGS_ERR_BAD_ARG;
  fgs::k_adam<<<(unsigned)((cnt + 255) / 256), 256, 0, (cudaStream_t)stream>>>(param, grad, exp_avg, exp_avg_sq,
                                                                               visible, lr, b1, b2, eps, N, M);
  FGS_LAUNCH_CHECK();
  return FGS_OK;
}
