// Library-wide C entry points: status strings, device error word, SM count
// cache, and the masked Adam step.
#include <algorithm>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "fgs_common.cuh"

namespace fgs {

namespace {
// Zero fill as a kernel of the launch chain (a memset node would break the
// programmatic dependent launches around it), of up to two byte ranges in one
// launch: the 16-byte-aligned middle with vector stores, the ragged head and
// tail byte by byte.
struct ZeroRange {
  unsigned char* p;
  size_t head, n16, tail;
};
ZeroRange zero_range(void* ptr, size_t bytes) {
  ZeroRange r{static_cast<unsigned char*>(ptr), 0, 0, 0};
  if (!ptr || bytes == 0) return r;
  r.head = std::min<size_t>(bytes, (16 - (reinterpret_cast<uintptr_t>(ptr) & 15)) & 15);
  r.n16 = (bytes - r.head) / 16;
  r.tail = bytes - r.head - 16 * r.n16;
  return r;
}
__device__ __forceinline__ void zero_fill(const ZeroRange& r, size_t t, size_t stride) {
  uint4* mid = reinterpret_cast<uint4*>(r.p + r.head);
  for (size_t i = t; i < r.n16; i += stride) mid[i] = make_uint4(0u, 0u, 0u, 0u);
  if (t < r.head) r.p[t] = 0;
  if (t < r.tail) r.p[r.head + 16 * r.n16 + t] = 0;
}
__global__ void __launch_bounds__(256) k_zero(ZeroRange r0, ZeroRange r1) {
  pdl_wait();
  pdl_trigger();
  const size_t t = blockIdx.x * 256ull + threadIdx.x, stride = (size_t)gridDim.x * 256;
  zero_fill(r0, t, stride);
  zero_fill(r1, t, stride);
}
}  // namespace

fgs_status zero_async(void* ptr, size_t bytes, cudaStream_t s, void* ptr2, size_t bytes2) {
  const ZeroRange r0 = zero_range(ptr, bytes), r1 = zero_range(ptr2, bytes2);
  if (r0.head + r0.n16 + r0.tail + r1.head + r1.n16 + r1.tail == 0) return FGS_OK;
  KernelTimer kt__(FGS_K_ZERO, s);
  const size_t want = (r0.n16 + r1.n16 + 1023) / 1024;  // about four 16-byte stores per thread
  const unsigned blocks = (unsigned)std::max<size_t>(1, std::min<size_t>(want, (size_t)num_sms() * 8));
  (void)launch_pdl(k_zero, dim3(blocks), dim3(256), 0, s, r0, r1);
  kt__.stop();
  FGS_LAUNCH_CHECK();
  return FGS_OK;
}

cudaError_t allow_dyn_smem(const void* kernel, int bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> done;  // (kernel, device) -> bytes allowed
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  int& have = done[{kernel, dev}];
  if (have >= bytes) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) have = bytes;
  return e;
}

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
struct TimerSlot {
  std::mutex mu;
  bool enabled = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pairs;  // recorded since the last read
  int kernels = 0;                                         // launches inside those pairs
  cudaEvent_t open = nullptr;
};
TimerSlot g_timers[FGS_K_COUNT];

}  // namespace

void timer_begin(int id, cudaStream_t s) {
  if (id < 0 || id >= FGS_K_COUNT) return;
  TimerSlot& t = g_timers[id];
  if (!t.enabled) return;
  // no event pairs inside a CUDA graph capture: the launch is not executed now
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
  std::lock_guard<std::mutex> lk(t.mu);
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  cudaEventRecord(e, s);
  t.open = e;
}

void timer_end(int id, cudaStream_t s, int kernels) {
  if (id < 0 || id >= FGS_K_COUNT) return;
  TimerSlot& t = g_timers[id];
  if (!t.enabled) return;
  std::lock_guard<std::mutex> lk(t.mu);
  if (!t.open) return;
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  cudaEventRecord(e, s);
  t.pairs.emplace_back(t.open, e);
  t.kernels += kernels;
  t.open = nullptr;
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
  adam_step(param, m1, m2, p, grad[p], lr, b1, b2, eps);
}
// FP32 issue ceiling for the compositing kernels' roofline: every thread runs
// 8 independent FMA chains, so the FMA pipe, not latency, limits the rate.
constexpr int kPeakChains = 8;
constexpr int kPeakIters = 2048;
__device__ float g_peak_sink;

}  // namespace

// Every translation unit's error word, gathered (and optionally cleared) by
// one tiny kernel so that reading them costs one synchronisation.
constexpr int kErrorUnits = 5;
struct ErrorWords {
  int* w[kErrorUnits];
};
__device__ int g_error_gather;
__global__ void k_gather_errors(ErrorWords e, bool clear, int* out) {
  if (threadIdx.x != 0) return;
  int v = 0;
  for (int j = 0; j < kErrorUnits; ++j) {
    v |= clear ? atomicExch(e.w[j], 0) : atomicOr(e.w[j], 0);
  }
  *out = v;
}

namespace {
__global__ void __launch_bounds__(256) k_ffma_peak(float a, float b) {
  float x[kPeakChains];
#pragma unroll
  for (int j = 0; j < kPeakChains; ++j) x[j] = a + (float)(threadIdx.x + j);
#pragma unroll 4
  for (int i = 0; i < kPeakIters; ++i)
#pragma unroll
    for (int j = 0; j < kPeakChains; ++j) x[j] = fmaf(x[j], b, a);
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < kPeakChains; ++j) s += x[j];
  if (s == 12345.678f) g_peak_sink = s;  // never true; keeps the chains live
}

// The same chains on packed pairs: one fma.rn.f32x2 per step (4 FLOP).
__global__ void __launch_bounds__(256) k_ffma2_peak(float a, float b) {
  f2x x[kPeakChains];
#pragma unroll
  for (int j = 0; j < kPeakChains; ++j) x[j] = f2_pack(a + (float)(threadIdx.x + j), a - (float)j);
  const f2x a2 = f2_pack(a, a), b2 = f2_pack(b, b);
#pragma unroll 4
  for (int i = 0; i < kPeakIters; ++i)
#pragma unroll
    for (int j = 0; j < kPeakChains; ++j) x[j] = f2_fma(x[j], b2, a2);
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < kPeakChains; ++j) {
    float lo, hi;
    f2_unpack(x[j], lo, hi);
    s += lo + hi;
  }
  if (s == 12345.678f) g_peak_sink = s;
}

// MUFU ex2 issue ceiling (the alpha of every pixel-Gaussian evaluation is one
// ex2.approx): 8 independent chains x = ex2(x) * -0.5 per thread, values
// bounded in (-0.5, 0]; the multiply runs on the FMA pipe, beside the MUFU.
__global__ void __launch_bounds__(256) k_ex2_peak(float a) {
  float x[kPeakChains];
#pragma unroll
  for (int j = 0; j < kPeakChains; ++j) x[j] = -a * (float)(1 + ((threadIdx.x + j) & 7));
#pragma unroll 4
  for (int i = 0; i < kPeakIters; ++i)
#pragma unroll
    for (int j = 0; j < kPeakChains; ++j) x[j] = ex2_approx(x[j]) * -0.5f;
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < kPeakChains; ++j) s += x[j];
  if (s == 12345.678f) g_peak_sink = s;
}

template <typename Launch>
cudaError_t best_ms(Launch launch, cudaStream_t s, float* out) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t err = cudaEventCreate(&e0);
  if (err == cudaSuccess) err = cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; err == cudaSuccess && rep < 4; ++rep) {  // first launch warms up
    cudaEventRecord(e0, s);
    launch();
    cudaEventRecord(e1, s);
    err = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0) best = ms < best ? ms : best;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  *out = best;
  return err == cudaSuccess ? cudaGetLastError() : err;
}

}  // namespace

}  // namespace fgs

extern "C" fgs_status fgs_peak_ex2(double* gops, void* stream) {
  if (!gops) return FGS_ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int blocks = fgs::num_sms() * 8;
  float best = 0.f;
  FGS_TRY(fgs::best_ms([&] { fgs::k_ex2_peak<<<blocks, 256, 0, s>>>(0.25f); }, s, &best));
  const double ops = (double)blocks * 256.0 * fgs::kPeakIters * fgs::kPeakChains;
  *gops = ops / (best * 1e-3) / 1e9;
  return FGS_OK;
}

extern "C" fgs_status fgs_peak_fp32(double* tflops, void* stream) {
  if (!tflops) return FGS_ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int blocks = fgs::num_sms() * 8;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  FGS_TRY(cudaEventCreate(&e0));
  FGS_TRY(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {  // first launch warms up
    cudaEventRecord(e0, s);
    fgs::k_ffma_peak<<<blocks, 256, 0, s>>>(0.5f, 0.999f);
    cudaEventRecord(e1, s);
    FGS_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0) best = ms < best ? ms : best;
  }
  FGS_LAUNCH_CHECK();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double flops = 2.0 * blocks * 256.0 * fgs::kPeakIters * fgs::kPeakChains;
  *tflops = flops / (best * 1e-3) / 1e12;
  return FGS_OK;
}

extern "C" fgs_status fgs_peak_fp32x2(double* tflops, void* stream) {
  if (!tflops) return FGS_ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int blocks = fgs::num_sms() * 8;
  float best = 0.f;
  FGS_TRY(fgs::best_ms([&] { fgs::k_ffma2_peak<<<blocks, 256, 0, s>>>(0.5f, 0.999f); }, s, &best));
  const double flops = 4.0 * blocks * 256.0 * fgs::kPeakIters * fgs::kPeakChains;
  *tflops = flops / (best * 1e-3) / 1e12;
  return FGS_OK;
}

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
  int dev = 0;
  FGS_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return FGS_ERR_UNSUPPORTED;
  static std::mutex mu;
  static fgs::ErrorWords cache[64];
  static bool have[64] = {false};
  fgs::ErrorWords w;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!have[dev]) {
      cache[dev] = fgs::ErrorWords{{fgs::error_word_preprocess(), fgs::error_word_sort(), fgs::error_word_render(),
                                    fgs::error_word_backward(), fgs::error_word_aux()}};
      for (int* p : cache[dev].w)
        if (!p) return FGS_ERR_CUDA;
      have[dev] = true;
    }
    w = cache[dev];
  }
  int* out = nullptr;
  FGS_TRY(cudaGetSymbolAddress(reinterpret_cast<void**>(&out), fgs::g_error_gather));
  fgs::k_gather_errors<<<1, 32, 0, s>>>(w, clear != 0, out);
  FGS_LAUNCH_CHECK();
  FGS_TRY(cudaMemcpyAsync(flags, out, sizeof(int), cudaMemcpyDeviceToHost, s));
  FGS_TRY(cudaStreamSynchronize(s));
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

namespace fgs {
namespace {
// Two device words into mapped host memory, stored by the GPU itself.
__global__ void k_store_counts(const int32_t* a, const int32_t* b, int32_t* out) {
  out[0] = a ? *a : 0;
  out[1] = b ? *b : 0;
}
}  // namespace
}  // namespace fgs

extern "C" fgs_status fgs_read_counts(const int32_t* curr_offset, const int32_t* counters, int32_t* host_out,
                                      void* stream) {
  if (!host_out || (!curr_offset && !counters)) return FGS_ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  void* dptr = nullptr;
  if (cudaHostGetDevicePointer(&dptr, host_out, 0) == cudaSuccess && dptr) {
    fgs::KernelTimer kt__(FGS_K_READ_COUNTS, s);
    fgs::k_store_counts<<<1, 1, 0, s>>>(curr_offset, counters, static_cast<int32_t*>(dptr));
    kt__.stop();
    FGS_LAUNCH_CHECK();
    return FGS_OK;
  }
  (void)cudaGetLastError();  // not mapped host memory: copy instead
  if (curr_offset) FGS_TRY(cudaMemcpyAsync(host_out, curr_offset, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  if (counters) FGS_TRY(cudaMemcpyAsync(host_out + 1, counters, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  return FGS_OK;
}

extern "C" fgs_status fgs_kernel_timer(int kernel_id, int enable) {
  if (kernel_id < 0 || kernel_id >= FGS_K_COUNT) return FGS_ERR_BAD_ARG;
  fgs::g_timers[kernel_id].enabled = enable != 0;
  return FGS_OK;
}

extern "C" fgs_status fgs_kernel_timer_read(int kernel_id, double* total_ms, int* launches) {
  if (kernel_id < 0 || kernel_id >= FGS_K_COUNT || !total_ms || !launches) return FGS_ERR_BAD_ARG;
  auto& t = fgs::g_timers[kernel_id];
  std::lock_guard<std::mutex> lk(t.mu);
  double sum = 0.0;
  for (auto& pr : t.pairs) {
    float ms = 0.f;
    if (cudaEventSynchronize(pr.second) != cudaSuccess) return FGS_ERR_CUDA;
    if (cudaEventElapsedTime(&ms, pr.first, pr.second) != cudaSuccess) return FGS_ERR_CUDA;
    sum += ms;
    cudaEventDestroy(pr.first);
    cudaEventDestroy(pr.second);
  }
  *total_ms = sum;
  *launches = t.kernels;
  t.kernels = 0;
  t.pairs.clear();
  return FGS_OK;
}
