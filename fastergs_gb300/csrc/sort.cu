// Stable LSD radix sort of (u64 key, u32 value) pairs, sm_103a.
//
// Replaces the cub::DeviceRadixSort::SortPairs call of FB
// (csrc/cuda_rasterizer/sort.cu:28-44) with a single-pass-per-digit
// ("onesweep") sort written for this GPU:
//   * one upfront kernel builds the 8-bit digit histograms of every pass in a
//     single read of the keys and turns them into global digit bases;
//   * each pass is one kernel: a CTA of 512 threads (8 keys each, few enough
//     registers for 2 CTAs = 32 warps per SM) ranks a 4096-key tile in shared
//     memory (ballot digit masks + per-warp digit counters, so ranks are
//     stable), publishes its per-digit counts, sorts the tile locally, obtains
//     the exclusive prefix of all earlier tiles by a decoupled look-back, and
//     scatters so that global writes form contiguous runs per digit;
//   * only the key bits that can differ are sorted: 31 depth bits (a depth is
//     a positive float, so bit 31 of a key is zero) plus ceil(log2(tiles))
//     tile bits.  The first pass packs each key to (tile << 31) | depth bits
//     and the last one unpacks it, so 17 tile bits (the 16 views of a batched
//     frame) still fit six 8-bit passes; 4-6 passes for 1..131072 tiles.  A
//     key with bit 31 set is not a (tile, depth) key: the histogram raises the
//     capacity bit of the error word for it.
// Every look-back wait is bounded (kSpinLimit polls); on expiry the kernel
// records kErrTimeout in the error word and continues, so it never hangs.
#include <algorithm>
#include <mutex>

#include <cuda.h>

#include "internal.cuh"


namespace fgs {
namespace {

constexpr int kSortThreads = 512;
constexpr int kSortWarps = kSortThreads / kWarp;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;   // 4096 keys
constexpr int kRadix = 256;
constexpr int kMaxPasses = 8;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagInc = 2u << 30;
constexpr uint32_t kValueMask = (1u << 30) - 1;
// Predecessor words read per look-back round.  The nearest few predecessors
// usually hold an inclusive prefix already, so a narrow window wins: per C2
// pass (3.1M keys) 38.5 us at 32 words, 36.3 at 16, 35.4 at 8 and 4, 35.9 at
// 2; a 47M-key batched sort 2.47 / 2.32 / 2.24 / 2.22 / 2.28 ms.
constexpr int kLookWindow = 4;
constexpr int kSortDynSmem = (int)((sizeof(unsigned long long) + sizeof(uint32_t)) * kSortTile);

struct SortLayout {
  size_t hist = 0, counters = 0, lookback = 0, alt_keys = 0, alt_vals = 0, total = 0;
  int64_t tiles = 0;
};

constexpr size_t up256(size_t v) { return (v + 255) & ~(size_t)255; }

constexpr SortLayout layout_for(int64_t n) {
  constexpr auto up = up256;
  SortLayout L;
  L.tiles = (n + kSortTile - 1) / kSortTile;
  size_t off = 0;
  L.hist = off;      off = up(off + sizeof(uint32_t) * kMaxPasses * kRadix);
  L.counters = off;  off = up(off + sizeof(uint32_t) * (kMaxPasses + 1));  // tile counters, histogram done count
  L.lookback = off;  off = up(off + sizeof(uint32_t) * kMaxPasses * (size_t)L.tiles * kRadix);
  L.alt_keys = off;  off = up(off + sizeof(uint64_t) * (size_t)n);
  L.alt_vals = off;  off = up(off + sizeof(uint32_t) * (size_t)n);
  L.total = off;
  return L;
}

// (tile << 32) | depth bits  <->  (tile << 31) | depth bits.
__device__ __forceinline__ unsigned long long pack_key(unsigned long long k) {
  return ((k >> 32) << 31) | (k & 0x7fffffffull);
}
__device__ __forceinline__ unsigned long long unpack_key(unsigned long long c) {
  return ((c >> 31) << 32) | (c & 0x7fffffffull);
}

// All pass histograms in one read of the keys; the last block to finish turns
// them into exclusive digit offsets (the global base of every digit of every
// pass), so the pass kernels read their bases instead of scanning.
// Lanes of the warp whose 8-bit digit equals this lane's: one ballot per
// digit bit (ALU votes; a warp match instruction on this GPU queues on the
// same pipe as shared and global memory accesses and throttled the passes).
__device__ __forceinline__ uint32_t digit_peers(uint32_t d) {
  uint32_t m = 0xffffffffu;
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    const bool bit = (d >> b) & 1u;
    const uint32_t bal = __ballot_sync(0xffffffffu, bit);
    m &= bit ? bal : ~bal;
  }
  return m;
}

// Pair count: the host bound, or min(bound, *n_dev) when the count lives on
// the device (batched / graph-captured frames).
__device__ __forceinline__ long long pair_count(long long n_cap, const int* n_dev) {
  return n_dev ? min(n_cap, (long long)(unsigned int)*n_dev) : n_cap;
}

__global__ void __launch_bounds__(kSortThreads) k_histogram(const unsigned long long* keys, long long n_cap,
                                                            const int* n_dev, int passes, uint32_t* hist,
                                                            uint32_t* done) {
  pdl_wait();  // the preceding kernel of the stream is done
  pdl_trigger();
  __shared__ uint32_t s_h4[4][kMaxPasses][kRadix];
  __shared__ bool s_last;
  const long long n = pair_count(n_cap, n_dev);
  for (int j = threadIdx.x; j < 4 * kMaxPasses * kRadix; j += kSortThreads) (&s_h4[0][0][0])[j] = 0;
  // four copies of the counters (warp % 4), summed at the end: fewer warps
  // contend for one shared-memory word (C2 histogram 20.2 -> 19.4 us, a 47M-key
  // batched one 0.129 -> 0.119 ms)
  uint32_t (*s_h)[kRadix] = s_h4[(threadIdx.x >> 5) & 3];
  __syncthreads();
  // 8 keys per thread and step, loaded before they are counted (memory-level
  // parallelism with few blocks: every block adds passes x 256 global counts).
  constexpr int kHistItems = 8;
  const long long stride = (long long)gridDim.x * kSortThreads * kHistItems;
  for (long long k0 = blockIdx.x * (long long)kSortThreads * kHistItems + threadIdx.x; k0 < n; k0 += stride) {
    unsigned long long key[kHistItems];
#pragma unroll
    for (int r = 0; r < kHistItems; ++r) {
      const long long k = k0 + (long long)r * kSortThreads;
      key[r] = k < n ? __ldg(keys + k) : 0ull;
    }
#pragma unroll
    for (int r = 0; r < kHistItems; ++r) {
      if (k0 + (long long)r * kSortThreads >= n) break;
      if (key[r] & 0x80000000ull) raise_error(kErrCapacity);
      const unsigned long long c = pack_key(key[r]);
      for (int p = 0; p < passes; ++p) atomicAdd(&s_h[p][(c >> (8 * p)) & 0xff], 1u);
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < passes * kRadix; j += kSortThreads) {
    const uint32_t v = (&s_h4[0][0][0])[j] + (&s_h4[1][0][0])[j] + (&s_h4[2][0][0])[j] + (&s_h4[3][0][0])[j];
    if (v) atomicAdd(&hist[j], v);
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // One warp per pass: exclusive scan of its 256 counts, 8 per lane.
  const int lane = threadIdx.x & 31, p = threadIdx.x >> 5;
  if (p < passes) {
    uint32_t c[8], sum = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      c[j] = ld_volatile_u32(hist + p * kRadix + lane * 8 + j);
      sum += c[j];
    }
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    uint32_t run = incl - sum;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      hist[p * kRadix + lane * 8 + j] = run;
      run += c[j];
    }
  }
}

// One digit pass.  Per tile of kSortTile keys:
//   1. rank every key within its warp's digit counters (warp match: stable);
//   2. per digit: counts of the warps, tile count published for look-back;
//   3. tile-local digit offsets (block scan) and a local sort of the tile into
//      shared memory;
//   4. per digit: decoupled look-back over a window of kLookWindow
//      predecessors per round, with no key registers live;
//   5. global scatter from shared memory, contiguous per digit run.
__global__ void __launch_bounds__(kSortThreads, 2) k_onesweep(
    const unsigned long long* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
    unsigned long long* __restrict__ keys_out, uint32_t* __restrict__ vals_out, long long n_cap, const int* n_dev,
    int shift, bool first, bool last, const uint32_t* __restrict__ digit_base, uint32_t* lookback,
    uint32_t* tile_counter) {
  pdl_wait();  // the preceding kernel of the stream is done
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char s_dyn[];  // kSortDynSmem bytes
  unsigned long long* s_keys = reinterpret_cast<unsigned long long*>(s_dyn);
  uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_dyn + sizeof(unsigned long long) * kSortTile);
  __shared__ uint32_t s_whist[kSortWarps][kRadix];
  __shared__ uint32_t s_dst[kRadix];
  __shared__ uint32_t s_toff[kRadix];
  __shared__ uint32_t s_tmp[kSortWarps];
  __shared__ uint32_t s_tile;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_tile = atomicAdd(tile_counter, 1u);
  for (int j = tid; j < kSortWarps * kRadix; j += kSortThreads) (&s_whist[0][0])[j] = 0;
  __syncthreads();
  const uint32_t tile = s_tile;
  const long long tile_base = (long long)tile * kSortTile;
  const long long n = pair_count(n_cap, n_dev);
  if (tile_base >= n) return;  // grid sized for the capacity; this tile is empty
  const int valid = (int)min((long long)kSortTile, n - tile_base);

  // Load: warp w owns keys [tile_base + w*32*items, ...), 32 consecutive per
  // step, so (warp, step, lane) is the input order and the ranks are stable.
  unsigned long long k[kSortItems];
  uint32_t v[kSortItems];
  uint32_t rank[kSortItems];
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const long long idx = tile_base + warp * (kWarp * kSortItems) + r * kWarp + lane;
    if (idx < n) {
      k[r] = first ? pack_key(keys_in[idx]) : keys_in[idx];
      v[r] = vals_in[idx];
    } else {
      k[r] = ~0ull;  // digit 255, ranked after every real key of the tile
      v[r] = 0;
    }
  }
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const uint32_t d = (uint32_t)(k[r] >> shift) & 0xff;
    const uint32_t peers = digit_peers(d);
    const uint32_t before = s_whist[warp][d];
    __syncwarp();
    if ((peers & lanemask_lt()) == 0) s_whist[warp][d] = before + __popc(peers);
    __syncwarp();
    rank[r] = before + __popc(peers & lanemask_lt());
  }
  __syncthreads();

  // Per digit (threads 0..255, warps 0..7): warp offsets, tile count, publish.
  const uint32_t d = (uint32_t)tid;
  uint32_t cnt = 0, incl = 0;
  uint32_t* lb = lookback + (size_t)tile * kRadix;
  if (tid < kRadix) {
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
      const uint32_t x = s_whist[w][d];
      s_whist[w][d] = cnt;
      cnt += x;
    }
    // padding keys (last tile only) all sit in digit 255
    const uint32_t real = (d == 255) ? cnt - (uint32_t)(kSortTile - valid) : cnt;
    st_volatile_u32(lb + d, (tile == 0 ? kFlagInc : kFlagAgg) | real);
    incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    if (lane == 31) s_tmp[warp] = incl;
  }
  __syncthreads();
  uint32_t toff = 0;
  if (tid < kRadix) {
    for (int w = 0; w < warp; ++w) toff += s_tmp[w];
    toff += incl - cnt;
    s_toff[d] = toff;
  }
  __syncthreads();

  // Local sort of the tile into shared memory.
#pragma unroll
  for (int r = 0; r < kSortItems; ++r) {
    const uint32_t dd = (uint32_t)(k[r] >> shift) & 0xff;
    const uint32_t slot = s_toff[dd] + s_whist[warp][dd] + rank[r];
    s_keys[slot] = k[r];
    s_vals[slot] = v[r];
  }

  if (tid < kRadix) {
    uint32_t excl = 0;
    if (tile != 0) {
      // Windowed look-back: the words of the kLookWindow nearest unvisited
      // predecessors are loaded together (independent loads, one latency),
      // then summed newest first until an inclusive prefix; a word that is
      // not published yet is re-polled (bounded) before the walk goes on.
      long long pred = (long long)tile - 1;
      int polls = 0;
      bool done = false;
      while (!done) {
        uint32_t w[kLookWindow];
#pragma unroll
        for (int j = 0; j < kLookWindow; ++j)
          w[j] = pred - j >= 0 ? ld_volatile_u32(lookback + (size_t)(pred - j) * kRadix + d) : kFlagInc;
        int used = 0;
#pragma unroll
        for (int j = 0; j < kLookWindow; ++j) {
          if (done || used != j) continue;
          const uint32_t flag = w[j] & ~kValueMask;
          if (flag == 0) continue;  // not yet published: stop consuming here
          excl += w[j] & kValueMask;
          used = j + 1;
          if (flag == kFlagInc) done = true;
        }
        pred -= used;
        if (!done && used == 0) {  // the nearest unvisited predecessor has not published
          if (++polls > kSpinLimit) {
            raise_error(kErrTimeout);
            break;
          }
          __nanosleep(64);
        }
      }
      const uint32_t real = (d == 255) ? cnt - (uint32_t)(kSortTile - valid) : cnt;
      st_volatile_u32(lb + d, kFlagInc | (excl + real));
    }
    s_dst[d] = digit_base[d] + excl - toff;  // global position of shared slot i = s_dst[digit] + i
  }
  __syncthreads();

  for (int j = tid; j < valid; j += kSortThreads) {
    const unsigned long long kk = s_keys[j];
    const uint32_t pos = s_dst[(uint32_t)(kk >> shift) & 0xff] + (uint32_t)j;
    if ((long long)pos < n) {
      keys_out[pos] = last ? unpack_key(kk) : kk;
      vals_out[pos] = s_vals[j];
    } else {
      raise_error(kErrTimeout);  // only reachable after an expired look-back
    }
  }
  __syncthreads();
}

}  // namespace
}  // namespace fgs

FGS_DEFINE_ERROR_ACCESSOR(sort)

extern "C" size_t fgs_sort_temp_bytes(int64_t num_rendered) { return fgs::sort_temp_bytes(num_rendered); }

namespace fgs {
fgs_status run_sort(int64_t n_cap, const int32_t* n_dev, uint32_t tiles, void* temp, size_t temp_bytes,
                    const uint64_t* keys_in, const uint32_t* values_in, uint64_t* keys_out, uint32_t* values_out,
                    cudaStream_t s) {
  if (n_cap == 0) return FGS_OK;
  if (n_cap >= (int64_t)kValueMask) return FGS_ERR_CAPACITY;
  if (!temp || !keys_in || !values_in || !keys_out || !values_out) return FGS_ERR_BAD_ARG;
  if (((uintptr_t)temp & 255) || ((uintptr_t)keys_in & 7) || ((uintptr_t)keys_out & 7)) return FGS_ERR_BAD_ARG;
  const SortLayout L = layout_for(n_cap);
  if (temp_bytes < L.total) return FGS_ERR_CAPACITY;
  const int bits = 31 + tile_bits(tiles);
  const int passes = (bits + 7) / 8;
  char* base = static_cast<char*>(temp);
  uint32_t* hist = reinterpret_cast<uint32_t*>(base + L.hist);
  uint32_t* counters = reinterpret_cast<uint32_t*>(base + L.counters);
  uint32_t* lookback = reinterpret_cast<uint32_t*>(base + L.lookback);
  auto* alt_k = reinterpret_cast<unsigned long long*>(base + L.alt_keys);
  auto* alt_v = reinterpret_cast<uint32_t*>(base + L.alt_vals);
  // hist, counters and the look-back words of every pass start at zero.
  {
    const fgs_status z = zero_async(base, L.alt_keys, s);
    if (z != FGS_OK) return z;
  }
  // histogram blocks: up to 3 per SM (a 47M-key batched histogram 0.119 ms
  // at 2 per SM, 0.115 at 3)
  const int hist_blocks = (int)std::max<int64_t>(
      1, std::min<int64_t>((n_cap + kSortThreads * 8 - 1) / (kSortThreads * 8), (int64_t)num_sms() * 3));
  {
    KernelTimer kt__(FGS_K_SORT_HIST, s);
    (void)launch_pdl(k_histogram, dim3(hist_blocks), dim3(kSortThreads), 0, s,
                     reinterpret_cast<const unsigned long long*>(keys_in), n_cap, n_dev, passes, hist,
                     counters + kMaxPasses);
    kt__.stop();
  }
  FGS_LAUNCH_CHECK();
  FGS_TRY(allow_dyn_smem(reinterpret_cast<const void*>(&k_onesweep), kSortDynSmem));
  const unsigned long long* src_k = reinterpret_cast<const unsigned long long*>(keys_in);
  const uint32_t* src_v = values_in;
  for (int p = 0; p < passes; ++p) {
    // Ping-pong so that the last pass lands in the output buffers.
    const bool to_out = ((passes - 1 - p) % 2) == 0;
    unsigned long long* dk = to_out ? reinterpret_cast<unsigned long long*>(keys_out) : alt_k;
    uint32_t* dv = to_out ? values_out : alt_v;
    {
      KernelTimer kt__(FGS_K_SORT_PASS, s);
      (void)launch_pdl(k_onesweep, dim3((unsigned)L.tiles), dim3(kSortThreads), kSortDynSmem, s, src_k, src_v, dk,
                       dv, n_cap, n_dev, 8 * p, p == 0, p == passes - 1, hist + p * kRadix,
                       lookback + (size_t)p * L.tiles * kRadix, counters + p);
      kt__.stop();
    }
    FGS_LAUNCH_CHECK();
    src_k = dk;
    src_v = dv;
  }
  return FGS_OK;
}

size_t sort_temp_bytes(int64_t n) { return layout_for(n < 1 ? 1 : n).total; }
}  // namespace fgs

extern "C" fgs_status fgs_sort(int64_t num_rendered, int width, int height, int block_x, int block_y, void* temp,
                               size_t temp_bytes, const uint64_t* keys_in, const uint32_t* values_in,
                               uint64_t* keys_out, uint32_t* values_out, void* stream) {
  using namespace fgs;
  if (num_rendered < 0 || width <= 0 || height <= 0 || block_x <= 0 || block_y <= 0) return FGS_ERR_BAD_ARG;
  const uint32_t tiles = (uint32_t)(((width + block_x - 1) / block_x) * ((height + block_y - 1) / block_y));
  return run_sort(num_rendered, nullptr, tiles, temp, temp_bytes, keys_in, values_in, keys_out, values_out,
                  (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// Sort without caller-provided scratch (fgs_sort_noalloc).
//
// Some callers cannot allocate device memory at the point where they sort:
// code running inside a memory pool or arena they do not own, plugins whose
// host forbids allocation after start-up, and real-time loops that must not
// stall on cudaMalloc.  For them the scratch of fgs_sort lives in this
// file-scope array, sized for FGS_SORT_NOALLOC_MAX_PAIRS pairs.  Every GPU
// that loads the library holds it (about 14 MiB) until the process exits.
namespace fgs {
namespace {
constexpr int64_t kNoAllocMaxPairs = FGS_SORT_NOALLOC_MAX_PAIRS;
constexpr size_t kNoAllocBytes = layout_for(kNoAllocMaxPairs).total;
static __device__ __align__(256) unsigned char g_sort_scratch[kNoAllocBytes];

// Device address of g_sort_scratch, looked up once per device and CUDA
// context (the host-side name of a __device__ array is not a device address).
// The cache is keyed on the context's process-unique id: after
// cudaDeviceReset, or under another context on the same device, the array
// lives at a new address and is looked up again.  The two driver calls are
// reached through the runtime's entry-point query, so the library does not
// link libcuda.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Id of the calling thread's current context, or 0 when there is none or the
// driver does not provide the query (the caller then looks the address up).
unsigned long long current_context_id() {
  static const CtxGetCurrentFn get_current = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 4000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      fn = nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(fn);
  }();
  static const CtxGetIdFn get_id = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      fn = nullptr;
    return reinterpret_cast<CtxGetIdFn>(fn);
  }();
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

struct ScratchAddress {
  unsigned long long context_id = 0;
  void* ptr = nullptr;
};
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
ScratchAddress g_scratch_addr[kMaxDevices];
}  // namespace
}  // namespace fgs

extern "C" fgs_status fgs_sort_noalloc(int64_t num_rendered, int width, int height, int block_x, int block_y,
                                       const uint64_t* keys_in, const uint32_t* values_in, uint64_t* keys_out,
                                       uint32_t* values_out, void* stream) {
  using namespace fgs;
  if (num_rendered < 0) return FGS_ERR_BAD_ARG;
  if (num_rendered > kNoAllocMaxPairs) return FGS_ERR_CAPACITY;
  int dev = 0;
  FGS_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return FGS_ERR_UNSUPPORTED;
  void* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    ScratchAddress& a = g_scratch_addr[dev];
    const unsigned long long ctx = current_context_id();
    if (!a.ptr || ctx == 0 || ctx != a.context_id) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
      if (e != cudaSuccess || !p) return FGS_ERR_CUDA;
      a.ptr = p;
      a.context_id = current_context_id();  // the lookup makes the runtime's context current
    }
    scratch = a.ptr;
  }
  // fgs_sort zeroes the histogram and look-back words it needs on every call.
  return fgs_sort(num_rendered, width, height, block_x, block_y, scratch, kNoAllocBytes, keys_in, values_in,
                  keys_out, values_out, stream);
}
