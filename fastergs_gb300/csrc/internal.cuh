// Internal launch interfaces shared by the plain and the batched entry
// points (not part of the C ABI).
#pragma once
#include "fgs_common.cuh"

namespace fgs {

struct PreArgs {
  Views views;
  int P, D, M;
  const float* means;
  const float* colors;
  const float* dc;
  const float* shs;
  const float* opac;
  const float* scales;
  const float* rots;
  const uint8_t* culling;
  float* splat;          // records, (V * P) x 32 floats, record index = view * P + Gaussian
  unsigned long long* keys;
  uint32_t* vals;        // record index of each pair
  long long cap;
  uint32_t* tasks;
  long long task_cap;    // in tasks (2 words each)
  unsigned int* curr;
  int* counters;
  int* radii;            // V * P
  int large_tiles;       // footprints of >= large_tiles tiles are split into sub-tasks of that many tiles
                         // (a multiple of 32; FB: 128)
  int packet;            // small footprints: consecutive candidate tiles each lane tests per step (1, 2, 4, 8)
};

// Preprocess + large-Gaussian emission for every view (grid.y = view).
fgs_status run_preprocess(PreArgs& a, cudaStream_t s);

// Stable radix sort of n pairs on 31 depth + ceil(log2 tiles) tile bits.  n = n_cap,
// or min(n_cap, *n_dev) when n_dev is given (grids are sized for n_cap).
fgs_status run_sort(int64_t n_cap, const int32_t* n_dev, uint32_t tiles, void* temp, size_t temp_bytes,
                    const uint64_t* keys_in, const uint32_t* values_in, uint64_t* keys_out, uint32_t* values_out,
                    cudaStream_t s);
size_t sort_temp_bytes(int64_t n);

bool tile_shape_ok(int bx, int by);

struct PbwdArgs {
  Views views;
  int P, D, M;
  const float* means;
  const int* radii;     // V * P
  const float* dc;
  const float* shs;
  const float* splat;   // V * P records
  const float* scales;
  const float* rots;
  const float* grad;    // V * P gradient records
  float* dmean2D;       // V * P (optional)
  float* dconic;        // V * P (optional)
  float* dopac;         // summed over views from here on
  float* dcolor;
  float* dmean3D;
  float* dcov3D;
  float* ddc;
  float* dsh;
  float* dscale;
  float* drot;
  float* accum;         // densification statistics, accumulated per view
  float* accum_abs;
  float* max_radii;
  float* denom;
  int sh_staged = 0;    // set by run_preprocess_bwd: SH rows and dL/dsh rows in shared memory
  // Fused sparse Adam (adam_on): the gradient outputs above are unused; the
  // activation backward and the Adam step update the raw parameters instead.
  int adam_on = 0;
  const float* opac = nullptr;  // activated opacities (P), for the sigmoid backward
  fgs_adam_fused adam{};
};

// Host check of a fused Adam description (moments for every stepped group,
// step sizes, known activations, 16-byte rotation rows, f_rest only with SH).
bool adam_args_ok(const fgs_adam_fused* ad, const float* shs, const float* opacities);

fgs_status run_preprocess_bwd(PbwdArgs& a, cudaStream_t s);
// cudaMemsetAsync(ptr, 0, bytes) as a kernel launched with programmatic
// dependent launch, so the chain of the path's kernels is not broken; a
// second range (ptr2, bytes2) is zeroed by the same launch.
fgs_status zero_async(void* ptr, size_t bytes, cudaStream_t s, void* ptr2 = nullptr, size_t bytes2 = 0);

// Tile ranges of the sorted keys; (zero_also, zero_bytes) is zeroed by the
// same launch that clears the ranges.
fgs_status run_tile_ranges(int64_t n_cap, const int32_t* n_dev, uint32_t tiles, const uint64_t* keys_sorted,
                           uint32_t* ranges, cudaStream_t s, void* zero_also = nullptr, size_t zero_bytes = 0);

}  // namespace fgs
