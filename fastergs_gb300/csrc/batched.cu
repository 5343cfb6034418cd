// Batched multi-camera rasterization: many views of uneven resolution per
// launch, no host round trip, so a whole fwd+bwd step can be captured in a
// CUDA graph.
//
// Every stage runs once for all views: preprocess (grid.y = view), one radix
// sort over a global tile index space (view k owns tiles [tile_off_k, ...)),
// one tile-range pass, one bucket setup, one persistent composite launch over
// the buckets of all views, one merge over all tiles, one persistent backward
// launch, and one per-Gaussian backward that sums the views.  Capacities
// (pairs, buckets) are fixed when the workspace is planned; overflow is
// latched on the device and reported by fgs_batch_status, never written past.
#include <algorithm>
#include <vector>

#include "internal.cuh"
#include "render_common.cuh"

namespace fgs {
namespace {

// Largest pair capacity: the sort's look-back words carry 30-bit counts.
constexpr int64_t kMaxBatchPairs = ((int64_t)1 << 30) - 2;

struct BatchLayout {
  size_t counters, curr, records, keys_u, vals_u, keys_s, vals_s, tasks, sort_tmp, ranges, image, sample, grad,
      last_contrib, ts_final, total;
  size_t sort_bytes, image_bytes, sample_bytes;
  int64_t pairs, buckets, records_n, pixels;
  uint32_t tiles;
};

BatchLayout plan(int P, int V, const int* W, const int* H, int bx, int by, int64_t pairs, int bucket_size,
                 bool recompute) {
  BatchLayout L;
  L.pairs = pairs;
  L.tiles = 0;
  L.pixels = 0;
  for (int v = 0; v < V; ++v) {
    L.tiles += (uint32_t)(((W[v] + bx - 1) / bx) * ((H[v] + by - 1) / by));
    L.pixels += (int64_t)W[v] * H[v];
  }
  const int64_t sub = sub_bucket_size(bucket_size);  // sample state is per sub-bucket
  L.buckets = (pairs + sub - 1) / sub + std::min<int64_t>((int64_t)L.tiles, pairs);
  if (L.buckets < 1) L.buckets = 1;
  L.records_n = (int64_t)V * P;
  L.sort_bytes = sort_temp_bytes(pairs);
  L.image_bytes = carve_image(nullptr, (size_t)L.pixels, L.tiles).bytes;
  L.sample_bytes = carve_sample(nullptr, L.buckets, recompute ? (int64_t)L.tiles : L.buckets).bytes;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off = align_up(off + bytes, 256);
    return at;
  };
  L.counters = take(sizeof(int32_t) * FGS_COUNTER_WORDS);
  L.curr = take(sizeof(int32_t) * 4);
  L.records = take(sizeof(float) * 32 * (size_t)L.records_n);
  L.keys_u = take(sizeof(uint64_t) * (size_t)pairs);
  L.vals_u = take(sizeof(uint32_t) * (size_t)pairs);
  L.keys_s = take(sizeof(uint64_t) * (size_t)pairs);
  L.vals_s = take(sizeof(uint32_t) * (size_t)pairs);
  L.tasks = take(sizeof(uint32_t) * (size_t)pairs);
  L.sort_tmp = take(L.sort_bytes);
  L.ranges = take(sizeof(uint32_t) * 2 * (size_t)L.tiles);
  L.image = take(L.image_bytes);
  L.sample = take(L.sample_bytes);
  L.grad = take(sizeof(float) * FGS_GRAD_STRIDE * (size_t)L.records_n);
  L.last_contrib = take(sizeof(int32_t) * (size_t)L.pixels);
  L.ts_final = take(sizeof(float) * (size_t)L.pixels);
  L.total = off;
  return L;
}

bool config_ok(const fgs_tune_config* c) {
  return c && c->bucket_size >= 1 && c->bucket_size <= kMaxBucket && tile_shape_ok(c->block_x, c->block_y) &&
         (c->packet == 1 || c->packet == 2 || c->packet == 4 || c->packet == 8) &&
         (c->recompute == 0 || c->recompute == 1) && c->chain >= 0 && c->chain <= kRounds;
}

bool cameras_ok(int V, const fgs_camera* cams) {
  if (V < 1 || V > kMaxViews || !cams) return false;
  for (int v = 0; v < V; ++v)
    if (cams[v].width <= 0 || cams[v].height <= 0 || !cams[v].viewmatrix || !cams[v].projmatrix ||
        !cams[v].campos || !cams[v].bg || !(cams[v].tan_fovx > 0.f) || !(cams[v].tan_fovy > 0.f))
      return false;
  return true;
}

Views make_views(int V, const fgs_camera* cams, int bx, int by) {
  Views vs;
  vs.V = V; vs.bx = bx; vs.by = by;
  uint32_t tile_off = 0, pix_off = 0;
  for (int v = 0; v < V; ++v) {
    const fgs_camera& c = cams[v];
    set_view(vs.v[v], c.width, c.height, bx, by, c.viewmatrix, c.projmatrix, c.campos, c.bg, c.tan_fovx, c.tan_fovy,
             c.mult, c.scale_modifier);
    vs.v[v].tile_off = tile_off;
    vs.v[v].pix_off = pix_off;
    tile_off += (uint32_t)(vs.v[v].gx * vs.v[v].gy);
    pix_off += (uint32_t)(c.width * c.height);
  }
  vs.tiles = tile_off;
  return vs;
}

BatchLayout plan_for(int P, int V, const fgs_camera* cams, const fgs_tune_config* c, int64_t pairs) {
  std::vector<int> W(V), H(V);
  for (int v = 0; v < V; ++v) { W[v] = cams[v].width; H[v] = cams[v].height; }
  return plan(P, V, W.data(), H.data(), c->block_x, c->block_y, pairs, c->bucket_size, c->recompute != 0);
}

}  // namespace
}  // namespace fgs

using namespace fgs;

extern "C" fgs_status fgs_batch_workspace_bytes(int P, int num_views, const fgs_camera* cams,
                                                const fgs_tune_config* cfg, int64_t pair_capacity, size_t* bytes) {
  if (P < 0 || pair_capacity < 1 || !bytes || !cameras_ok(num_views, cams) || !config_ok(cfg))
    return FGS_ERR_BAD_ARG;
  if (pair_capacity > kMaxBatchPairs || (int64_t)num_views * P >= ((int64_t)1 << 32)) return FGS_ERR_CAPACITY;
  *bytes = plan_for(P, num_views, cams, cfg, pair_capacity).total;
  return FGS_OK;
}

extern "C" fgs_status fgs_render_batched_fwd(int P, int D, int M, const float* means3D,
                                             const float* colors_precomp, const float* dc, const float* shs,
                                             const float* opacities, const float* scales, const float* rotations,
                                             const uint8_t* culling, int num_views, const fgs_camera* cams,
                                             const fgs_tune_config* cfg, int64_t pair_capacity, void* workspace,
                                             size_t workspace_bytes, float* out_color, int32_t* radii,
                                             void* stream) {
  if (P < 0 || D < 0 || D > 3 || !cameras_ok(num_views, cams) || !config_ok(cfg) || pair_capacity < 1 ||
      !workspace || !out_color || (P > 0 && !radii))
    return FGS_ERR_BAD_ARG;
  if (pair_capacity > kMaxBatchPairs || (int64_t)num_views * P >= ((int64_t)1 << 32)) return FGS_ERR_CAPACITY;
  const int bucket_size = cfg->bucket_size;
  if (P > 0 && (!means3D || !opacities || !scales || !rotations)) return FGS_ERR_BAD_ARG;
  if (!colors_precomp && P > 0 && (!dc || (D > 0 && (!shs || M < (D + 1) * (D + 1) - 1)))) return FGS_ERR_BAD_ARG;
  if (((uintptr_t)workspace & 255) || ((uintptr_t)rotations & 15)) return FGS_ERR_BAD_ARG;
  const BatchLayout L = plan_for(P, num_views, cams, cfg, pair_capacity);
  if (workspace_bytes < L.total) return FGS_ERR_CAPACITY;
  char* ws = static_cast<char*>(workspace);
  cudaStream_t s = (cudaStream_t)stream;
  const Views views = make_views(num_views, cams, cfg->block_x, cfg->block_y);
  int32_t* curr = reinterpret_cast<int32_t*>(ws + L.curr);
  FGS_TRY(cudaMemsetAsync(curr, 0, sizeof(int32_t) * 4, s));
  if (P > 0) {
    PreArgs a;
    a.views = views;
    a.P = P; a.D = D; a.M = M;
    a.means = means3D; a.colors = colors_precomp; a.dc = dc; a.shs = shs; a.opac = opacities;
    a.scales = scales; a.rots = rotations; a.culling = culling;
    a.splat = reinterpret_cast<float*>(ws + L.records);
    a.keys = reinterpret_cast<unsigned long long*>(ws + L.keys_u);
    a.vals = reinterpret_cast<uint32_t*>(ws + L.vals_u);
    a.cap = pair_capacity;
    a.tasks = reinterpret_cast<uint32_t*>(ws + L.tasks);
    a.task_cap = pair_capacity / 2;
    a.curr = reinterpret_cast<unsigned int*>(curr);
    a.counters = reinterpret_cast<int*>(ws + L.counters);
    a.radii = radii;
    a.large_tiles = kLargeTiles;
    a.packet = cfg->packet;
    const fgs_status st = run_preprocess(a, s);
    if (st != FGS_OK) return st;
  }
  fgs_status st = run_sort(pair_capacity, curr, views.tiles, ws + L.sort_tmp, L.sort_bytes,
                           reinterpret_cast<uint64_t*>(ws + L.keys_u), reinterpret_cast<uint32_t*>(ws + L.vals_u),
                           reinterpret_cast<uint64_t*>(ws + L.keys_s), reinterpret_cast<uint32_t*>(ws + L.vals_s), s);
  if (st != FGS_OK) return st;
  const ImageState im = carve_image(ws + L.image, (size_t)L.pixels, L.tiles);
  const SampleState sm = carve_sample(ws + L.sample, L.buckets, cfg->recompute ? (int64_t)L.tiles : L.buckets);
  return run_render_fwd(views, pair_capacity, curr, bucket_size, reinterpret_cast<float*>(ws + L.records),
                        reinterpret_cast<uint64_t*>(ws + L.keys_s), reinterpret_cast<uint32_t*>(ws + L.vals_s),
                        reinterpret_cast<uint32_t*>(ws + L.ranges), out_color,
                        reinterpret_cast<int32_t*>(ws + L.last_contrib), reinterpret_cast<float*>(ws + L.ts_final),
                        im, sm, L.buckets, cfg->recompute != 0, s, cfg->chain > 0 ? cfg->chain : kChainBuckets);
}

extern "C" fgs_status fgs_render_batched_bwd(int P, int D, int M, const float* means3D, const float* dc,
                                             const float* shs, const float* scales, const float* rotations,
                                             int num_views, const fgs_camera* cams, const fgs_tune_config* cfg,
                                             int64_t pair_capacity, void* workspace, size_t workspace_bytes,
                                             const int32_t* radii, const float* dL_dpixels, float* dL_dmean3D,
                                             float* dL_ddc, float* dL_dsh, float* dL_dopacity, float* dL_dscale,
                                             float* dL_drot, float* dL_dcolor, float* dL_dcov3D,
                                             float* xyz_gradient_accum, float* xyz_gradient_accum_abs,
                                             float* max_radii, float* denom, void* stream) {
  if (P < 0 || D < 0 || D > 3 || !cameras_ok(num_views, cams) || !config_ok(cfg) || pair_capacity < 1 ||
      !workspace || (P > 0 && !radii) || !dL_dpixels)
    return FGS_ERR_BAD_ARG;
  if (pair_capacity > kMaxBatchPairs || (int64_t)num_views * P >= ((int64_t)1 << 32)) return FGS_ERR_CAPACITY;
  const int bucket_size = cfg->bucket_size;
  if (P == 0) return FGS_OK;
  if (!means3D || !scales || !rotations || !dL_dmean3D || !dL_ddc || !dL_dopacity || !dL_dscale || !dL_drot ||
      !dL_dcolor || !dL_dcov3D)
    return FGS_ERR_BAD_ARG;
  if (shs && (!dc || (D > 0 && M < (D + 1) * (D + 1) - 1) || !dL_dsh)) return FGS_ERR_BAD_ARG;
  if (((uintptr_t)workspace & 255) || ((uintptr_t)rotations & 15) || ((uintptr_t)dL_drot & 15))
    return FGS_ERR_BAD_ARG;
  const BatchLayout L = plan_for(P, num_views, cams, cfg, pair_capacity);
  if (workspace_bytes < L.total) return FGS_ERR_CAPACITY;
  char* ws = static_cast<char*>(workspace);
  cudaStream_t s = (cudaStream_t)stream;
  const Views views = make_views(num_views, cams, cfg->block_x, cfg->block_y);
  const ImageState im = carve_image(ws + L.image, (size_t)L.pixels, L.tiles);
  const SampleState sm = carve_sample(ws + L.sample, L.buckets, cfg->recompute ? (int64_t)L.tiles : L.buckets);
  float* grad = reinterpret_cast<float*>(ws + L.grad);
  fgs_status st = run_render_bwd(views, L.records_n, bucket_size, reinterpret_cast<uint32_t*>(ws + L.vals_s),
                                 reinterpret_cast<uint32_t*>(ws + L.ranges), reinterpret_cast<float*>(ws + L.records),
                                 reinterpret_cast<float*>(ws + L.ts_final),
                                 reinterpret_cast<int32_t*>(ws + L.last_contrib), im, sm, dL_dpixels, grad,
                                 cfg->recompute != 0, xyz_gradient_accum_abs != nullptr, s);
  if (st != FGS_OK) return st;
  PbwdArgs a;
  a.views = views;
  a.P = P; a.D = D; a.M = M;
  a.means = means3D; a.radii = radii; a.dc = dc; a.shs = shs; a.splat = reinterpret_cast<float*>(ws + L.records);
  a.scales = scales; a.rots = rotations; a.grad = grad;
  a.dmean2D = nullptr; a.dconic = nullptr; a.dopac = dL_dopacity; a.dcolor = dL_dcolor;
  a.dmean3D = dL_dmean3D; a.dcov3D = dL_dcov3D; a.ddc = dL_ddc; a.dsh = (M > 0) ? dL_dsh : nullptr;
  a.dscale = dL_dscale; a.drot = dL_drot;
  a.accum = xyz_gradient_accum; a.accum_abs = xyz_gradient_accum_abs; a.max_radii = max_radii; a.denom = denom;
  return run_preprocess_bwd(a, s);
}

extern "C" fgs_status fgs_render_batched_bwd_adam(int P, int D, int M, const float* means3D, const float* shs,
                                                  const float* opacities, const float* scales,
                                                  const float* rotations, int num_views, const fgs_camera* cams,
                                                  const fgs_tune_config* cfg, int64_t pair_capacity, void* workspace,
                                                  size_t workspace_bytes, const int32_t* radii,
                                                  const float* dL_dpixels, const fgs_adam_fused* adam,
                                                  float* xyz_gradient_accum, float* xyz_gradient_accum_abs,
                                                  float* max_radii, float* denom, void* stream) {
  if (P < 0 || D < 0 || D > 3 || !cameras_ok(num_views, cams) || !config_ok(cfg) || pair_capacity < 1 ||
      !workspace || (P > 0 && !radii) || !dL_dpixels)
    return FGS_ERR_BAD_ARG;
  if (pair_capacity > kMaxBatchPairs || (int64_t)num_views * P >= ((int64_t)1 << 32)) return FGS_ERR_CAPACITY;
  if (P == 0) return FGS_OK;
  if (!means3D || !scales || !rotations || !adam_args_ok(adam, shs, opacities)) return FGS_ERR_BAD_ARG;
  if (shs && D > 0 && M < (D + 1) * (D + 1) - 1) return FGS_ERR_BAD_ARG;
  if (((uintptr_t)workspace & 255) || ((uintptr_t)rotations & 15)) return FGS_ERR_BAD_ARG;
  const BatchLayout L = plan_for(P, num_views, cams, cfg, pair_capacity);
  if (workspace_bytes < L.total) return FGS_ERR_CAPACITY;
  char* ws = static_cast<char*>(workspace);
  cudaStream_t s = (cudaStream_t)stream;
  const Views views = make_views(num_views, cams, cfg->block_x, cfg->block_y);
  const ImageState im = carve_image(ws + L.image, (size_t)L.pixels, L.tiles);
  const SampleState sm = carve_sample(ws + L.sample, L.buckets, cfg->recompute ? (int64_t)L.tiles : L.buckets);
  float* grad = reinterpret_cast<float*>(ws + L.grad);
  fgs_status st = run_render_bwd(views, L.records_n, cfg->bucket_size, reinterpret_cast<uint32_t*>(ws + L.vals_s),
                                 reinterpret_cast<uint32_t*>(ws + L.ranges), reinterpret_cast<float*>(ws + L.records),
                                 reinterpret_cast<float*>(ws + L.ts_final),
                                 reinterpret_cast<int32_t*>(ws + L.last_contrib), im, sm, dL_dpixels, grad,
                                 cfg->recompute != 0, xyz_gradient_accum_abs != nullptr, s);
  if (st != FGS_OK) return st;
  PbwdArgs a;
  a.views = views;
  a.P = P; a.D = D; a.M = M;
  a.means = means3D; a.radii = radii; a.dc = nullptr; a.shs = shs; a.splat = reinterpret_cast<float*>(ws + L.records);
  a.scales = scales; a.rots = rotations; a.grad = grad;
  a.dmean2D = nullptr; a.dconic = nullptr; a.dopac = nullptr; a.dcolor = nullptr;
  a.dmean3D = nullptr; a.dcov3D = nullptr; a.ddc = nullptr; a.dsh = nullptr; a.dscale = nullptr; a.drot = nullptr;
  a.accum = xyz_gradient_accum; a.accum_abs = xyz_gradient_accum_abs; a.max_radii = max_radii; a.denom = denom;
  a.adam_on = 1; a.opac = opacities; a.adam = *adam;
  return run_preprocess_bwd(a, s);
}

extern "C" fgs_status fgs_batch_status(int P, int num_views, const fgs_camera* cams, const fgs_tune_config* cfg,
                                       int64_t pair_capacity, const void* workspace, int64_t* pairs,
                                       int64_t* buckets, void* stream) {
  if (P < 0 || !cameras_ok(num_views, cams) || !config_ok(cfg) || !workspace || pair_capacity < 1)
    return FGS_ERR_BAD_ARG;
  if (pair_capacity > kMaxBatchPairs) return FGS_ERR_CAPACITY;
  const BatchLayout L = plan_for(P, num_views, cams, cfg, pair_capacity);
  const char* ws = static_cast<const char*>(workspace);
  cudaStream_t s = (cudaStream_t)stream;
  int32_t k = 0;
  uint32_t b[2] = {0, 0};
  const ImageState im = carve_image(const_cast<char*>(ws) + L.image, (size_t)L.pixels, L.tiles);
  FGS_TRY(cudaMemcpyAsync(&k, ws + L.curr, sizeof(k), cudaMemcpyDeviceToHost, s));
  FGS_TRY(cudaMemcpyAsync(b, im.bucket_sum, sizeof(b), cudaMemcpyDeviceToHost, s));
  FGS_TRY(cudaStreamSynchronize(s));
  if (pairs) *pairs = (int64_t)(uint32_t)k;
  if (buckets) *buckets = b[1];
  if ((int64_t)(uint32_t)k > pair_capacity || (int64_t)b[1] > L.buckets) return FGS_ERR_CAPACITY;
  return FGS_OK;
}

extern "C" fgs_status fgs_batch_offsets(int P, int num_views, const fgs_camera* cams, const fgs_tune_config* cfg,
                                        int64_t pair_capacity, int64_t* offsets, int n) {
  if (P < 0 || !cameras_ok(num_views, cams) || !config_ok(cfg) || pair_capacity < 1 || !offsets || n < 10)
    return FGS_ERR_BAD_ARG;
  if (pair_capacity > kMaxBatchPairs) return FGS_ERR_CAPACITY;
  const BatchLayout L = plan_for(P, num_views, cams, cfg, pair_capacity);
  const int64_t v[10] = {(int64_t)L.curr,     (int64_t)L.records,      (int64_t)L.keys_u,  (int64_t)L.vals_u,
                         (int64_t)L.keys_s,   (int64_t)L.vals_s,       (int64_t)L.ranges,  (int64_t)L.last_contrib,
                         (int64_t)L.ts_final, (int64_t)L.grad};
  for (int i = 0; i < 10; ++i) offsets[i] = v[i];
  return FGS_OK;
}

// ---------------------------------------------------------------------------
// Autotuner (C entry of fastergs_gb300.tune.autotune).
namespace {
constexpr size_t kTuneAlign = 256;
size_t tune_up(size_t v) { return (v + kTuneAlign - 1) & ~(kTuneAlign - 1); }
// Float counts of the gradient arrays carved from the tuner's arena, in order:
// dmean3D, ddc, dsh, dopacity, dscale, drot, dcolor, dcov3D.
void tune_grad_sizes(int64_t P, int M, size_t (&n)[8]) {
  n[0] = 3 * P; n[1] = 3 * P; n[2] = 3 * (size_t)M * P; n[3] = P;
  n[4] = 3 * P; n[5] = 4 * P; n[6] = 3 * P; n[7] = 6 * P;
}
}  // namespace

extern "C" size_t fgs_tune_grad_bytes(int P, int M) {
  if (P < 0 || M < 0) return 0;
  size_t n[8];
  tune_grad_sizes(P, M, n);
  size_t total = 0;
  for (size_t v : n) total += tune_up(sizeof(float) * v);
  return total;
}

extern "C" fgs_status fgs_tune(int P, int D, int M, const float* means3D, const float* colors_precomp,
                               const float* dc, const float* shs, const float* opacities, const float* scales,
                               const float* rotations, const uint8_t* culling, int num_views, const fgs_camera* cams,
                               const fgs_tune_config* candidates, int n_candidates, int64_t pair_capacity,
                               void* workspace, size_t workspace_bytes, float* out_color, int32_t* radii,
                               const float* dL_dpixels, void* grad_arena, size_t grad_arena_bytes, int reps,
                               int* best, float* ms, void* stream) {
  if (!candidates || n_candidates < 1 || !best || !ms || reps < 1 || !workspace) return FGS_ERR_BAD_ARG;
  if (dL_dpixels && (!grad_arena || grad_arena_bytes < fgs_tune_grad_bytes(P, M) ||
                     ((uintptr_t)grad_arena & (kTuneAlign - 1))))
    return FGS_ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  float* g[8] = {nullptr};
  if (dL_dpixels) {
    size_t n[8];
    tune_grad_sizes(P, M, n);
    char* p = static_cast<char*>(grad_arena);
    for (int k = 0; k < 8; ++k) {
      g[k] = reinterpret_cast<float*>(p);
      p += tune_up(sizeof(float) * n[k]);
    }
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  FGS_TRY(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return FGS_ERR_CUDA;
  }
  auto step = [&](const fgs_tune_config* cfg) -> fgs_status {
    fgs_status st = fgs_render_batched_fwd(P, D, M, means3D, colors_precomp, dc, shs, opacities, scales, rotations,
                                           culling, num_views, cams, cfg, pair_capacity, workspace, workspace_bytes,
                                           out_color, radii, stream);
    if (st != FGS_OK || !dL_dpixels) return st;
    return fgs_render_batched_bwd(P, D, M, means3D, dc, shs, scales, rotations, num_views, cams, cfg, pair_capacity,
                                  workspace, workspace_bytes, radii, dL_dpixels, g[0], g[1], g[2],
                                  g[3], g[4], g[5], g[6], g[7], nullptr, nullptr, nullptr, nullptr, stream);
  };
  int chosen = -1;
  fgs_status result = FGS_OK;
  for (int i = 0; i < n_candidates; ++i) {
    ms[i] = -1.f;  // does not fit the workspace, is not a valid config, or failed
    size_t need = 0;
    if (fgs_batch_workspace_bytes(P, num_views, cams, candidates + i, pair_capacity, &need) != FGS_OK ||
        need > workspace_bytes)
      continue;
    if (step(candidates + i) != FGS_OK) continue;  // warm-up
    int64_t pairs = 0, buckets = 0;
    const fgs_status st = fgs_batch_status(P, num_views, cams, candidates + i, pair_capacity, workspace, &pairs,
                                           &buckets, stream);
    if (st == FGS_ERR_CAPACITY) {
      ms[i] = -2.f;  // the frame outgrew pair_capacity
      continue;
    }
    if (st != FGS_OK) continue;
    bool ok = cudaEventRecord(e0, s) == cudaSuccess;
    for (int r = 0; ok && r < reps; ++r) ok = step(candidates + i) == FGS_OK;
    ok = ok && cudaEventRecord(e1, s) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess;
    float t = 0.f;
    if (!ok || cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) {
      result = FGS_ERR_CUDA;
      break;
    }
    ms[i] = t / (float)reps;
    if (chosen < 0 || ms[i] < ms[chosen]) chosen = i;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *best = chosen;
  if (result != FGS_OK) return result;
  return chosen < 0 ? FGS_ERR_CAPACITY : FGS_OK;
}
