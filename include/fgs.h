/*
 * fgs.h - C ABI of the GB300 (sm_103a) Gaussian-splatting rasterizer.
 *
 * Drop-in for the CUDA backend of FasterGS
 * (gs_submodules/diff-gaussian-rasterization_faster, "FB" below).  Every entry
 * point takes plain device pointers, sizes and a cudaStream_t passed as void*,
 * launches its kernels on that stream, never allocates, and returns an
 * fgs_status.  Nothing here synchronises the stream unless a parameter asks
 * for a host-side value (documented per function).
 *
 * Tensor layouts are FB's: means (P,3), opacities (P,1), scales (P,3),
 * rotations (P,4) raw quaternions (r,x,y,z), dc (P,1,3), shs (P,M,3),
 * column-major 4x4 view / full-projection matrices, images (3,H,W),
 * per-pixel buffers (H,W,1), 64-bit keys (tile << 32 | float bits of depth).
 */
#ifndef FGS_H_
#define FGS_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  FGS_OK = 0,
  FGS_ERR_BAD_ARG = 1,        /* null / misaligned pointer, bad size or shape */
  FGS_ERR_CAPACITY = 2,       /* a caller-provided buffer is too small */
  FGS_ERR_CUDA = 3,           /* a CUDA runtime call or launch failed */
  FGS_ERR_TIMEOUT = 4,        /* a bounded device-side wait gave up */
  FGS_ERR_UNSUPPORTED = 5     /* valid call that this build does not implement */
} fgs_status;

/* Number of int32 words of the device counter block used by fgs_preprocess. */
#define FGS_COUNTER_WORDS 16
/* Floats per Gaussian of the interleaved gradient record written by
 * fgs_render_bwd: [dmean2D.xyzw | conic moments | dcolor.rgb, dopacity].
 * The conic moments are -1/2 x (sum dp w^2, sum dp w dy, 0, sum dp dy^2)
 * over the Gaussian's pixels, dp = dL/d(exponent), in the frame
 * w = dx + P dy of the splat record's exponent (P = record float 7);
 * fgs_preprocess_bwd turns them into FB's dL/dconic. */
#define FGS_GRAD_STRIDE 12
/* Floats per Gaussian of the splat record (FB rasterizer_imp.h:27-38). */
#define FGS_SPLAT_STRIDE 32

const char* fgs_status_string(int status);
/* Build identification, e.g. "fgs 0.1 sm_103a". */
const char* fgs_version(void);

/* Reads and optionally clears the device error word that kernels set when a
 * bounded wait gives up (bit 0) or a capacity check skips writes (bit 1).
 * Synchronises the stream.  *flags receives the word. */
fgs_status fgs_device_errors(int* flags, int clear, void* stream);

/* Writes [*curr_offset, counters[0]] (either may be NULL: 0) into host_out,
 * two int32 of page-locked host memory, with a one-thread kernel that stores
 * through the buffer's mapped device address: the read of a frame's pair and
 * task counts then never queues behind large copies on the copy engines.
 * Falls back to cudaMemcpyAsync when host_out is not mapped.  The caller
 * synchronises the stream before reading host_out. */
fgs_status fgs_read_counts(const int32_t* curr_offset, const int32_t* counters, int32_t* host_out, void* stream);

/* Self-check of the bounded device waits: one warp runs the wait of the
 * compositing chain on `flag` (one device u32, zeroed here), which nothing
 * sets; the wait gives up after its bounded spin (about a second), raises the
 * timeout bit (bit 0) in the device error word and the kernel returns, so
 * the context stays usable.  Read the bit with fgs_device_errors. */
fgs_status fgs_selftest_wait(uint32_t* flag, void* stream);

/*
 * Per-Gaussian preprocess and (tile, Gaussian) key emission.
 * Replaces faster::preprocess (FB csrc/ops.h:71-85, body
 * csrc/cuda_rasterizer/preprocess.cu:928-971).
 *
 * Small-footprint Gaussians (rect < 128 tiles) are packed across warp lanes;
 * large ones are split into 128-tile sub-tasks queued in task_scratch
 * (FB keeps the same queue in gaussian_values_sorted) and drained by a second
 * kernel without a host round trip.  Appends K pairs at *curr_offset, which
 * the caller zeroes beforehand, exactly like FB.  Writes past pair_capacity
 * are skipped while *curr_offset keeps counting, so the caller detects
 * overflow by comparing K with the capacity.  counters: device int32
 * [FGS_COUNTER_WORDS], zeroed here.  radii (P) is fully written.
 */
fgs_status fgs_preprocess(
    int P, int D, int M,
    const float* means3D, const float* colors_precomp, const float* dc, const float* shs,
    const float* opacities, const float* scales, const float* rotations, float scale_modifier,
    int width, int height, int block_x, int block_y,
    const float* campos, const float* viewmatrix, const float* projmatrix,
    float tan_fovx, float tan_fovy, float zfar, float znear, float mult, const uint8_t* culling,
    float* splat_buffer, int64_t splat_rows,
    uint64_t* keys_unsorted, uint32_t* values_unsorted, int64_t pair_capacity,
    uint32_t* task_scratch, int64_t task_scratch_words,
    int32_t* curr_offset, int32_t* counters, int32_t* radii, void* stream);

/* Temporary bytes fgs_sort needs for up to num_rendered pairs.
 * Replaces faster::get_sort_buffer_size (FB csrc/ops.h:94, sort.cu:46-54). */
size_t fgs_sort_temp_bytes(int64_t num_rendered);

/*
 * Stable ascending LSD radix sort of (key, value) pairs on the key bits
 * that can differ: 31 depth bits and ceil(log2(tiles)) tile bits,
 * tiles = ceil(W/bx)*ceil(H/by).  Keys are (tile << 32) | the bits of a
 * positive float depth, so bit 31 is zero (FB's keys, whose depths exceed
 * the 0.2 near cut); a key with bit 31 set raises the capacity bit of the
 * device error word.
 * Replaces faster::sort_gaussian (FB csrc/ops.h:87-92, sort.cu:28-44), which
 * calls cub::DeviceRadixSort::SortPairs.  Inputs are not modified.
 */
fgs_status fgs_sort(int64_t num_rendered, int width, int height, int block_x, int block_y,
                    void* temp, size_t temp_bytes,
                    const uint64_t* keys_in, const uint32_t* values_in,
                    uint64_t* keys_out, uint32_t* values_out, void* stream);

/*
 * fgs_sort for callers that cannot allocate device memory when they sort
 * (code inside a memory pool or arena it does not own, hosts that forbid
 * allocation after start-up, real-time loops that must not stall on
 * cudaMalloc).  No counterpart in the reference.  The scratch is a
 * library-owned static device array sized for FGS_SORT_NOALLOC_MAX_PAIRS
 * pairs (about 14 MiB, held by every GPU that loads the library until the
 * process exits); larger num_rendered returns FGS_ERR_CAPACITY.  The first
 * call on a device looks up the array's device address, so make that first
 * call before any stream capture; the address is cached per CUDA context and
 * looked up again after cudaDeviceReset or under another context of the same
 * device (make that first call outside capture too).  All calls share the
 * array: calls that
 * overlap on the GPU (other streams, other threads) race and must be
 * serialised by the caller.  Calls no allocator.
 */
#define FGS_SORT_NOALLOC_MAX_PAIRS (1 << 20)
fgs_status fgs_sort_noalloc(int64_t num_rendered, int width, int height, int block_x, int block_y,
                            const uint64_t* keys_in, const uint32_t* values_in,
                            uint64_t* keys_out, uint32_t* values_out, void* stream);

/* [start, end) of every tile in a sorted key list; ranges is (tiles, 2) u32
 * and is zeroed first.  Replaces identifyTileRanges and its launch
 * (FB render.cu:54-79, :406-412). */
fgs_status fgs_tile_ranges(int64_t num_rendered, int num_tiles, const uint64_t* keys_sorted,
                           uint32_t* ranges, void* stream);

/* Upper bound on the composited bucket count of a frame with num_rendered
 * pairs: the units of the sample state.  bucket_size is the merge's stop
 * granularity (FB's BUCKET_SIZE, 128); buckets larger than 64 Gaussians are
 * composited as 64-Gaussian sub-buckets, each with its own prefix sample, and
 * the transmittance stop is tested only at the end of a full bucket. */
int64_t fgs_max_buckets(int64_t num_rendered, int width, int height, int block_x, int block_y,
                        int bucket_size);

/* Bytes of the per-image state and per-bucket sample state that fgs_render_fwd
 * fills and fgs_render_bwd consumes (FB ImageState / SampleState,
 * rasterizer_imp.h:76-102, rasterizer_imp.cu:7-48). */
fgs_status fgs_state_bytes(int width, int height, int block_x, int block_y, int64_t max_buckets,
                           size_t* image_bytes, size_t* sample_bytes);

/*
 * Forward composite: tile ranges, bucket bookkeeping, parallel per-bucket
 * compositing and the associative (colour, transmittance) merge.
 * Replaces faster::render_16x16 (FB csrc/ops.h:96-106, render.cu:393-470).
 * out_color (3,H,W), last_contributor (H,W), Ts_final (H,W) are written.
 * If bucket_sum_host is non-NULL the stream is synchronised at the end and
 * the count of buckets of bucket_size Gaussians is stored there (FB returns
 * it to Python; it does not count sub-buckets).
 */
fgs_status fgs_render_fwd(int P, int64_t num_rendered, int width, int height, int block_x, int block_y,
                          int bucket_size, const float* splat_buffer, const uint64_t* keys_sorted,
                          const uint32_t* values_sorted, uint32_t* ranges, const float* bg,
                          float* out_color, int32_t* last_contributor, float* Ts_final,
                          void* image_state, size_t image_bytes, void* sample_state, size_t sample_bytes,
                          int64_t max_buckets, uint32_t* bucket_sum_host, void* stream);

/*
 * Backward composite, bucket-parallel, front-to-back inside each bucket.
 * Replaces faster::render_backward (FB csrc/ops.h:123-135,
 * backward.cu:956-977).  grad_record (P, FGS_GRAD_STRIDE) is zeroed here and
 * accumulated with vector reductions.  flags = 0 computes every slot, as FB
 * does; FGS_BWD_NO_ABS skips the |dL/dmean2D| sums, whose only consumer is
 * the xyz_gradient_accum_abs statistic.
 */
#define FGS_BWD_NO_ABS 1  /* flags: leave dmean2D.zw (the sums of |dL/dmean2D|) at zero */
fgs_status fgs_render_bwd(int P, int width, int height, int block_x, int block_y, int bucket_size,
                          const uint32_t* values_sorted, const uint32_t* ranges, const float* bg,
                          const float* splat_buffer, const float* Ts_final, const int32_t* last_contributor,
                          const void* image_state, const void* sample_state, int64_t max_buckets,
                          const float* dL_dpixels, float* grad_record, int flags, void* stream);

/*
 * Per-Gaussian backward of projection, EWA covariance, SH and 3D covariance;
 * scatters the render gradients into FB's output tensors and, when
 * xyz_gradient_accum is non-NULL, accumulates densification statistics.
 * Replaces faster::preprocess_backward + add_densification_stats
 * (FB csrc/ops.h:108-121,137-145; backward.cu:922-954,980-999) and the
 * output allocation of backward_torch (FB csrc/pybind.cpp:258-267).
 * All outputs are fully written (zeros where FB leaves zeros).  dL_dmean2D,
 * dL_dconic, dL_dcolor and dL_dcov3D may be NULL: an autograd step needs
 * none of them unless colours or covariances are precomputed.
 */
fgs_status fgs_preprocess_bwd(
    int P, int D, int M, const float* means3D, const int32_t* radii, const float* dc, const float* shs,
    const float* splat_buffer, const float* scales, const float* rotations, float scale_modifier,
    const float* viewmatrix, const float* projmatrix, int width, int height, float tan_fovx, float tan_fovy,
    const float* campos, const float* grad_record,
    float* dL_dmean2D, float* dL_dconic, float* dL_dopacity, float* dL_dcolor,
    float* dL_dmean3D, float* dL_dcov3D, float* dL_ddc, float* dL_dsh, float* dL_dscale, float* dL_drot,
    float* xyz_gradient_accum, float* xyz_gradient_accum_abs, float* max_radii, float* denom,
    void* stream);

/* Densification statistics alone (FB backward.cu:892-918).  Each output is
 * optional; dL_dmean2D is (P,4). */
fgs_status fgs_densify_stats(int P, const int32_t* radii, const float* dL_dmean2D, float* xyz_gradient_accum,
                             float* xyz_gradient_accum_abs, float* max_radii, float* denom, void* stream);

/*
 * Importance pass (FB render_16x16_simp, csrc/ops.h; pybind.cpp:179-208;
 * render_simp.cu): per Gaussian the sum of blend weights alpha T over the
 * pixels of its tiles, the number of pixels where alpha >= 1/255, and the
 * number of pixels where it has the largest weight; each 16x16 tile composites
 * its list in order and stops after a pair of Gaussians once all its pixels
 * have T < 1e-4.  Computes the tile ranges first (like FB).  Outputs (P) are
 * zeroed and fully written.
 */
fgs_status fgs_render_simp(int P, int64_t num_rendered, int width, int height, const float* splat_buffer,
                           const uint64_t* keys_sorted, const uint32_t* values_sorted, uint32_t* ranges,
                           float* accum_weights, int32_t* accum_count, float* accum_max_count, void* stream);

/*
 * Depth pass (FB render_16x16_depth; pybind.cpp:135-176; render_depth.cu):
 * per pixel, along the ray through the pixel, the Gaussian of largest weight
 * gives out_pts (3,H,W) (closest point of its 3-sigma ellipsoid to the ray),
 * out_depth (H,W), discriminants (H,W) and gidx (H,W); accum_alpha (H,W) is
 * the final transmittance.  means3D (P,3), scales (P,3) activated without
 * the scale modifier, rotations (P,4), projmatrix the full projection,
 * campos (3).
 */
fgs_status fgs_render_depth(int P, int64_t num_rendered, int width, int height, const float* splat_buffer,
                            const uint64_t* keys_sorted, const uint32_t* values_sorted, uint32_t* ranges,
                            const float* means3D, const float* scales, const float* rotations,
                            const float* projmatrix, const float* campos, float* out_pts, float* out_depth,
                            float* accum_alpha, int32_t* gidx, float* discriminants, void* stream);

/* Masked Adam step over N rows of M floats; rows with visible[i]==0 are left
 * untouched.  Replaces ADAM::adamUpdate (FB adam.h, adam.cu:9-66). */
fgs_status fgs_adam_update(float* param, const float* grad, float* exp_avg, float* exp_avg_sq,
                           const uint8_t* visible, float lr, float b1, float b2, float eps,
                           uint32_t N, uint32_t M, void* stream);

/*
 * Sparse Adam fused into the preprocess backward.  FB's training step writes
 * every per-Gaussian gradient (dL/dmean3D, dc, sh, opacity, scale, rotation:
 * 59 floats per Gaussian at SH degree 3), lets autograd push them through the
 * activations (sigmoid, exp, normalize), and reads them back in
 * SparseGaussianAdam.step (FB __init__.py:267-298, adam.cu:9-38).  The fused
 * form applies the activation backward and FB's masked Adam step to the raw
 * parameters in the kernel that produces the gradients; no gradient reaches
 * memory.  A Gaussian is stepped when its radius is > 0 in at least one view
 * (FB: visible = radii > 0).
 *
 * Groups (the names FasterGS's optimisers give their parameter groups):
 * xyz (P,3), f_dc (P,1,3), f_rest (P,M,3), opacity (P,1), scaling (P,3),
 * rotation (P,4); a group whose param is NULL is not stepped.  Step sizes are
 * already multiplied by FB's bias compensation sqrt(1 - b2^t) / (1 - b1^t):
 * lr_value by value, or, when lr is not NULL, FGS_ADAM_GROUPS device floats
 * at lr, so that a captured CUDA graph picks up step sizes written between
 * replays.  Activations: opacities =
 * sigmoid(raw), scales = exp(raw), rotations = raw / |raw| (FGS_ACT_*), or
 * identity where the rasterizer is given the raw tensor itself.
 */
enum {
  FGS_ADAM_XYZ = 0, FGS_ADAM_F_DC = 1, FGS_ADAM_F_REST = 2, FGS_ADAM_OPACITY = 3, FGS_ADAM_SCALING = 4,
  FGS_ADAM_ROTATION = 5, FGS_ADAM_GROUPS = 6
};
enum { FGS_ACT_IDENTITY = 0, FGS_ACT_SIGMOID = 1, FGS_ACT_EXP = 2, FGS_ACT_NORMALIZE = 3 };
typedef struct {
  float* param[FGS_ADAM_GROUPS];
  float* exp_avg[FGS_ADAM_GROUPS];
  float* exp_avg_sq[FGS_ADAM_GROUPS];
  const float* lr;                /* device step sizes, or NULL: lr_value */
  float lr_value[FGS_ADAM_GROUPS];
  float eps[FGS_ADAM_GROUPS];
  float b1, b2;
  int opacity_act;                /* FGS_ACT_SIGMOID or FGS_ACT_IDENTITY */
  int scaling_act;                /* FGS_ACT_EXP or FGS_ACT_IDENTITY */
  int rotation_act;               /* FGS_ACT_NORMALIZE or FGS_ACT_IDENTITY */
} fgs_adam_fused;

/* fgs_preprocess_bwd with the sparse Adam step in place of the gradient
 * outputs.  opacities (P) are the activated opacities the forward used
 * (needed for FGS_ACT_SIGMOID).  f_rest rows are staged in shared memory:
 * M <= 16 when shs is given and D > 0.  Densification statistics as in
 * fgs_preprocess_bwd. */
fgs_status fgs_preprocess_bwd_adam(
    int P, int D, int M, const float* means3D, const int32_t* radii, const float* shs,
    const float* splat_buffer, const float* opacities, const float* scales, const float* rotations,
    float scale_modifier, const float* viewmatrix, const float* projmatrix, int width, int height,
    float tan_fovx, float tan_fovy, const float* campos, const float* grad_record, const fgs_adam_fused* adam,
    float* xyz_gradient_accum, float* xyz_gradient_accum_abs, float* max_radii, float* denom, void* stream);

/*
 * SSIM (the fused-ssim extension FasterGS's backbones train with,
 * gs_submodules/fused-ssim/ssim.cu; the SSIM of 3DGS/utils/loss_utils.py:33-63):
 * 11-tap Gaussian window of sigma 1.5, zero padding.  Images are `planes`
 * contiguous H x W float planes (batch x channels).
 *
 * fgs_ssim_fwd: the SSIM map, and, when dm_dmu1 / dm_dsigma1_sq / dm_dsigma12
 * are given (all or none), the map's partial derivatives w.r.t. mu1, E[x^2]
 * and E[xy] that fgs_ssim_bwd needs (fusedssim, ssim.cu:185-285).
 * fgs_ssim_bwd: dL/dimg1 from dL/dmap (fusedssim_backward, ssim.cu:287-365).
 */
fgs_status fgs_ssim_fwd(int planes, int H, int W, float C1, float C2, const float* img1, const float* img2,
                        float* ssim_map, float* dm_dmu1, float* dm_dsigma1_sq, float* dm_dsigma12, void* stream);
fgs_status fgs_ssim_bwd(int planes, int H, int W, const float* img1, const float* img2, const float* dL_dmap,
                        const float* dm_dmu1, const float* dm_dsigma1_sq, const float* dm_dsigma12,
                        float* dL_dimg1, void* stream);

/*
 * The training loss of FasterGS's backbones in one pass with its gradient
 * (taming-3dgs/train_faster.py:121-125, FastGS/train_faster.py:105-109):
 *   loss = (1 - lambda) mean|img - gt| + lambda (1 - mean SSIM(img, gt)),
 * C1 = 0.01^2, C2 = 0.03^2, "same" padding.  Writes *loss, *ssim_mean
 * (optional) and dL_dimg = dloss/dimg (device), never the SSIM map.  scratch:
 * fgs_l1_dssim_scratch_bytes(planes, H, W) bytes, 8-byte aligned.
 */
size_t fgs_l1_dssim_scratch_bytes(int planes, int H, int W);
fgs_status fgs_l1_dssim(int planes, int H, int W, float lambda, const float* img, const float* gt, void* scratch,
                        size_t scratch_bytes, float* loss, float* ssim_mean, float* dL_dimg, void* stream);

/*
 * Batched multi-camera rendering.  No counterpart in FB, which renders one
 * camera per call and reads the pair and bucket counts back to the host
 * three times per step (FB __init__.py:106-132, rasterizer_imp.cu:141-147),
 * so it cannot be captured in a CUDA graph.  Here one call renders up to
 * FGS_MAX_VIEWS cameras of different resolutions with one launch per stage
 * (preprocess with grid.y = camera, one sort over a global tile index space,
 * one persistent composite launch over the buckets of every camera, one
 * merge), with no host synchronisation, so fwd and bwd can be captured in a
 * CUDA graph and replayed.  Capacities are fixed by the caller; a frame that
 * overflows pair_capacity skips the extra writes, latches a device flag and
 * is reported by fgs_batch_status.
 *
 * Per-camera outputs are concatenated: camera k's image (3, H_k, W_k) starts
 * at float offset 3 * sum_{j<k} H_j W_j of out_color / dL_dpixels, and its
 * radii at k * P of radii (num_views, P).
 */
#define FGS_MAX_VIEWS 32
typedef struct {
  const float* viewmatrix;  /* 4x4 column-major world -> view, device */
  const float* projmatrix;  /* 4x4 column-major full projection, device */
  const float* campos;      /* 3, device */
  const float* bg;          /* 3, device */
  int width, height;
  float tan_fovx, tan_fovy;
  float scale_modifier;     /* FB GaussianRasterizationSettings.scale_modifier */
  float mult;               /* FB GaussianRasterizationSettings.mult */
} fgs_camera;

/* Launch configuration picked by the autotuner; FB's fixed choice is
 * {128, 16, 16, 4, 0}.  bucket_size 1..128 Gaussians per bucket; tile 16x16,
 * 8x32 or 32x8 pixels; packet 1, 2, 4 or 8: the small-footprint packing
 * width of the preprocess, i.e. how many consecutive candidate tiles of the
 * warp's flattened list each lane tests per step (FB packs one per lane;
 * footprints of 128 tiles or more are split into 128-tile sub-tasks as FB
 * does).  The tile shape and the bucket size change images at the level of
 * the T < 1e-4 stopping rule (which acts per bucket; a 128-Gaussian bucket is
 * composited as two 64-Gaussian sub-buckets with the stop tested after the
 * second, as for fgs_render_fwd); packet changes only the order in which
 * pairs are emitted (the sort keeps equal keys in that order).
 * chain 1..4096 (0: 8): the length of each tile's fold chain in the forward
 * composite, in composited (sub-)buckets; a tile's later buckets composite
 * without waiting and are folded pixel-parallel afterwards.  Results are
 * bit-identical for every length; it only moves time between the chain's
 * serial links and the speculative compositing of deep tiles.
 * recompute 1: the forward keeps one running (colour, transmittance) prefix
 * per tile instead of one per (sub-)bucket (4 KB each), and the backward
 * rebuilds each one's prefix from it -- bit-identical prefixes, a
 * workspace smaller by about 4 KB per (sub-)bucket, one extra compositing
 * pass over the needed buckets. */
typedef struct {
  int bucket_size;
  int block_x, block_y;
  int packet;
  int recompute;
  int chain;
} fgs_tune_config;

/* Workspace bytes (256-byte aligned base required) of a batched frame. */
fgs_status fgs_batch_workspace_bytes(int P, int num_views, const fgs_camera* cams, const fgs_tune_config* cfg,
                                     int64_t pair_capacity, size_t* bytes);

/* Forward of every camera: out_color (concatenated images), radii
 * (num_views, P).  Inputs use FB's layouts; colors_precomp replaces
 * dc/shs when non-NULL; culling (P) is optional. */
fgs_status fgs_render_batched_fwd(int P, int D, int M, const float* means3D, const float* colors_precomp,
                                  const float* dc, const float* shs, const float* opacities, const float* scales,
                                  const float* rotations, const uint8_t* culling, int num_views,
                                  const fgs_camera* cams, const fgs_tune_config* cfg, int64_t pair_capacity,
                                  void* workspace, size_t workspace_bytes, float* out_color, int32_t* radii,
                                  void* stream);

/* Backward of the last fgs_render_batched_fwd on the same workspace.
 * Gradients are summed over cameras and fully written; the optional
 * densification statistics are accumulated once per camera, as FB's
 * per-camera backward does.  dL_dcolor (P,3) and dL_dcov3D (P,6) are
 * summed over cameras too. */
fgs_status fgs_render_batched_bwd(int P, int D, int M, const float* means3D, const float* dc, const float* shs,
                                  const float* scales, const float* rotations, int num_views,
                                  const fgs_camera* cams, const fgs_tune_config* cfg, int64_t pair_capacity,
                                  void* workspace, size_t workspace_bytes, const int32_t* radii,
                                  const float* dL_dpixels, float* dL_dmean3D, float* dL_ddc, float* dL_dsh,
                                  float* dL_dopacity, float* dL_dscale, float* dL_drot, float* dL_dcolor,
                                  float* dL_dcov3D, float* xyz_gradient_accum, float* xyz_gradient_accum_abs,
                                  float* max_radii, float* denom, void* stream);

/* fgs_render_batched_bwd with the sparse Adam step fused into its preprocess
 * backward (see fgs_adam_fused): gradients summed over the cameras step the
 * raw parameters of every Gaussian that some camera saw. */
fgs_status fgs_render_batched_bwd_adam(int P, int D, int M, const float* means3D, const float* shs,
                                       const float* opacities, const float* scales, const float* rotations,
                                       int num_views, const fgs_camera* cams, const fgs_tune_config* cfg,
                                       int64_t pair_capacity, void* workspace, size_t workspace_bytes,
                                       const int32_t* radii, const float* dL_dpixels, const fgs_adam_fused* adam,
                                       float* xyz_gradient_accum, float* xyz_gradient_accum_abs,
                                       float* max_radii, float* denom, void* stream);

/*
 * Autotuner over launch configurations (the C entry of
 * fastergs_gb300.tune.autotune; FB fixes bucket 128, 16x16 tiles and the
 * 128-tile sub-task size at compile time).  For every candidate: skipped
 * (ms = -1) unless its fgs_batch_workspace_bytes fits workspace_bytes; one
 * warm-up frame, skipped (ms = -2) if it overflows pair_capacity; then `reps`
 * frames timed with CUDA events on the stream, ms = mean per frame.  A frame
 * is the batched forward, plus the backward when dL_dpixels is given (its
 * gradients go to grad_arena, fgs_tune_grad_bytes(P, M) bytes, 256-byte
 * aligned; densification statistics are not touched).  *best receives the
 * index of the fastest candidate; FGS_ERR_CAPACITY when none ran.
 * Synchronises the stream.
 */
size_t fgs_tune_grad_bytes(int P, int M);
fgs_status fgs_tune(int P, int D, int M, const float* means3D, const float* colors_precomp, const float* dc,
                    const float* shs, const float* opacities, const float* scales, const float* rotations,
                    const uint8_t* culling, int num_views, const fgs_camera* cams, const fgs_tune_config* candidates,
                    int n_candidates, int64_t pair_capacity, void* workspace, size_t workspace_bytes,
                    float* out_color, int32_t* radii, const float* dL_dpixels, void* grad_arena,
                    size_t grad_arena_bytes, int reps, int* best, float* ms, void* stream);

/* Reads the pair and bucket counts of the last batched forward on this
 * workspace (synchronises the stream).  Returns FGS_ERR_CAPACITY when the
 * frame overflowed pair_capacity (or its bucket bound); the counts are then
 * the sizes the frame needed. */
fgs_status fgs_batch_status(int P, int num_views, const fgs_camera* cams, const fgs_tune_config* cfg,
                            int64_t pair_capacity, const void* workspace, int64_t* pairs, int64_t* buckets,
                            void* stream);

/* Byte offsets inside a batched workspace, for inspection and tests:
 * [0] pair count (int32), [1] splat records (num_views*P, FGS_SPLAT_STRIDE
 * floats, record = camera * P + Gaussian), [2] unsorted keys, [3] unsorted
 * values, [4] sorted keys (u64, global tile << 32 | depth), [5] sorted
 * values (record indices), [6] tile ranges (u32 pairs over the global tile
 * index space, camera after camera), [7] last contributor (int32 per pixel,
 * cameras concatenated), [8] final transmittance, [9] gradient records
 * (num_views*P, FGS_GRAD_STRIDE).  n >= 10. */
fgs_status fgs_batch_offsets(int P, int num_views, const fgs_camera* cams, const fgs_tune_config* cfg,
                             int64_t pair_capacity, int64_t* offsets, int n);

/* Kernel-level timing for benchmarks.  While enabled for a kernel id, the
 * library records a CUDA event pair around every launch of that kernel on its
 * launch stream; fgs_kernel_timer_read synchronises those events and returns
 * the summed device time and the number of kernel launches inside the timed
 * regions since the last read (FGS_K_BUCKET_SETUP times its three kernels as
 * one region; FGS_K_READ_COUNTS is the one-thread store of the pair and task
 * counts that fgs_read_counts launches; FGS_K_BWD_LIST builds the backward's
 * list of buckets that some pixel reaches; FGS_K_DEEP_MERGE folds the buckets
 * of deep tiles past their chain; FGS_K_ZERO is the zero fill of counters,
 * tile ranges, sort look-back words and gradient records, a kernel so that
 * the programmatic dependent launches of the path stay chained).  No
 * counterpart in FB (its DEBUG_TIME macros are unused, ops.h:10-14). */
enum {
  FGS_K_PREPROCESS = 0, FGS_K_PREPROCESS_LARGE = 1, FGS_K_SORT_HIST = 2, FGS_K_SORT_PASS = 3,
  FGS_K_TILE_RANGES = 4, FGS_K_BUCKET_SETUP = 5, FGS_K_RENDER_FWD = 6, FGS_K_EMPTY_TILES = 7,
  FGS_K_RENDER_BWD = 8, FGS_K_PREPROCESS_BWD = 9, FGS_K_LOSS = 10, FGS_K_SIMP = 11, FGS_K_DEPTH = 12,
  FGS_K_READ_COUNTS = 13, FGS_K_BWD_LIST = 14, FGS_K_DEEP_MERGE = 15, FGS_K_ZERO = 16, FGS_K_COUNT = 17
};
fgs_status fgs_kernel_timer(int kernel_id, int enable);
fgs_status fgs_kernel_timer_read(int kernel_id, double* total_ms, int* launches);

/* FP32 FMA throughput of this GPU in TFLOP/s (8 independent FMA chains per
 * thread on every SM; synchronises the stream): the ceiling for the
 * compositing kernels, which are bound by FP32 issue, not by HBM. */
fgs_status fgs_peak_fp32(double* tflops, void* stream);
/* The same with packed fma.rn.f32x2 (two FMAs per instruction, 4 FLOP), the
 * form the compositing kernels issue their pixel pairs in. */
fgs_status fgs_peak_fp32x2(double* tflops, void* stream);
/* MUFU ex2.approx throughput in Gop/s (8 independent chains per thread on
 * every SM; synchronises the stream): one ex2 per pixel-Gaussian evaluation
 * in both compositing kernels. */
fgs_status fgs_peak_ex2(double* gops, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FGS_H_ */
