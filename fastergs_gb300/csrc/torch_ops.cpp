// The compiled `_C` of the drop-in package `diff_gaussian_rasterization_faster`.
//
// A PyTorch C++ extension over the C ABI of libfgs.so (include/fgs.h): each op
// checks its tensors, takes raw device pointers, allocates its outputs with
// torch and calls the C entry on torch's current stream.  The `ops` submodule
// carries the names, argument order, tensor shapes and dtypes of the
// reference backend's binding (FB csrc/pybind.cpp:371-416: preprocess,
// sort_gaussian, get_sort_buffer_size, render_16x16, render_simp,
// render_depth, backward, adamUpdate), so FB's Python layer and every
// backbone's --fastergs path call it unchanged.  Extra keyword arguments
// (render_16x16's read_bucket_sum, backward's abs_grad / minimal) default to
// FB's behaviour.
//
// Built by fastergs_gb300/build.py with g++ against the installed torch and
// linked to libfgs.so; no CUDA code lives here.
#include <ATen/ATen.h>
#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>
#include <torch/csrc/utils/pybind.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>

#include "fgs.h"

namespace {

using at::Tensor;

constexpr int kTile = 16;
constexpr int kBucket = 128;
// The sample state is handed to Python as a (rows, kSampleRow) byte tensor with
// rows = max_buckets + 1, so its first dimension carries the bucket capacity
// the forward reserved to the backward (per bucket: 256 16-byte prefix samples,
// its owner tile, queue slot and live-list entry).
constexpr int64_t kSampleRow = 4120;

void check(int status, const char* fn) {
  if (status != FGS_OK) throw std::runtime_error(std::string(fn) + " failed: " + fgs_status_string(status));
}

void* ptr(const Tensor& t) { return (t.defined() && t.numel() != 0) ? t.data_ptr() : nullptr; }

bool nonempty(const Tensor& t) { return t.defined() && t.numel() != 0; }

at::Device cuda_device_of(const Tensor& t) {
  if (!t.is_cuda()) throw std::invalid_argument("the rasterizer runs on CUDA tensors only (no CPU fallback)");
  return t.device();
}

// Contiguous float32 tensor on dev, or an undefined tensor for "absent" (empty).
Tensor f32(const char* name, const Tensor& t, const at::Device& dev) {
  if (!nonempty(t)) return Tensor();
  if (t.scalar_type() != at::kFloat) throw std::invalid_argument(std::string(name) + " must be float32");
  if (t.device() != dev) throw std::invalid_argument(std::string(name) + " must be on " + dev.str());
  return t.contiguous();
}

void need(const char* name, const Tensor& t, at::ScalarType dt, const at::Device& dev) {
  if (!t.defined() || t.scalar_type() != dt || !t.is_contiguous() || t.device() != dev)
    throw std::invalid_argument(std::string(name) + " must be a contiguous " + c10::toString(dt) + " tensor on " +
                                dev.str());
}

cudaStream_t stream_of(const at::Device& dev) { return c10::cuda::getCurrentCUDAStream(dev.index()).stream(); }

// Work counters of fgs_preprocess (zeroed and counted into by every call), one
// set per (device, stream) so that calls in flight on different streams do not
// share them.  Never freed: they live as long as the process.
Tensor counters(const at::Device& dev) {
  static std::mutex mu;
  static auto* sets = new std::map<std::pair<int, cudaStream_t>, Tensor>();
  std::lock_guard<std::mutex> lk(mu);
  const auto key = std::make_pair(static_cast<int>(dev.index()), stream_of(dev));
  auto it = sets->find(key);
  if (it == sets->end())
    it = sets->emplace(key, at::zeros({FGS_COUNTER_WORDS}, at::TensorOptions().dtype(at::kInt).device(dev))).first;
  return it->second;
}

// FB pybind.cpp:26-76.  Returns radii (P,) int32; appends (tile|depth, id) pairs at curr_offset.
Tensor preprocess(int deg, const Tensor& orig_points, const Tensor& color_precomp, const Tensor& dc,
                  const Tensor& shs, const Tensor& opacities, const Tensor& scales, const Tensor& rotations,
                  float scale_modifier, int width, int height, int block_x, int block_y, const Tensor& campos,
                  const Tensor& view_matrix, const Tensor& proj_matrix, float tan_fovx, float tan_fovy, float zFar,
                  float zNear, Tensor& keys_unsorted, Tensor& values_unsorted, Tensor& values_sorted,
                  Tensor& curr_offset, float mult, Tensor& splat_buffer, const Tensor& culling) {
  const at::Device dev = cuda_device_of(opacities);
  c10::cuda::CUDAGuard guard(dev);
  const int64_t P = opacities.size(0);
  const int M = (nonempty(shs) && shs.dim() >= 2 && shs.size(0) != 0) ? static_cast<int>(shs.size(1)) : 0;
  const Tensor means = f32("means3D", orig_points, dev), colors = f32("colors_precomp", color_precomp, dev);
  const Tensor dcc = f32("dc", dc, dev), shc = f32("shs", shs, dev), op = f32("opacities", opacities, dev);
  const Tensor sc = f32("scales", scales, dev), ro = f32("rotations", rotations, dev);
  if (!sc.defined() || !ro.defined())
    throw std::invalid_argument("precomputed 3D covariances are not supported: FB ignores cov3D_precomp and "
                                "needs scales and rotations (FB __init__.py:107-115)");
  const Tensor cam = f32("campos", campos, dev), vm = f32("viewmatrix", view_matrix, dev);
  const Tensor pm = f32("projmatrix", proj_matrix, dev);
  Tensor cull;
  if (nonempty(culling)) {
    if (culling.scalar_type() != at::kBool) throw std::invalid_argument("culling must be a bool tensor");
    cull = culling.to(dev).contiguous();
  }
  need("gaussian_keys_unsorted", keys_unsorted, at::kLong, dev);
  need("gaussian_values_unsorted", values_unsorted, at::kInt, dev);
  need("gaussian_values_sorted", values_sorted, at::kInt, dev);
  need("curr_offset", curr_offset, at::kInt, dev);
  need("splat_buffer", splat_buffer, at::kFloat, dev);
  Tensor radii = at::empty({P}, at::TensorOptions().dtype(at::kInt).device(dev));
  const int64_t cap = std::min(keys_unsorted.numel(), values_unsorted.numel());
  check(fgs_preprocess(static_cast<int>(P), deg, M, static_cast<const float*>(ptr(means)),
                       static_cast<const float*>(ptr(colors)), static_cast<const float*>(ptr(dcc)),
                       static_cast<const float*>(ptr(shc)), static_cast<const float*>(ptr(op)),
                       static_cast<const float*>(ptr(sc)), static_cast<const float*>(ptr(ro)), scale_modifier, width,
                       height, block_x, block_y, static_cast<const float*>(ptr(cam)),
                       static_cast<const float*>(ptr(vm)), static_cast<const float*>(ptr(pm)), tan_fovx, tan_fovy,
                       zFar, zNear, mult, static_cast<const uint8_t*>(ptr(cull)),
                       static_cast<float*>(ptr(splat_buffer)), splat_buffer.size(0),
                       static_cast<uint64_t*>(ptr(keys_unsorted)), static_cast<uint32_t*>(ptr(values_unsorted)), cap,
                       static_cast<uint32_t*>(ptr(values_sorted)), values_sorted.numel(),
                       static_cast<int32_t*>(ptr(curr_offset)), static_cast<int32_t*>(counters(dev).data_ptr()),
                       static_cast<int32_t*>(ptr(radii)), stream_of(dev)),
        "fgs_preprocess");
  return radii;
}

// The frame's pair count and large-footprint task count, stored by a kernel into
// two int32 of pinned host memory (host_counts); the caller synchronises the stream.
void read_counts(const Tensor& curr_offset, Tensor& host_counts) {
  const at::Device dev = cuda_device_of(curr_offset);
  if (host_counts.is_cuda() || host_counts.scalar_type() != at::kInt || host_counts.numel() < 2)
    throw std::invalid_argument("host_counts must be two int32 of (pinned) host memory");
  check(fgs_read_counts(static_cast<const int32_t*>(curr_offset.data_ptr()),
                        static_cast<const int32_t*>(counters(dev).data_ptr()),
                        static_cast<int32_t*>(host_counts.data_ptr()), stream_of(dev)),
        "fgs_read_counts");
}

void sort_gaussian(int64_t num_rendered, int width, int height, int block_x, int block_y, Tensor& sorting_space,
                   const Tensor& keys_unsorted, const Tensor& values_unsorted, Tensor& keys_sorted,
                   Tensor& values_sorted);

// The drop-in forward's host read and sort in one call: the pair and task
// counts stored into pinned memory, one stream synchronisation, and -- when
// the pairs fit max_pairs and the tasks fit task_words / 2 -- the sort
// launched at once, so no Python runs between the synchronisation and the
// first sort kernel.  Returns (pairs, tasks); the caller raises on overflow.
std::tuple<int64_t, int64_t> count_and_sort(const Tensor& curr_offset, Tensor& host_counts, int64_t max_pairs,
                                            int64_t task_words, int width, int height, int block_x, int block_y,
                                            Tensor& sorting_space, const Tensor& keys_unsorted,
                                            const Tensor& values_unsorted, Tensor& keys_sorted,
                                            Tensor& values_sorted) {
  read_counts(curr_offset, host_counts);
  const at::Device dev = cuda_device_of(curr_offset);
  if (cudaStreamSynchronize(stream_of(dev)) != cudaSuccess) throw std::runtime_error("count_and_sort: sync failed");
  const int32_t* hc = static_cast<const int32_t*>(host_counts.data_ptr());
  const int64_t pairs = hc[0], tasks = hc[1];
  if (pairs < max_pairs && tasks <= task_words / 2)
    sort_gaussian(pairs, width, height, block_x, block_y, sorting_space, keys_unsorted, values_unsorted, keys_sorted,
                  values_sorted);
  return {pairs, tasks};
}

// FB pybind.cpp:78-93: stable sort of the first num_rendered pairs.
void sort_gaussian(int64_t num_rendered, int width, int height, int block_x, int block_y, Tensor& sorting_space,
                   const Tensor& keys_unsorted, const Tensor& values_unsorted, Tensor& keys_sorted,
                   Tensor& values_sorted) {
  const at::Device dev = cuda_device_of(keys_unsorted);
  check(fgs_sort(num_rendered, width, height, block_x, block_y, ptr(sorting_space),
                 static_cast<size_t>(sorting_space.numel() * sorting_space.element_size()),
                 static_cast<const uint64_t*>(ptr(keys_unsorted)), static_cast<const uint32_t*>(ptr(values_unsorted)),
                 static_cast<uint64_t*>(ptr(keys_sorted)), static_cast<uint32_t*>(ptr(values_sorted)),
                 stream_of(dev)),
        "fgs_sort");
}

// FB pybind.cpp:95-98.
size_t get_sort_buffer_size(int64_t num_rendered) { return fgs_sort_temp_bytes(num_rendered); }

// Bucket capacity, image-state bytes and sample-state bytes of a frame.
std::tuple<int64_t, size_t, size_t> state_sizes(int64_t num_rendered, int width, int height, int bucket_size) {
  const int64_t mb = fgs_max_buckets(num_rendered, width, height, kTile, kTile, bucket_size);
  size_t ib = 0, sb = 0;
  check(fgs_state_bytes(width, height, kTile, kTile, mb, &ib, &sb), "fgs_state_bytes");
  return {mb, ib, sb};
}

// FB pybind.cpp:100-133: (bucket_sum, out_color (3,H,W), img_buffer, smp_buffer).  With
// read_bucket_sum=false the host read of the bucket count (and its synchronisation) is
// skipped and the reserved bucket capacity is returned in its place.
std::tuple<int64_t, Tensor, Tensor, Tensor> render_16x16(int P, int64_t num_rendered, int width, int height,
                                                         const Tensor& splat_buffer, const Tensor& keys_sorted,
                                                         const Tensor& values_sorted, Tensor& ranges,
                                                         const Tensor& bg_color, Tensor& last_contributor,
                                                         Tensor& Ts_final, int bucket_size, bool read_bucket_sum) {
  const at::Device dev = cuda_device_of(splat_buffer);
  c10::cuda::CUDAGuard guard(dev);
  const Tensor bg = f32("bg", bg_color, dev);
  if (!bg.defined() || bg.numel() != 3) throw std::invalid_argument("bg must hold 3 values");
  if (last_contributor.scalar_type() != at::kInt || Ts_final.scalar_type() != at::kFloat)
    throw std::invalid_argument("last_contributor must be int32 and Ts_final float32");
  auto [mb, ib, sb] = state_sizes(num_rendered, width, height, bucket_size);
  mb = std::max<int64_t>(mb, 1);
  const int64_t rows = mb + 1;
  if (rows * kSampleRow < static_cast<int64_t>(sb))
    throw std::runtime_error("sample-state row sizing is inconsistent with the library");
  const auto u8 = at::TensorOptions().dtype(at::kByte).device(dev);
  Tensor out_color = at::empty({3, height, width}, at::TensorOptions().dtype(at::kFloat).device(dev));
  Tensor img_buffer = at::empty({static_cast<int64_t>(ib)}, u8);
  Tensor smp_buffer = at::empty({rows, kSampleRow}, u8);
  uint32_t bsum = 0;
  check(fgs_render_fwd(P, num_rendered, width, height, kTile, kTile, bucket_size,
                       static_cast<const float*>(ptr(splat_buffer)), static_cast<const uint64_t*>(ptr(keys_sorted)),
                       static_cast<const uint32_t*>(ptr(values_sorted)), static_cast<uint32_t*>(ptr(ranges)),
                       static_cast<const float*>(ptr(bg)), static_cast<float*>(ptr(out_color)),
                       static_cast<int32_t*>(ptr(last_contributor)), static_cast<float*>(ptr(Ts_final)),
                       ptr(img_buffer), ib, ptr(smp_buffer), static_cast<size_t>(rows * kSampleRow), mb,
                       read_bucket_sum ? &bsum : nullptr, stream_of(dev)),
        "fgs_render_fwd");
  return {read_bucket_sum ? static_cast<int64_t>(bsum) : mb, out_color, img_buffer, smp_buffer};
}

using Grads = std::tuple<Tensor, Tensor, Tensor, Tensor, Tensor, Tensor, Tensor, Tensor, Tensor>;

// FB pybind.cpp:210-339: (dL_dmean2D (P,4), dL_dcolor (P,3), dL_dopacity (P,1), dL_dmean3D (P,3),
// dL_dcov3D (P,6), dL_ddc (P,1,3), dL_dsh (P,M,3), dL_dscale (P,3), dL_drot (P,4)).
// abs_grad=false leaves the |dL/dmean2D| sums (dL_dmean2D[:, 2:]) at zero and skips their work;
// minimal=true (an autograd step) returns empty dL_dmean2D and dL_dcov3D, and an empty dL_dcolor
// when SH coefficients are given, without computing them.
Grads backward(int degree, int64_t bucket_sum, const Tensor& means3D, const Tensor& radii, const Tensor& dc,
               const Tensor& sh, const Tensor& opacities, const Tensor& scales, const Tensor& rotations,
               float scale_modifier, int width, int height, int block_x, int block_y, float tan_fovx, float tan_fovy,
               float zFar, float zNear, const Tensor& campos, const Tensor& viewmatrix, const Tensor& projmatrix,
               const Tensor& img_buffer, const Tensor& smp_buffer, const Tensor& splat_buffer,
               const Tensor& point_list, const Tensor& ranges, const Tensor& background,
               const Tensor& last_contributor, const Tensor& Ts_final, const Tensor& dL_dout_color,
               Tensor& xyz_gradient_accum, Tensor& xyz_gradient_accum_abs, Tensor& max_radii, Tensor& denom,
               int bucket_size, bool abs_grad, bool minimal) {
  (void)bucket_sum;
  (void)zFar;
  (void)zNear;
  const at::Device dev = cuda_device_of(means3D);
  c10::cuda::CUDAGuard guard(dev);
  const int64_t P = means3D.size(0);
  const int M = (nonempty(sh) && sh.dim() >= 2 && sh.size(0) != 0) ? static_cast<int>(sh.size(1)) : 0;
  const auto f = at::TensorOptions().dtype(at::kFloat).device(dev);
  const Tensor none = at::empty({0}, f);
  Tensor dmean2D = minimal ? none : at::empty({P, 4}, f);
  Tensor dcolor = (minimal && nonempty(sh)) ? none : at::empty({P, 3}, f);
  Tensor dopac = at::empty({P, 1}, f), dmean3D = at::empty({P, 3}, f);
  Tensor dcov3D = minimal ? none : at::empty({P, 6}, f);
  Tensor ddc = at::empty({P, 1, 3}, f), dsh = at::empty({P, M, 3}, f);
  Tensor dscale = at::empty({P, 3}, f), drot = at::empty({P, 4}, f);
  if (P == 0) return {dmean2D, dcolor, dopac, dmean3D, dcov3D, ddc, dsh, dscale, drot};
  Tensor dconic = minimal ? none : at::empty({P, 2, 2}, f);
  Tensor grad_record = at::empty({P, FGS_GRAD_STRIDE}, f);
  const Tensor means = f32("means3D", means3D, dev), dcc = f32("dc", dc, dev), shc = f32("sh", sh, dev);
  const Tensor sc = f32("scales", scales, dev), ro = f32("rotations", rotations, dev);
  const Tensor dL = f32("dL_dout_color", dL_dout_color, dev), bg = f32("background", background, dev);
  const Tensor cam = f32("campos", campos, dev), vm = f32("viewmatrix", viewmatrix, dev);
  const Tensor pm = f32("projmatrix", projmatrix, dev);
  if (!dL.defined() || dL.numel() != 3LL * width * height)
    throw std::invalid_argument("dL_dout_color must be (3, H, W)");
  const int64_t mb = smp_buffer.size(0) - 1;
  const cudaStream_t s = stream_of(dev);
  check(fgs_render_bwd(static_cast<int>(P), width, height, block_x, block_y, bucket_size,
                       static_cast<const uint32_t*>(ptr(point_list)), static_cast<const uint32_t*>(ptr(ranges)),
                       static_cast<const float*>(ptr(bg)), static_cast<const float*>(ptr(splat_buffer)),
                       static_cast<const float*>(ptr(Ts_final)), static_cast<const int32_t*>(ptr(last_contributor)),
                       ptr(img_buffer), ptr(smp_buffer), mb, static_cast<const float*>(ptr(dL)),
                       static_cast<float*>(ptr(grad_record)), abs_grad ? 0 : FGS_BWD_NO_ABS, s),
        "fgs_render_bwd");
  const bool stats = nonempty(xyz_gradient_accum) && xyz_gradient_accum.size(0) != 0;
  check(fgs_preprocess_bwd(
            static_cast<int>(P), degree, M, static_cast<const float*>(ptr(means)),
            static_cast<const int32_t*>(ptr(radii)), static_cast<const float*>(ptr(dcc)),
            static_cast<const float*>(ptr(shc)), static_cast<const float*>(ptr(splat_buffer)),
            static_cast<const float*>(ptr(sc)), static_cast<const float*>(ptr(ro)), scale_modifier,
            static_cast<const float*>(ptr(vm)), static_cast<const float*>(ptr(pm)), width, height, tan_fovx,
            tan_fovy, static_cast<const float*>(ptr(cam)), static_cast<const float*>(ptr(grad_record)),
            static_cast<float*>(ptr(dmean2D)), static_cast<float*>(ptr(dconic)), static_cast<float*>(ptr(dopac)),
            static_cast<float*>(ptr(dcolor)), static_cast<float*>(ptr(dmean3D)), static_cast<float*>(ptr(dcov3D)),
            static_cast<float*>(ptr(ddc)), static_cast<float*>(ptr(dsh)), static_cast<float*>(ptr(dscale)),
            static_cast<float*>(ptr(drot)), stats ? static_cast<float*>(ptr(xyz_gradient_accum)) : nullptr,
            stats ? static_cast<float*>(ptr(xyz_gradient_accum_abs)) : nullptr,
            stats ? static_cast<float*>(ptr(max_radii)) : nullptr, stats ? static_cast<float*>(ptr(denom)) : nullptr,
            s),
        "fgs_preprocess_bwd");
  return {dmean2D, dcolor, dopac, dmean3D, dcov3D, ddc, dsh, dscale, drot};
}

// FB pybind.cpp:341-366: masked Adam over N rows of M floats.
void adamUpdate(Tensor& param, const Tensor& param_grad, Tensor& exp_avg, Tensor& exp_avg_sq, const Tensor& visible,
                float lr, float b1, float b2, float eps, uint32_t N, uint32_t M) {
  const at::Device dev = cuda_device_of(param);
  for (const auto& [name, t] : {std::pair<const char*, const Tensor*>{"param", &param}, {"param_grad", &param_grad},
                                {"exp_avg", &exp_avg}, {"exp_avg_sq", &exp_avg_sq}})
    need(name, *t, at::kFloat, dev);
  const Tensor vis = visible.contiguous();
  if (vis.scalar_type() != at::kBool) throw std::invalid_argument("visible must be a bool tensor");
  check(fgs_adam_update(static_cast<float*>(ptr(param)), static_cast<const float*>(ptr(param_grad)),
                        static_cast<float*>(ptr(exp_avg)), static_cast<float*>(ptr(exp_avg_sq)),
                        static_cast<const uint8_t*>(ptr(vis)), lr, b1, b2, eps, N, M, stream_of(dev)),
        "fgs_adam_update");
}

// FB pybind.cpp:179-208 (importance pass): (0, accum_weights (P,), accum_count (P,) int32, accum_max_count (P,)).
std::tuple<int64_t, Tensor, Tensor, Tensor> render_simp(int P, int64_t num_rendered, int width, int height,
                                                        const Tensor& splat_buffer, const Tensor& keys_sorted,
                                                        const Tensor& values_sorted, Tensor& ranges) {
  const at::Device dev = cuda_device_of(splat_buffer);
  c10::cuda::CUDAGuard guard(dev);
  Tensor w = at::empty({P}, at::TensorOptions().dtype(at::kFloat).device(dev));
  Tensor cnt = at::empty({P}, at::TensorOptions().dtype(at::kInt).device(dev));
  Tensor mx = at::empty({P}, at::TensorOptions().dtype(at::kFloat).device(dev));
  check(fgs_render_simp(P, num_rendered, width, height, static_cast<const float*>(ptr(splat_buffer)),
                        static_cast<const uint64_t*>(ptr(keys_sorted)), static_cast<const uint32_t*>(ptr(values_sorted)),
                        static_cast<uint32_t*>(ptr(ranges)), static_cast<float*>(ptr(w)),
                        static_cast<int32_t*>(ptr(cnt)), static_cast<float*>(ptr(mx)), stream_of(dev)),
        "fgs_render_simp");
  return {0, w, cnt, mx};
}

// FB pybind.cpp:135-176 (depth pass): out_pts (3,H,W), out_depth, accum_alpha, gidx (int32), discriminants (1,H,W).
std::tuple<Tensor, Tensor, Tensor, Tensor, Tensor> render_depth(
    int P, int64_t num_rendered, int width, int height, const Tensor& splat_buffer, const Tensor& keys_sorted,
    const Tensor& values_sorted, Tensor& ranges, const Tensor& means3D, const Tensor& scales,
    const Tensor& rotations, const Tensor& proj_matrix, const Tensor& campos) {
  const at::Device dev = cuda_device_of(splat_buffer);
  c10::cuda::CUDAGuard guard(dev);
  const auto f = at::TensorOptions().dtype(at::kFloat).device(dev);
  Tensor pts = at::empty({3, height, width}, f), depth = at::empty({1, height, width}, f);
  Tensor alpha = at::empty({1, height, width}, f), disc = at::empty({1, height, width}, f);
  Tensor gidx = at::empty({1, height, width}, at::TensorOptions().dtype(at::kInt).device(dev));
  const Tensor m = f32("means3D", means3D, dev), sc = f32("scales", scales, dev);
  const Tensor ro = f32("rotations", rotations, dev), pm = f32("proj_matrix", proj_matrix, dev);
  const Tensor cam = f32("campos", campos, dev);
  check(fgs_render_depth(P, num_rendered, width, height, static_cast<const float*>(ptr(splat_buffer)),
                         static_cast<const uint64_t*>(ptr(keys_sorted)),
                         static_cast<const uint32_t*>(ptr(values_sorted)), static_cast<uint32_t*>(ptr(ranges)),
                         static_cast<const float*>(ptr(m)), static_cast<const float*>(ptr(sc)),
                         static_cast<const float*>(ptr(ro)), static_cast<const float*>(ptr(pm)),
                         static_cast<const float*>(ptr(cam)), static_cast<float*>(ptr(pts)),
                         static_cast<float*>(ptr(depth)), static_cast<float*>(ptr(alpha)),
                         static_cast<int32_t*>(ptr(gidx)), static_cast<float*>(ptr(disc)), stream_of(dev)),
        "fgs_render_depth");
  return {pts, depth, alpha, gidx, disc};
}

}  // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
  namespace py = pybind11;
  m.doc() = "GB300 (sm_103a) Gaussian rasterizer: the reference backend's _C over the libfgs C ABI";
  auto ops = m.def_submodule("ops", "the reference backend's operators");
  ops.def("preprocess", &preprocess, "per-Gaussian preprocess and (tile|depth, id) key emission");
  ops.def("sort_gaussian", &sort_gaussian, "stable radix sort of the key/value pairs");
  ops.def("get_sort_buffer_size", &get_sort_buffer_size, "scratch bytes of sort_gaussian");
  ops.def("render_16x16", &render_16x16, "tile ranges, bucketed compositing and merge", py::arg("P"),
          py::arg("num_rendered"), py::arg("width"), py::arg("height"), py::arg("splat_buffer"),
          py::arg("gaussian_keys_sorted"), py::arg("gaussian_values_sorted"), py::arg("ranges"), py::arg("bg_color"),
          py::arg("last_contributor"), py::arg("Ts_final"), py::arg("bucket_size") = kBucket,
          py::arg("read_bucket_sum") = true);
  ops.def("render_simp", &render_simp, "importance pass");
  ops.def("render_depth", &render_depth, "depth pass");
  ops.def("backward", &backward, "composite backward and preprocess backward", py::arg("degree"),
          py::arg("bucket_sum"), py::arg("means3D"), py::arg("radii"), py::arg("dc"), py::arg("sh"),
          py::arg("opacities"), py::arg("scales"), py::arg("rotations"), py::arg("scale_modifier"), py::arg("width"),
          py::arg("height"), py::arg("block_x"), py::arg("block_y"), py::arg("tan_fovx"), py::arg("tan_fovy"),
          py::arg("zFar"), py::arg("zNear"), py::arg("campos"), py::arg("viewmatrix"), py::arg("projmatrix"),
          py::arg("img_buffer"), py::arg("smp_buffer"), py::arg("splat_buffer"), py::arg("point_list"),
          py::arg("ranges"), py::arg("background"), py::arg("last_contributor"), py::arg("Ts_final"),
          py::arg("dL_dout_color"), py::arg("xyz_gradient_accum"), py::arg("xyz_gradient_accum_abs"),
          py::arg("max_radii"), py::arg("denom"), py::arg("bucket_size") = kBucket, py::arg("abs_grad") = true,
          py::arg("minimal") = false);
  ops.def("adamUpdate", &adamUpdate, "masked Adam step");
  m.def("read_counts", &read_counts, "pair and task counts of the last preprocess into pinned host memory");
  m.def("count_and_sort", &count_and_sort, "read_counts, one synchronisation and the sort when the pairs fit");
  m.def("version", [] { return std::string(fgs_version()); });
}
