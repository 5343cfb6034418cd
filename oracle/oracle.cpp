// FP64 CPU oracle of the FasterGS differentiable Gaussian rasterizer.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in double precision, the
// math of the reference backend gs_submodules/diff-gaussian-rasterization_faster
// (called FB below) so that the CUDA product can be checked against it.  It is
// linked only by tests/, by __graft_entry__.smoke() and by the CPU-baseline leg
// of bench.py; the product never calls it.
//
// Parity status: pinned.  The reference ships no tests, golden vectors or CPU
// code for this path.  The pieces of the reference that are plain Python (SH
// evaluation, scale/rotation covariance, camera matrices) are pinned by
// fixtures under tests/golden/ made from that Python code; the rasterizer core
// (tile test, key emission, sort order, tile ranges, compositing and merge,
// backward, densification statistics) is pinned by tests/golden/fb_*.npz, the
// outputs of the reference CUDA backend itself, built for sm_103a from its own
// sources (oracle/fb_ref.py) and run on a GB300 on three seeded scenes
// (tests/golden/make_fb_golden.py, tests/test_fb_golden_cpu.py).
//
// Reference map (paths relative to the FasterGS repository):
//   FB/csrc/cuda_rasterizer/preprocess.cu:79-117   2D covariance (EWA)
//   FB/csrc/cuda_rasterizer/preprocess.cu:119-166  SH -> RGB, clamp flags
//   FB/csrc/cuda_rasterizer/preprocess.cu:168-218  tile / ellipse test
//   FB/csrc/cuda_rasterizer/preprocess.cu:364-400  3D covariance (raw quaternion)
//   FB/csrc/cuda_rasterizer/preprocess.cu:414-746  per-Gaussian preprocess + key emission
//   FB/csrc/cuda_rasterizer/rasterizer_imp.h:24-41,532-541  record layout, getRect
//   FB/csrc/cuda_rasterizer/sort.cu:28-44          stable sort on (tile | depth)
//   FB/csrc/cuda_rasterizer/render.cu:13-79        tile ranges, buckets
//   FB/csrc/cuda_rasterizer/render.cu:99-275       bucket compositing
//   FB/csrc/cuda_rasterizer/render.cu:285-391      associative bucket merge
//   FB/csrc/cuda_rasterizer/backward.cu:549-878    per-bucket composite backward
//   FB/csrc/cuda_rasterizer/backward.cu:250-403    conic/cov2D/cov3D/mean backward
//   FB/csrc/cuda_rasterizer/backward.cu:121-245,407-539  SH, scale/rotation, projection backward
//   FB/csrc/cuda_rasterizer/backward.cu:892-918    densification statistics
//   FB/csrc/cuda_rasterizer/render_simp.cu:35-284  importance pass (per-tile, pairwise stop)
//   FB/csrc/cuda_rasterizer/render_depth.cu:97-327 depth pass (per pixel, ray / 3-sigma ellipsoid)
//
// Build: g++ -O2 -fopenmp -shared -fPIC oracle/oracle.cpp -o oracle/liboracle.so
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// Record field offsets, one 32-float record per Gaussian.  Same fields as FB's
// record (rasterizer_imp.h:27-38) in the device library's order; the alpha
// exponent is stored as log2 o + A1 (dx + P dy)^2 + C1 dy^2 and the pixel
// position as floor(float(x)) + fraction, which in exact arithmetic equals
// FB's con_o form (preprocess.cu:709-710) and pixel position.
enum : int {
  F_XY = 0, F_RGB = 2, F_DEPTH = 5, F_CHOL = 6, F_LOG2O = 9, F_FRAC = 10, F_RMIN = 12, F_RMAX = 14,
  F_CONIC = 16, F_POWER = 19, F_CLAMP = 20, F_COV3D = 23, F_PVIEW = 29, REC = 32
};

constexpr double kLn2 = 0.693147180559945309417232121458;
constexpr double kLog2e = 1.442695040888963407359924681001;

// Real spherical-harmonic normalisation constants, bands 0..3.
constexpr double kY0 = 0.28209479177387814;
constexpr double kY1 = 0.4886025119029199;
constexpr double kY2a = 1.0925484305920792, kY2b = 0.31539156525252005, kY2c = 0.5462742152960396;
constexpr double kY3a = 0.5900435899266435, kY3b = 2.890611442640554, kY3c = 0.4570457994644658,
                 kY3d = 0.3731763325901154, kY3e = 1.445305721320277;

// SH basis in the sign convention FB uses (preprocess.cu:132-155): returns
// (deg+1)^2 values B[k] with rgb = sum_k B[k] * coeff[k], coeff[0] = dc.
// dB (optional) receives dB[k][0..2] = d B[k] / d(x, y, z).
void sh_basis(int deg, double x, double y, double z, double* B, double (*dB)[3]) {
  const double xx = x * x, yy = y * y, zz = z * z;
  double b[16] = {0}, d[16][3] = {{0}};
  b[0] = kY0;
  if (deg > 0) {
    b[1] = -kY1 * y;  d[1][1] = -kY1;
    b[2] = kY1 * z;   d[2][2] = kY1;
    b[3] = -kY1 * x;  d[3][0] = -kY1;
  }
  if (deg > 1) {
    b[4] = kY2a * x * y;               d[4][0] = kY2a * y;       d[4][1] = kY2a * x;
    b[5] = -kY2a * y * z;              d[5][1] = -kY2a * z;      d[5][2] = -kY2a * y;
    b[6] = kY2b * (2 * zz - xx - yy);  d[6][0] = -2 * kY2b * x;  d[6][1] = -2 * kY2b * y; d[6][2] = 4 * kY2b * z;
    b[7] = -kY2a * x * z;              d[7][0] = -kY2a * z;      d[7][2] = -kY2a * x;
    b[8] = kY2c * (xx - yy);           d[8][0] = 2 * kY2c * x;   d[8][1] = -2 * kY2c * y;
  }
  if (deg > 2) {
    b[9] = -kY3a * y * (3 * xx - yy);
    d[9][0] = -kY3a * 6 * x * y;  d[9][1] = -kY3a * (3 * xx - 3 * yy);
    b[10] = kY3b * x * y * z;
    d[10][0] = kY3b * y * z;  d[10][1] = kY3b * x * z;  d[10][2] = kY3b * x * y;
    b[11] = -kY3c * y * (4 * zz - xx - yy);
    d[11][0] = kY3c * 2 * x * y;  d[11][1] = -kY3c * (4 * zz - xx - 3 * yy);  d[11][2] = -kY3c * 8 * y * z;
    b[12] = kY3d * z * (2 * zz - 3 * xx - 3 * yy);
    d[12][0] = -kY3d * 6 * x * z;  d[12][1] = -kY3d * 6 * y * z;  d[12][2] = kY3d * (6 * zz - 3 * xx - 3 * yy);
    b[13] = -kY3c * x * (4 * zz - xx - yy);
    d[13][0] = -kY3c * (4 * zz - 3 * xx - yy);  d[13][1] = kY3c * 2 * x * y;  d[13][2] = -kY3c * 8 * x * z;
    b[14] = kY3e * z * (xx - yy);
    d[14][0] = kY3e * 2 * x * z;  d[14][1] = -kY3e * 2 * y * z;  d[14][2] = kY3e * (xx - yy);
    b[15] = -kY3a * x * (xx - 3 * yy);
    d[15][0] = -kY3a * (3 * xx - 3 * yy);  d[15][1] = kY3a * 6 * x * y;
  }
  const int n = (deg + 1) * (deg + 1);
  for (int k = 0; k < n; ++k) {
    B[k] = b[k];
    if (dB) { dB[k][0] = d[k][0]; dB[k][1] = d[k][1]; dB[k][2] = d[k][2]; }
  }
}

// Rotation matrix of a raw (not normalised) quaternion q = (r, x, y, z), as
// FB builds it (preprocess.cu:375-386, glm column fill), written row-major in
// the usual mathematical orientation.  dR (optional): dR[k][a][b] = dR_ab/dq_k.
void quat_rot(const double* q, double R[3][3], double dR[4][3][3]) {
  const double r = q[0], x = q[1], y = q[2], z = q[3];
  R[0][0] = 1 - 2 * (y * y + z * z); R[0][1] = 2 * (x * y - r * z);     R[0][2] = 2 * (x * z + r * y);
  R[1][0] = 2 * (x * y + r * z);     R[1][1] = 1 - 2 * (x * x + z * z); R[1][2] = 2 * (y * z - r * x);
  R[2][0] = 2 * (x * z - r * y);     R[2][1] = 2 * (y * z + r * x);     R[2][2] = 1 - 2 * (x * x + y * y);
  if (!dR) return;
  const double v[4][3][3] = {
      {{0, -2 * z, 2 * y}, {2 * z, 0, -2 * x}, {-2 * y, 2 * x, 0}},                       // d/dr
      {{0, 2 * y, 2 * z}, {2 * y, -4 * x, -2 * r}, {2 * z, 2 * r, -4 * x}},               // d/dx
      {{-4 * y, 2 * x, 2 * r}, {2 * x, 0, 2 * z}, {-2 * r, 2 * z, -4 * y}},               // d/dy
      {{-4 * z, -2 * r, 2 * x}, {2 * r, -4 * z, 2 * y}, {2 * x, 2 * y, 0}}};              // d/dz
  std::memcpy(dR, v, sizeof(v));
}

struct Cam {
  int W = 0, H = 0, bx = 16, by = 16, gx = 0, gy = 0;
  double view[16], proj[16], campos[3];
  double tanx = 0, tany = 0, fx = 0, fy = 0, mult = 1, smod = 1;
  // 4x3 / 4x4 transforms of a column-major 3DGS matrix (rasterizer_imp.h:502-520).
  void view_pt(const double* p, double* t) const {
    for (int r = 0; r < 3; ++r) t[r] = view[r] * p[0] + view[4 + r] * p[1] + view[8 + r] * p[2] + view[12 + r];
  }
  void proj_pt(const double* p, double* h) const {
    for (int r = 0; r < 4; ++r) h[r] = proj[r] * p[0] + proj[4 + r] * p[1] + proj[8 + r] * p[2] + proj[12 + r];
  }
  double Rw(int a, int b) const { return view[b * 4 + a]; }  // rotation part of world->view
};

struct Scene {
  int P = 0, D = 0, M = 0;
  bool has_colors = false, has_shs = false, has_scales = true;
  std::vector<double> means, colors, dc, shs, opac, scales, rots;
  std::vector<uint8_t> culling;
  Cam cam;
  // preprocess
  std::vector<double> rec;
  std::vector<int> radii, rect_area;
  std::vector<uint8_t> valid, gauss_amb;
  // sorted lists
  std::vector<uint64_t> keys;
  std::vector<int> ids;
  std::vector<uint8_t> pair_amb;
  std::vector<int> ranges;
  // pairs the FP64 test rejects but an FP32 evaluation may accept (kept out of
  // the lists; tests count them as flagged)
  std::vector<uint64_t> cand_keys;
  std::vector<int> cand_ids;
  // composite
  int bucket_size = 128;
  std::vector<int> tile_boff;     // T+1 bucket offsets
  std::vector<double> accT, accC; // per (bucket, pixel-in-tile): T, C rgb
  std::vector<double> out_color, pix_color, Ts_final;
  std::vector<int> last_contrib, max_contrib;
  std::vector<uint8_t> pix_amb;
  std::vector<uint8_t> gauss_clamped;   // some evaluated alpha hit the 0.99 clamp
  int64_t n_alpha_on = 0, n_clamped = 0; // decision signature of the last composite
  double bg[3] = {0, 0, 0};
  double eps_alpha = 1e-5, eps_T = 1e-5;
  int T() const { return cam.gx * cam.gy; }
};

float as_float(double v) { return (float)v; }
uint32_t float_bits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

// Per-Gaussian preprocess (preprocess.cu:450-499, 698-721).
void preprocess_one(Scene& s, int i) {
  double* r = &s.rec[(size_t)i * REC];
  std::fill(r, r + REC, 0.0);
  s.radii[i] = 0; s.valid[i] = 0; s.rect_area[i] = 0; s.gauss_amb[i] = 0;
  if (!s.culling.empty() && s.culling[i]) return;
  const Cam& c = s.cam;
  const double* p = &s.means[3 * (size_t)i];
  double t[3];
  c.view_pt(p, t);
  if (t[2] <= 0.2) return;                       // near cull
  const double o = s.opac[i];
  if (255.0 * o < 1.0) return;                   // opacity cull
  double h[4];
  c.proj_pt(p, h);
  const double pw = 1.0 / (h[3] + 1e-7);
  const double ndc[2] = {h[0] * pw, h[1] * pw};

  // 3D covariance from the raw quaternion and the modified scale.
  double R[3][3];
  quat_rot(&s.rots[4 * (size_t)i], R, nullptr);
  double s2[3];
  for (int k = 0; k < 3; ++k) { const double sk = c.smod * s.scales[3 * (size_t)i + k]; s2[k] = sk * sk; }
  double Sig[3][3];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      double v = 0;
      for (int k = 0; k < 3; ++k) v += R[a][k] * s2[k] * R[b][k];
      Sig[a][b] = v;
    }
  r[F_COV3D + 0] = Sig[0][0]; r[F_COV3D + 1] = Sig[0][1]; r[F_COV3D + 2] = Sig[0][2];
  r[F_COV3D + 3] = Sig[1][1]; r[F_COV3D + 4] = Sig[1][2]; r[F_COV3D + 5] = Sig[2][2];

  // EWA screen covariance with the FOV clamp and the 0.3 px^2 low-pass.
  const double limx = 1.3 * c.tanx, limy = 1.3 * c.tany;
  const double tz = t[2];
  const double tx = std::min(limx, std::max(-limx, t[0] / tz)) * tz;
  const double ty = std::min(limy, std::max(-limy, t[1] / tz)) * tz;
  const double J[2][3] = {{c.fx / tz, 0, -c.fx * tx / (tz * tz)}, {0, c.fy / tz, -c.fy * ty / (tz * tz)}};
  double Mm[2][3];
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 3; ++b) {
      double v = 0;
      for (int k = 0; k < 3; ++k) v += J[a][k] * c.Rw(k, b);
      Mm[a][b] = v;
    }
  double cv[2][2];
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      double v = 0;
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) v += Mm[a][k] * Sig[k][l] * Mm[b][l];
      cv[a][b] = v;
    }
  const double ca = cv[0][0] + 0.3, cb = cv[0][1], cc = cv[1][1] + 0.3;
  const double det = ca * cc - cb * cb;
  const double conic[3] = {cc / det, -cb / det, ca / det};

  // Screen radius reported to the caller (preprocess.cu:480-485).
  const double mid = 0.5 * (ca + cc);
  const double extent = std::min(3.33, std::sqrt(2.0 * std::log(o * 255.0)));
  const double lambda = mid + std::sqrt(std::max(0.01, mid * mid - det));
  const double radius = std::ceil(extent * std::sqrt(lambda));

  // Tile rectangle from the 1/256 level set (preprocess.cu:488-497, rasterizer_imp.h:532-541).
  const double log2o = std::log2(o);
  const double power = (kLn2 * 8.0 + kLn2 * log2o) * c.mult;
  const double wf = 1.414214 * std::sqrt(ca * power) + 1.0;
  const double hf = 1.414214 * std::sqrt(cc * power) + 1.0;
  const int wpx = (int)wf, hpx = (int)hf;
  const double xy[2] = {((ndc[0] + 1.0) * c.W - 1.0) * 0.5, ((ndc[1] + 1.0) * c.H - 1.0) * 0.5};
  auto clampi = [](int v, int hi) { return std::min(hi, std::max(0, v)); };
  const int rminx = clampi((int)((xy[0] - wpx) / c.bx), c.gx);
  const int rminy = clampi((int)((xy[1] - hpx) / c.by), c.gy);
  const int rmaxx = clampi((int)((xy[0] + wpx) / c.bx) + 1, c.gx);
  const int rmaxy = clampi((int)((xy[1] + hpx) / c.by) + 1, c.gy);
  const int area = (rmaxx - rminx) * (rmaxy - rminy);
  // Integer truncations that sit within 1e-4 of a boundary may resolve differently
  // in FP32; such Gaussians are flagged so tests can treat them as ambiguous.
  auto near_int = [](double v) { return std::fabs(v - std::round(v)) < 1e-4; };
  if (near_int(wf) || near_int(hf) || near_int((xy[0] - wpx) / c.bx) || near_int((xy[1] - hpx) / c.by) ||
      near_int((xy[0] + wpx) / c.bx) || near_int((xy[1] + hpx) / c.by) || near_int(extent * std::sqrt(lambda)))
    s.gauss_amb[i] = 1;
  if (area <= 0) return;

  // Colour: precomputed or SH (preprocess.cu:119-166).
  double rgb[3];
  if (s.has_colors) {
    for (int k = 0; k < 3; ++k) rgb[k] = s.colors[3 * (size_t)i + k];
  } else {
    double dir[3] = {p[0] - c.campos[0], p[1] - c.campos[1], p[2] - c.campos[2]};
    const double n = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    for (double& v : dir) v /= n;
    double B[16];
    sh_basis(s.D, dir[0], dir[1], dir[2], B, nullptr);
    const int nb = (s.D + 1) * (s.D + 1);
    for (int ch = 0; ch < 3; ++ch) {
      double v = B[0] * s.dc[3 * (size_t)i + ch];
      for (int k = 1; k < nb; ++k) v += B[k] * s.shs[((size_t)i * s.M + (k - 1)) * 3 + ch];
      v += 0.5;
      r[F_CLAMP + ch] = v < 0 ? 1.0 : 0.0;
      rgb[ch] = std::max(v, 0.0);
    }
  }
  r[F_XY + 0] = xy[0]; r[F_XY + 1] = xy[1];
  r[F_RGB + 0] = rgb[0]; r[F_RGB + 1] = rgb[1]; r[F_RGB + 2] = rgb[2];
  r[F_DEPTH] = t[2];
  r[F_CHOL + 0] = -0.5 * kLog2e * conic[0];
  r[F_CHOL + 1] = -cb / cc;
  r[F_CHOL + 2] = -0.5 * kLog2e / cc;
  r[F_LOG2O] = log2o;
  r[F_FRAC + 0] = xy[0] - std::floor((double)(float)xy[0]);
  r[F_FRAC + 1] = xy[1] - std::floor((double)(float)xy[1]);
  r[F_RMIN + 0] = rminx; r[F_RMIN + 1] = rminy; r[F_RMAX + 0] = rmaxx; r[F_RMAX + 1] = rmaxy;
  r[F_CONIC + 0] = conic[0]; r[F_CONIC + 1] = conic[1]; r[F_CONIC + 2] = conic[2];
  r[F_POWER] = power;
  r[F_PVIEW + 0] = t[0]; r[F_PVIEW + 1] = t[1]; r[F_PVIEW + 2] = t[2];
  s.radii[i] = (int)radius;
  s.valid[i] = 1;
  s.rect_area[i] = area;
}

// Does the level set q(d) = 2*power of the conic cross the pixel rectangle
// [x0,x1]x[y0,y1]?  Centre-inside test plus a chord test against the edge
// nearest to the centre on each axis (preprocess.cu:168-218).
bool chord_hits(double A, double Bc, double C, double d, double l, double r) {
  const double disc = Bc * Bc - 4.0 * A * C;
  if (disc < 0) return false;
  const double t1 = (l - d) * (2.0 * A) + Bc;   // lower end of the segment vs. upper root
  const double t2 = (r - d) * (2.0 * A) + Bc;   // upper end of the segment vs. lower root
  return (t1 <= 0 || t1 * t1 <= disc) && (t2 >= 0 || t2 * t2 <= disc);
}
bool tile_hit(double x0, double x1, double y0, double y1, double cx, double cy, const double* cn, double power) {
  if (cx >= x0 && cx <= x1 && cy >= y0 && cy <= y1) return true;
  const double w = 2.0 * power;
  const double dx = cx - ((cx * 2.0 < x0 + x1) ? x0 : x1);
  if (chord_hits(cn[2], -2.0 * cn[1] * dx, cn[0] * dx * dx - w, cy, y0, y1)) return true;
  const double dy = cy - ((cy * 2.0 < y0 + y1) ? y0 : y1);
  return chord_hits(cn[0], -2.0 * cn[1] * dy, cn[2] * dy * dy - w, cx, x0, x1);
}

// FP32 decidability of the same test.  The device evaluates tile_hit in FP32 on
// the record's f32 values; here each comparison is made in FP64 together with a
// first-order bound on the FP32 evaluation error of its sides (unit roundoff
// 2^-24 per operation, propagated through dx, B, C, the discriminant and the
// segment ends, times a safety factor of 4).  A comparison inside its bound can
// resolve either way on the device, so the result is three-valued and a pair
// whose test stays undecided is ambiguous.  Thin footprints need this: the
// discriminant 4 dx^2 (b^2 - a c) + 4 c w cancels with the footprint's
// anisotropy, and a nudge of the centre or the power does not always bracket
// the FP32 outcome.
enum Tri : uint8_t { kNo = 0, kYes = 1, kMaybe = 2 };
Tri tri_and(Tri a, Tri b) { return (a == kNo || b == kNo) ? kNo : (a == kYes && b == kYes) ? kYes : kMaybe; }
Tri tri_or(Tri a, Tri b) { return (a == kYes || b == kYes) ? kYes : (a == kNo && b == kNo) ? kNo : kMaybe; }
Tri tri_pos(double v, double err) { return v > err ? kYes : (v < -err ? kNo : kMaybe); }
// chord_hits on A u^2 + B u + C with B = -2 b e, C = q e^2 - w, e = centre - edge.
Tri chord_tri(double A, double b, double q, double e, double w, double d, double l, double r) {
  const double u = 1.0 / 16777216.0, K = 4.0;
  const double err_e = u * std::fabs(e);
  const double B = -2.0 * b * e, C = q * e * e - w;
  const double err_B = u * std::fabs(B) + 2.0 * std::fabs(b) * err_e;
  const double err_C = 3.0 * u * (std::fabs(q) * e * e + std::fabs(w)) + 2.0 * std::fabs(q * e) * err_e;
  const double disc = B * B - 4.0 * A * C;
  const double err_disc = 2.0 * u * (B * B + 4.0 * std::fabs(A * C) + std::fabs(disc)) + 2.0 * std::fabs(B) * err_B +
                          4.0 * std::fabs(A) * err_C;
  auto seg = [&](double end, Tri& sign_ok, Tri& inside, bool lower) {
    const double t = (end - d) * (2.0 * A) + B;
    const double err_t = 3.0 * u * (std::fabs((end - d) * 2.0 * A) + std::fabs(B) + std::fabs(t)) + err_B;
    sign_ok = tri_pos(lower ? -t : t, K * err_t);   // t <= 0 (lower end) or t >= 0 (upper end)
    const double g = disc - t * t;                   // t^2 <= disc
    inside = tri_pos(g, K * (err_disc + u * t * t + 2.0 * std::fabs(t) * err_t));
  };
  Tri s1, i1, s2, i2;
  seg(l, s1, i1, true);
  seg(r, s2, i2, false);
  return tri_and(tri_pos(disc, K * err_disc), tri_and(tri_or(s1, i1), tri_or(s2, i2)));
}
Tri tile_hit_fp32(double x0, double x1, double y0, double y1, double cx, double cy, const double* cn, double power) {
  if (cx >= x0 && cx <= x1 && cy >= y0 && cy <= y1) return kYes;
  const double w = 2.0 * power;
  const double dx = cx - ((cx * 2.0 < x0 + x1) ? x0 : x1);
  const Tri first = chord_tri(cn[2], cn[1], cn[0], dx, w, cy, y0, y1);
  if (first == kYes) return kYes;
  const double dy = cy - ((cy * 2.0 < y0 + y1) ? y0 : y1);
  return tri_or(first, chord_tri(cn[0], cn[1], cn[2], dy, w, cx, x0, x1));
}

struct Pair { uint64_t key; double depth; int id; uint8_t amb; };

// Enumerate every (tile, Gaussian) pair FB emits: all tiles of the rectangle
// that pass tile_hit (preprocess.cu:536-696 small path, :749-860 large path),
// then sort by (tile, depth) keeping emission order (id ascending) for ties.
void emit_and_sort(Scene& s, double eps_pair) {
  const Cam& c = s.cam;
  std::vector<std::vector<Pair>> per(s.P);
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < s.P; ++i) {
    if (!s.valid[i]) continue;
    const double* r = &s.rec[(size_t)i * REC];
    const int x0 = (int)r[F_RMIN], y0 = (int)r[F_RMIN + 1], x1 = (int)r[F_RMAX], y1 = (int)r[F_RMAX + 1];
    const double cx = r[F_XY], cy = r[F_XY + 1], power = r[F_POWER];
    const float depth_f = as_float(r[F_DEPTH]);
    for (int ty = y0; ty < y1; ++ty)
      for (int tx = x0; tx < x1; ++tx) {
        const double px0 = tx * c.bx, px1 = px0 + c.bx - 1, py0 = ty * c.by, py1 = py0 + c.by - 1;
        const bool hit = tile_hit(px0, px1, py0, py1, cx, cy, r + F_CONIC, power);
        // Borderline check: grow/shrink the level set and nudge the centre.
        const double nx = std::min(std::max(cx, px0), px1) - cx, ny = std::min(std::max(cy, py0), py1) - cy;
        const double sx = nx > 0 ? 1 : (nx < 0 ? -1 : 0), sy = ny > 0 ? 1 : (ny < 0 ? -1 : 0);
        const double sh = 1e-3 * std::max(1.0, eps_pair / 1e-5);
        const bool hi = tile_hit(px0, px1, py0, py1, cx + sx * sh, cy + sy * sh, r + F_CONIC, power * (1 + eps_pair));
        const bool lo = tile_hit(px0, px1, py0, py1, cx - sx * sh, cy - sy * sh, r + F_CONIC, power * (1 - eps_pair));
        const bool amb = hi != lo || tile_hit_fp32(px0, px1, py0, py1, cx, cy, r + F_CONIC, power) == kMaybe;
        if (hit || amb) {
          Pair p;
          p.key = ((uint64_t)(uint32_t)(ty * c.gx + tx) << 32) | float_bits(depth_f);
          p.depth = r[F_DEPTH];
          p.id = i;
          p.amb = amb ? 1 : 0;
          if (!hit) p.amb |= 2;   // bit 1: pair present only as an ambiguous candidate
          per[i].push_back(p);
        }
      }
  }
  std::vector<Pair> all;
  for (auto& v : per) all.insert(all.end(), v.begin(), v.end());
  std::stable_sort(all.begin(), all.end(), [](const Pair& a, const Pair& b) {
    const uint32_t ta = (uint32_t)(a.key >> 32), tb = (uint32_t)(b.key >> 32);
    if (ta != tb) return ta < tb;
    return a.depth < b.depth;
  });
  s.keys.resize(all.size()); s.ids.resize(all.size()); s.pair_amb.resize(all.size());
  for (size_t k = 0; k < all.size(); ++k) { s.keys[k] = all[k].key; s.ids[k] = all[k].id; s.pair_amb[k] = all[k].amb; }
}

// Tile ranges over a sorted list whose pairs carry "candidate only" flags;
// candidate-only pairs are dropped from the list the compositor sees.
void build_ranges_from_pairs(Scene& s) {
  std::vector<uint64_t> k2; std::vector<int> i2; std::vector<uint8_t> a2;
  s.cand_keys.clear(); s.cand_ids.clear();
  for (size_t k = 0; k < s.keys.size(); ++k) {
    if (!(s.pair_amb[k] & 2)) { k2.push_back(s.keys[k]); i2.push_back(s.ids[k]); a2.push_back(s.pair_amb[k]); }
    else { s.cand_keys.push_back(s.keys[k]); s.cand_ids.push_back(s.ids[k]); }
  }
  s.keys.swap(k2); s.ids.swap(i2); s.pair_amb.swap(a2);
  s.ranges.assign(2 * (size_t)s.T(), 0);
  for (size_t k = 0; k < s.keys.size(); ++k) {
    const int t = (int)(s.keys[k] >> 32);
    if (k == 0 || (int)(s.keys[k - 1] >> 32) != t) s.ranges[2 * t] = (int)k;
    if (k + 1 == s.keys.size() || (int)(s.keys[k + 1] >> 32) != t) s.ranges[2 * t + 1] = (int)k + 1;
  }
}

// Exponent of alpha for pixel (px, py) and its partial derivatives with
// respect to the centre.  dx, dy = centre - pixel.
struct AlphaEval {
  double a, dx, dy, dedx, dedy;
};
inline AlphaEval alpha_of(const double* r, double px, double py) {
  AlphaEval v;
  v.dx = (std::floor((double)(float)r[F_XY]) - px) + r[F_FRAC];
  v.dy = (std::floor((double)(float)r[F_XY + 1]) - py) + r[F_FRAC + 1];
  const double A1 = r[F_CHOL], P = r[F_CHOL + 1], C1 = r[F_CHOL + 2];
  const double w = v.dx + P * v.dy;
  v.a = std::exp2(r[F_LOG2O] + A1 * w * w + C1 * v.dy * v.dy);
  v.dedx = 2 * A1 * w;
  v.dedy = 2 * A1 * P * w + 2 * C1 * v.dy;
  return v;
}

// Bucketed compositing and merge (render.cu:99-123,130-275,285-391).
void composite(Scene& s) {
  const Cam& c = s.cam;
  const int T = s.T(), bs = s.bucket_size, tp = c.bx * c.by;
  s.tile_boff.assign(T + 1, 0);
  for (int t = 0; t < T; ++t) {
    const int n = s.ranges[2 * t + 1] - s.ranges[2 * t];
    s.tile_boff[t + 1] = s.tile_boff[t] + (n + bs - 1) / bs;
  }
  const size_t B = (size_t)s.tile_boff[T];
  s.accT.assign(B * tp, 0.0);
  s.accC.assign(B * tp * 3, 0.0);
  const size_t HW = (size_t)c.W * c.H;
  s.out_color.assign(3 * HW, 0.0); s.pix_color.assign(3 * HW, 0.0); s.Ts_final.assign(HW, 0.0);
  s.last_contrib.assign(HW, 0); s.max_contrib.assign(T, 0); s.pix_amb.assign(HW, 0);
  s.gauss_clamped.assign(s.P, 0);
  const double cut = 1.0 / 255.0;
  int64_t n_on = 0, n_cl = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : n_on, n_cl)
  for (int t = 0; t < T; ++t) {
    const int tx = t % c.gx, ty = t / c.gx, start = s.ranges[2 * t], end = s.ranges[2 * t + 1];
    const int nb = s.tile_boff[t + 1] - s.tile_boff[t];
    int mc = 0;
    for (int lp = 0; lp < tp; ++lp) {
      const int px = tx * c.bx + lp % c.bx, py = ty * c.by + lp / c.bx;
      if (px >= c.W || py >= c.H) continue;
      double Tp = 1, C[3] = {0, 0, 0};
      int contrib = 0;
      bool amb = false;
      for (int b = 0; b < nb; ++b) {
        double Tb = 1, Cb[3] = {0, 0, 0};
        const int g0 = start + b * bs, g1 = std::min(end, g0 + bs);
        for (int g = g0; g < g1; ++g) {
          const double* r = &s.rec[(size_t)s.ids[g] * REC];
          double a = alpha_of(r, px, py).a;
          if (std::fabs(a - cut) <= s.eps_alpha * cut) amb = true;
          if (a > 0.99) { s.gauss_clamped[s.ids[g]] = 1; ++n_cl; }
          a = std::min(0.99, a);
          if (a < cut) a = 0; else ++n_on;
          for (int ch = 0; ch < 3; ++ch) Cb[ch] += r[F_RGB + ch] * a * Tb;
          Tb -= a * Tb;
        }
        for (int ch = 0; ch < 3; ++ch) C[ch] += Tp * Cb[ch];
        Tp *= Tb;
        const size_t sb = (size_t)(s.tile_boff[t] + b) * tp + lp;
        s.accT[sb] = Tp;
        for (int ch = 0; ch < 3; ++ch) s.accC[3 * sb + ch] = C[ch];
        contrib += g1 - g0;
        if (std::fabs(Tp - 1e-4) <= s.eps_T * 1e-4) amb = true;
        if (Tp < 1e-4) break;
      }
      const size_t pix = (size_t)py * c.W + px;
      s.last_contrib[pix] = contrib;
      s.Ts_final[pix] = Tp;
      for (int ch = 0; ch < 3; ++ch) {
        s.out_color[ch * HW + pix] = C[ch] + Tp * s.bg[ch];
        s.pix_color[3 * pix + ch] = C[ch];
      }
      s.pix_amb[pix] = amb ? 1 : 0;
      mc = std::max(mc, contrib);
    }
    s.max_contrib[t] = mc;
  }
  s.n_alpha_on = n_on;
  s.n_clamped = n_cl;
}

// Importance pass (render_simp.cu:35-284): each tile walks its list in
// order; a Gaussian with alpha >= 1/255 at a pixel adds its weight alpha T
// (T -= weight) to the Gaussian's sum and 1 to its count, and the pixel keeps
// the Gaussian of largest weight; after every pair of Gaussians (a lone
// first one when the count is odd) the tile stops if every one of its 256
// pixels has T < 1e-4 (pixels outside the image keep T = 1).  amb flags
// Gaussians whose sums or counts are within rounding distance of a different
// decision (alpha at the cut, a stop test at 1e-4, a near-tie for the
// largest weight).
void render_simp(const Scene& s, double eps_alpha, double eps_T, double eps_w, double* wsum, int* wcnt,
                 double* wmaxcnt, uint8_t* amb) {
  const Cam& c = s.cam;
  const int T = s.T(), tp = 256;
  const double cut = 1.0 / 255.0;
  std::fill(wsum, wsum + s.P, 0.0);
  std::fill(wcnt, wcnt + s.P, 0);
  std::fill(wmaxcnt, wmaxcnt + s.P, 0.0);
  std::fill(amb, amb + s.P, 0);
  for (int t = 0; t < T; ++t) {
    const int tx = t % c.gx, ty = t / c.gx, start = s.ranges[2 * t], end = s.ranges[2 * t + 1], n = end - start;
    std::vector<double> Tp(tp, 1.0), wmax(tp, 0.0), wsecond(tp, 0.0);
    std::vector<int> imax(tp, -1);
    std::vector<uint8_t> inside(tp, 0);
    for (int lp = 0; lp < tp; ++lp) {
      const int px = tx * 16 + lp % 16, py = ty * 16 + lp / 16;
      inside[lp] = px < c.W && py < c.H;
    }
    const int odd = n & 1;
    bool tile_amb = false;
    for (int i = 0; i < n; ++i) {
      const int g = s.ids[start + i];
      const double* r = &s.rec[(size_t)g * REC];
      double sum = 0;
      int cnt = 0;
      for (int lp = 0; lp < tp; ++lp) {
        if (!inside[lp]) continue;
        const int px = tx * 16 + lp % 16, py = ty * 16 + lp / 16;
        double a = std::min(0.99, alpha_of(r, px, py).a);
        if (std::fabs(a - cut) <= eps_alpha * cut) amb[g] = 1;
        if (a < cut) continue;
        const double w = a * Tp[lp];
        Tp[lp] -= w;
        sum += w;
        cnt += 1;
        if (wmax[lp] < w) { wsecond[lp] = wmax[lp]; wmax[lp] = w; imax[lp] = g; }
        else if (wsecond[lp] < w) wsecond[lp] = w;
      }
      if (g < s.P) { wsum[g] += sum; wcnt[g] += cnt; }
      if (tile_amb) amb[g] = 1;
      if (i >= odd && ((i - odd) & 1)) {
        bool done = true, near = false;
        for (int lp = 0; lp < tp; ++lp) {
          done = done && inside[lp] && Tp[lp] < 1e-4;
          if (inside[lp] && std::fabs(Tp[lp] - 1e-4) <= eps_T * 1e-4) near = true;
        }
        if (near) tile_amb = true;
        if (done) break;
      }
    }
    for (int lp = 0; lp < tp; ++lp) {
      if (!inside[lp] || imax[lp] < 0) continue;
      wmaxcnt[imax[lp]] += 1.0;
      if (wmax[lp] - wsecond[lp] <= eps_w * wmax[lp]) amb[imax[lp]] = 1;
    }
    if (tile_amb)
      for (int i = 0; i < n; ++i) amb[s.ids[start + i]] = 1;
  }
}

// 4x4 inverse (column-major, cofactors).
void invert4(const double* a, double* out) {
  double inv[16];
  inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
  inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
  inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
  inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
  inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
  inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
  inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
  inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
  inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
  inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
  inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
  inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
  inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
  inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
  inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
  inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
  const double det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
  for (int i = 0; i < 16; ++i) out[i] = det != 0 ? inv[i] / det : 0.0;
}

// Depth pass (render_depth.cu:97-327).  Per pixel: the ray from the camera
// through the pixel's NDC point (2p+1)/S - 1, scaled by 1.0000001, at
// z = 99/99.99, mapped by the inverse full projection without dividing by w;
// Gaussians in list order: alpha < 1/255 skipped, stop before one that would
// take T below 1e-4, then the closest approach of the ray to the Gaussian's
// 3-sigma ellipsoid (raw quaternion, scales without the modifier); a
// Gaussian behind the camera is skipped without changing T; the one of
// largest weight alpha T gives point, depth, discriminant and index.  amb
// flags pixels within rounding distance of a different decision.
void render_depth(const Scene& s, double eps_alpha, double eps_T, double eps_w, double* out_pts, double* out_depth,
                  double* accum_alpha, int* gidx, double* disc, uint8_t* amb) {
  const Cam& c = s.cam;
  const double cut = 1.0 / 255.0;
  const size_t HW = (size_t)c.W * c.H;
  double inv[16];
  invert4(c.proj, inv);
  const double* o = c.campos;
#pragma omp parallel for schedule(dynamic, 8)
  for (int pix = 0; pix < (int)HW; ++pix) {
    const int px = pix % c.W, py = pix / c.W;
    const int t = (py / 16) * c.gx + px / 16;
    const double nx = ((2.0 * px + 1.0) / c.W - 1.0) * 1.0000001, ny = ((2.0 * py + 1.0) / c.H - 1.0) * 1.0000001;
    const double nz = (100.0 - 100.0 * 0.01) / (100.0 - 0.01);
    double rd[3];
    for (int k = 0; k < 3; ++k) rd[k] = inv[k] * nx + inv[4 + k] * ny + inv[8 + k] * nz + inv[12 + k] - o[k];
    const double rlen = std::sqrt(rd[0] * rd[0] + rd[1] * rd[1] + rd[2] * rd[2]);
    const double dn[3] = {rd[0] / rlen, rd[1] / rlen, rd[2] / rlen};
    double T = 1, wmax = 0, wsecond = 0, dmax = 0, dsc = 0, pr[3] = {0, 0, 0};
    int im = 0;
    bool a_flag = false;
    for (int j = s.ranges[2 * t]; j < s.ranges[2 * t + 1]; ++j) {
      const int g = s.ids[j];
      const double* r = &s.rec[(size_t)g * REC];
      const double a = std::min(0.99, alpha_of(r, px, py).a);
      if (std::fabs(a - cut) <= eps_alpha * cut) a_flag = true;
      if (a < cut) continue;
      const double test_T = T * (1 - a);
      if (std::fabs(test_T - 1e-4) <= eps_T * 1e-4) a_flag = true;
      if (test_T < 1e-4) break;
      const double* q = &s.rots[4 * (size_t)g];
      const double qr = q[0], qx = q[1], qy = q[2], qz = q[3];
      const double R[3][3] = {{1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - qr * qz), 2 * (qx * qz + qr * qy)},
                              {2 * (qx * qy + qr * qz), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - qr * qx)},
                              {2 * (qx * qz - qr * qy), 2 * (qy * qz + qr * qx), 1 - 2 * (qx * qx + qy * qy)}};
      const double* m = &s.means[3 * (size_t)g];
      const double* sc = &s.scales[3 * (size_t)g];
      double lo[3], ld[3];
      for (int k = 0; k < 3; ++k) {
        lo[k] = (R[0][k] * (o[0] - m[0]) + R[1][k] * (o[1] - m[1]) + R[2][k] * (o[2] - m[2])) / (3 * sc[k]);
        ld[k] = (R[0][k] * dn[0] + R[1][k] * dn[1] + R[2][k] * dn[2]) / (3 * sc[k]);
      }
      const double qa = ld[0] * ld[0] + ld[1] * ld[1] + ld[2] * ld[2];
      const double qb = 2 * (ld[0] * lo[0] + ld[1] * lo[1] + ld[2] * lo[2]);
      const double qc = lo[0] * lo[0] + lo[1] * lo[1] + lo[2] * lo[2] - 1;
      const double tmin = -qb / 2 / qa;
      const double depth = tmin / rlen;
      if (std::fabs(depth) <= 1e-9) a_flag = true;
      if (depth < 0) continue;
      const double w = a * T;
      if (wmax < w) {
        wsecond = wmax; wmax = w; dmax = depth; dsc = qb * qb - 4 * qa * qc; im = g;
        for (int k = 0; k < 3; ++k) pr[k] = o[k] + tmin * dn[k];
      } else if (wsecond < w) {
        wsecond = w;
      }
      T = test_T;
    }
    for (int k = 0; k < 3; ++k) out_pts[k * HW + pix] = pr[k];
    out_depth[pix] = dmax;
    accum_alpha[pix] = T;
    disc[pix] = dsc;
    gidx[pix] = im;
    amb[pix] = (a_flag || (wmax > 0 && wmax - wsecond <= eps_w * wmax)) ? 1 : 0;
  }
}

inline void atomic_add(double& dst, double v) {
#pragma omp atomic
  dst += v;
}

// Per-bucket back-to-front composite backward (backward.cu:549-878).
// Outputs: dm2 (P,4) mean2D in NDC incl. |.| parts, dcn (P,4) conic with the
// off-diagonal halved as FB stores it, dop (P) opacity, dcol (P,3) colour.
void composite_backward(const Scene& s, const double* dL, double* dm2, double* dcn, double* dop, double* dcol) {
  const Cam& c = s.cam;
  const int T = s.T(), bs = s.bucket_size, tp = c.bx * c.by;
  const size_t HW = (size_t)c.W * c.H;
  const double cut = 1.0 / 255.0;
  const double hx = 0.5 * c.W, hy = 0.5 * c.H;
#pragma omp parallel for schedule(dynamic, 4)
  for (int t = 0; t < T; ++t) {
    const int tx = t % c.gx, ty = t / c.gx, start = s.ranges[2 * t], end = s.ranges[2 * t + 1];
    const int nb = s.tile_boff[t + 1] - s.tile_boff[t];
    for (int b = 0; b < nb; ++b) {
      if (b * bs >= s.max_contrib[t]) continue;
      const int g0 = start + b * bs, g1 = std::min(end, g0 + bs);
      const int n = g1 - g0;
      std::vector<double> acc((size_t)n * 12, 0.0);
      for (int lp = 0; lp < tp; ++lp) {
        const int px = tx * c.bx + lp % c.bx, py = ty * c.by + lp / c.bx;
        if (px >= c.W || py >= c.H) continue;
        const size_t pix = (size_t)py * c.W + px;
        if (s.last_contrib[pix] <= b * bs) continue;
        const size_t sb = (size_t)(s.tile_boff[t] + b) * tp + lp;
        double Tc = s.accT[sb];
        double res[3], d[3];
        for (int ch = 0; ch < 3; ++ch) {
          res[ch] = s.pix_color[3 * pix + ch] - s.accC[3 * sb + ch];
          d[ch] = dL[ch * HW + pix];
        }
        const double Tf = s.Ts_final[pix];
        const double bgd = s.bg[0] * d[0] + s.bg[1] * d[1] + s.bg[2] * d[2];
        for (int g = g1 - 1; g >= g0; --g) {
          const double* r = &s.rec[(size_t)s.ids[g] * REC];
          const AlphaEval ev = alpha_of(r, px, py);
          const double dx = ev.dx, dy = ev.dy;
          double a = std::min(0.99, ev.a);
          if (a < cut) a = 0;
          const double inv = 1.0 / (1.0 - a);
          Tc = std::min(Tc * inv, 1.0);
          const double w = a * Tc;
          double dLda = 0;
          for (int ch = 0; ch < 3; ++ch) dLda += (Tc * r[F_RGB + ch] - res[ch] * inv) * d[ch];
          for (int ch = 0; ch < 3; ++ch) res[ch] += w * r[F_RGB + ch];
          dLda += -Tf * inv * bgd;
          const double dpw = dLda * a * kLn2;
          double* q = &acc[(size_t)(g - g0) * 12];
          for (int ch = 0; ch < 3; ++ch) q[8 + ch] += w * d[ch];
          // dpower/dcentre (FB backward.cu:614-615), scaled by W/2, H/2 to NDC
          const double mx = dpw * ev.dedx * hx;
          const double my = dpw * ev.dedy * hy;
          q[0] += mx; q[1] += my; q[2] += std::fabs(mx); q[3] += std::fabs(my);
          const double k = -0.5 * kLog2e * dpw;
          q[4] += k * dx * dx; q[5] += k * dx * dy; q[7] += k * dy * dy;
          q[11] += dpw * kLog2e / std::exp2(r[F_LOG2O]);
        }
      }
      for (int g = g0; g < g1; ++g) {
        const int id = s.ids[g];
        const double* q = &acc[(size_t)(g - g0) * 12];
        for (int k = 0; k < 4; ++k) atomic_add(dm2[4 * (size_t)id + k], q[k]);
        for (int k = 0; k < 4; ++k) atomic_add(dcn[4 * (size_t)id + k], q[4 + k]);
        for (int k = 0; k < 3; ++k) atomic_add(dcol[3 * (size_t)id + k], q[8 + k]);
        atomic_add(dop[id], q[11]);
      }
    }
  }
}

// Per-Gaussian backward of projection, EWA covariance, SH and the 3D
// covariance (backward.cu:250-403, 407-483, 488-539, 121-245).
void preprocess_backward(const Scene& s, const double* dm2, const double* dcn, const double* dcol,
                         double* dmean, double* dcov, double* ddc, double* dsh, double* dscale, double* drot) {
  const Cam& c = s.cam;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < s.P; ++i) {
    double* gm = dmean + 3 * (size_t)i;
    gm[0] = gm[1] = gm[2] = 0;
    for (int k = 0; k < 6; ++k) dcov[6 * (size_t)i + k] = 0;
    for (int k = 0; k < 3; ++k) { ddc[3 * (size_t)i + k] = 0; dscale[3 * (size_t)i + k] = 0; }
    for (int k = 0; k < 4; ++k) drot[4 * (size_t)i + k] = 0;
    for (int k = 0; k < 3 * s.M; ++k) dsh[(size_t)i * 3 * s.M + k] = 0;
    if (!(s.radii[i] > 0)) continue;
    const double* p = &s.means[3 * (size_t)i];
    // --- screen covariance -> conic path (backward.cu:250-403)
    double R[3][3], dR[4][3][3];
    quat_rot(&s.rots[4 * (size_t)i], R, dR);
    double sv[3], s2[3];
    for (int k = 0; k < 3; ++k) { sv[k] = c.smod * s.scales[3 * (size_t)i + k]; s2[k] = sv[k] * sv[k]; }
    double Sig[3][3];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        double v = 0;
        for (int k = 0; k < 3; ++k) v += R[a][k] * s2[k] * R[b][k];
        Sig[a][b] = v;
      }
    double t[3];
    c.view_pt(p, t);
    const double limx = 1.3 * c.tanx, limy = 1.3 * c.tany;
    const double tz = t[2], txtz = t[0] / tz, tytz = t[1] / tz;
    const double tx = std::min(limx, std::max(-limx, txtz)) * tz;
    const double ty = std::min(limy, std::max(-limy, tytz)) * tz;
    const double xm = (txtz < -limx || txtz > limx) ? 0.0 : 1.0;
    const double ym = (tytz < -limy || tytz > limy) ? 0.0 : 1.0;
    const double J[2][3] = {{c.fx / tz, 0, -c.fx * tx / (tz * tz)}, {0, c.fy / tz, -c.fy * ty / (tz * tz)}};
    double Mm[2][3];
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 3; ++b) {
        double v = 0;
        for (int k = 0; k < 3; ++k) v += J[a][k] * c.Rw(k, b);
        Mm[a][b] = v;
      }
    double SM[2][3];  // Sigma * M_a^T
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 3; ++b) {
        double v = 0;
        for (int k = 0; k < 3; ++k) v += Sig[b][k] * Mm[a][k];
        SM[a][b] = v;
      }
    double ca = 0.3, cb = 0, cc = 0.3;
    for (int k = 0; k < 3; ++k) { ca += Mm[0][k] * SM[0][k]; cb += Mm[0][k] * SM[1][k]; cc += Mm[1][k] * SM[1][k]; }
    const double gx = dcn[4 * (size_t)i + 0], gy = dcn[4 * (size_t)i + 1], gz = dcn[4 * (size_t)i + 3];
    const double den = ca * cc - cb * cb;
    const double d2 = 1.0 / (den * den + 1e-7);
    const double dLa = d2 * (-cc * cc * gx + 2 * cb * cc * gy + (den - ca * cc) * gz);
    const double dLc = d2 * (-ca * ca * gz + 2 * ca * cb * gy + (den - ca * cc) * gx);
    const double dLb = d2 * 2 * (cb * cc * gx - (den + 2 * cb * cb) * gy + ca * cb * gz);
    double G[3][3];  // dL/dSigma, symmetric, per matrix element
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
        G[a][b] = Mm[0][a] * Mm[0][b] * dLa + 0.5 * (Mm[0][a] * Mm[1][b] + Mm[0][b] * Mm[1][a]) * dLb +
                  Mm[1][a] * Mm[1][b] * dLc;
    // Stored cov3D gradient: diagonal once, off-diagonal counted twice.
    double* gc = dcov + 6 * (size_t)i;
    gc[0] = G[0][0]; gc[1] = 2 * G[0][1]; gc[2] = 2 * G[0][2]; gc[3] = G[1][1]; gc[4] = 2 * G[1][2]; gc[5] = G[2][2];
    double dM[2][3];
    for (int b = 0; b < 3; ++b) {
      dM[0][b] = 2 * dLa * SM[0][b] + dLb * SM[1][b];
      dM[1][b] = 2 * dLc * SM[1][b] + dLb * SM[0][b];
    }
    double dJ[2][3];
    for (int a = 0; a < 2; ++a)
      for (int k = 0; k < 3; ++k) {
        double v = 0;
        for (int b = 0; b < 3; ++b) v += dM[a][b] * c.Rw(k, b);
        dJ[a][k] = v;
      }
    const double iz = 1.0 / tz, iz2 = iz * iz, iz3 = iz2 * iz;
    const double dtx = xm * -c.fx * iz2 * dJ[0][2];
    const double dty = ym * -c.fy * iz2 * dJ[1][2];
    const double dtz = -c.fx * iz2 * dJ[0][0] - c.fy * iz2 * dJ[1][1] + 2 * c.fx * tx * iz3 * dJ[0][2] +
                       2 * c.fy * ty * iz3 * dJ[1][2];
    for (int k = 0; k < 3; ++k) gm[k] = c.Rw(0, k) * dtx + c.Rw(1, k) * dty + c.Rw(2, k) * dtz;
    // --- projection path (backward.cu:504-526)
    double h[4];
    c.proj_pt(p, h);
    const double mw = 1.0 / (h[3] + 1e-7);
    const double g2x = dm2[4 * (size_t)i], g2y = dm2[4 * (size_t)i + 1];
    for (int k = 0; k < 3; ++k) {
      const double jx = c.proj[4 * k] * mw - c.proj[4 * k + 3] * h[0] * mw * mw;
      const double jy = c.proj[4 * k + 1] * mw - c.proj[4 * k + 3] * h[1] * mw * mw;
      gm[k] += jx * g2x + jy * g2y;
    }
    // --- SH path (backward.cu:121-245), only when SH coefficients were given
    if (s.has_shs) {
      const double* r = &s.rec[(size_t)i * REC];
      double v[3] = {p[0] - c.campos[0], p[1] - c.campos[1], p[2] - c.campos[2]};
      const double n2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2], n = std::sqrt(n2);
      double B[16], dB[16][3];
      sh_basis(s.D, v[0] / n, v[1] / n, v[2] / n, B, dB);
      double drgb[3];
      for (int ch = 0; ch < 3; ++ch) drgb[ch] = dcol[3 * (size_t)i + ch] * (1.0 - r[F_CLAMP + ch]);
      for (int ch = 0; ch < 3; ++ch) ddc[3 * (size_t)i + ch] = B[0] * drgb[ch];
      const int nb = (s.D + 1) * (s.D + 1);
      double ddir[3] = {0, 0, 0};
      for (int k = 1; k < nb; ++k) {
        const double* co = &s.shs[((size_t)i * s.M + (k - 1)) * 3];
        double dot = 0;
        for (int ch = 0; ch < 3; ++ch) {
          dsh[((size_t)i * s.M + (k - 1)) * 3 + ch] = B[k] * drgb[ch];
          dot += co[ch] * drgb[ch];
        }
        for (int j = 0; j < 3; ++j) ddir[j] += dB[k][j] * dot;
      }
      // d(v/|v|)/dv applied to ddir
      const double vd = v[0] * ddir[0] + v[1] * ddir[1] + v[2] * ddir[2];
      for (int j = 0; j < 3; ++j) gm[j] += (ddir[j] * n2 - v[j] * vd) / (n2 * n);
    }
    // --- scale / rotation path (backward.cu:407-483): Sigma = R diag(s^2) R^T
    if (s.has_scales) {
      for (int k = 0; k < 3; ++k) {
        double v = 0;
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) v += G[a][b] * R[a][k] * R[b][k];
        dscale[3 * (size_t)i + k] = 2 * sv[k] * v;  // w.r.t. the modified scale, as FB returns it
      }
      double dLR[3][3];  // 2 G R diag(s^2)
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          double v = 0;
          for (int k = 0; k < 3; ++k) v += G[a][k] * R[k][b];
          dLR[a][b] = 2 * v * s2[b];
        }
      for (int q = 0; q < 4; ++q) {
        double v = 0;
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) v += dLR[a][b] * dR[q][a][b];
        drot[4 * (size_t)i + q] = v;
      }
    }
  }
}

}  // namespace

extern "C" {

void* orc_new() { return new Scene(); }
void orc_free(void* h) { delete static_cast<Scene*>(h); }

// Set the scene and camera.  Arrays are float64; optional ones may be NULL.
// Matrices are the column-major 4x4 3DGS view / full-projection matrices.
int orc_set_scene(void* h, int P, int D, int M, const double* means, const double* colors, const double* dc,
                  const double* shs, const double* opac, const double* scales, const double* rots,
                  const uint8_t* culling, double scale_mod, int W, int H, int bx, int by, const double* view,
                  const double* proj, const double* campos, double tanx, double tany, double mult) {
  Scene& s = *static_cast<Scene*>(h);
  s.P = P; s.D = D; s.M = M;
  s.means.assign(means, means + 3 * (size_t)P);
  s.has_colors = colors != nullptr;
  if (colors) s.colors.assign(colors, colors + 3 * (size_t)P);
  if (dc) s.dc.assign(dc, dc + 3 * (size_t)P);
  s.has_shs = shs != nullptr;
  if (shs) s.shs.assign(shs, shs + 3 * (size_t)P * M);
  s.opac.assign(opac, opac + P);
  s.has_scales = scales != nullptr;
  if (!scales || !rots) return 1;
  s.scales.assign(scales, scales + 3 * (size_t)P);
  s.rots.assign(rots, rots + 4 * (size_t)P);
  if (culling) s.culling.assign(culling, culling + P); else s.culling.clear();
  if (!s.has_colors && (!dc || (D > 0 && !shs))) return 1;
  Cam& c = s.cam;
  c.W = W; c.H = H; c.bx = bx; c.by = by;
  c.gx = (W + bx - 1) / bx; c.gy = (H + by - 1) / by;
  std::memcpy(c.view, view, sizeof(c.view));
  std::memcpy(c.proj, proj, sizeof(c.proj));
  std::memcpy(c.campos, campos, sizeof(c.campos));
  c.tanx = tanx; c.tany = tany; c.mult = mult; c.smod = scale_mod;
  c.fx = W / (2.0 * tanx); c.fy = H / (2.0 * tany);
  return 0;
}

void orc_preprocess(void* h) {
  Scene& s = *static_cast<Scene*>(h);
  s.rec.assign((size_t)s.P * REC, 0.0);
  s.radii.assign(s.P, 0); s.rect_area.assign(s.P, 0); s.valid.assign(s.P, 0); s.gauss_amb.assign(s.P, 0);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < s.P; ++i) preprocess_one(s, i);
}

// Replace the per-Gaussian records (e.g. with the device's FP32 records, for
// replay comparisons).  valid[i] = Gaussian passed preprocess.
void orc_set_records(void* h, const double* rec, const int* radii, const uint8_t* valid) {
  Scene& s = *static_cast<Scene*>(h);
  s.rec.assign(rec, rec + (size_t)s.P * REC);
  s.radii.assign(radii, radii + s.P);
  s.valid.assign(valid, valid + s.P);
  s.rect_area.assign(s.P, 0); s.gauss_amb.assign(s.P, 0);
}

// Emit, sort and range the (tile, Gaussian) list.  Returns K.
int64_t orc_emit_sort(void* h, double eps_pair) {
  Scene& s = *static_cast<Scene*>(h);
  emit_and_sort(s, eps_pair);
  build_ranges_from_pairs(s);
  return (int64_t)s.keys.size();
}

// Replace the sorted id list and tile ranges (replay of the device's lists).
void orc_set_lists(void* h, int64_t K, const int* ids, const int* ranges) {
  Scene& s = *static_cast<Scene*>(h);
  s.ids.assign(ids, ids + K);
  s.keys.assign(K, 0);
  s.pair_amb.assign(K, 0);
  s.ranges.assign(ranges, ranges + 2 * (size_t)s.T());
}

void orc_render(void* h, const double* bg, int bucket_size, double eps_alpha, double eps_T) {
  Scene& s = *static_cast<Scene*>(h);
  std::memcpy(s.bg, bg, sizeof(s.bg));
  s.bucket_size = bucket_size;
  s.eps_alpha = eps_alpha; s.eps_T = eps_T;
  composite(s);
}

int64_t orc_num_pairs(void* h) { return (int64_t)static_cast<Scene*>(h)->keys.size(); }
int64_t orc_num_candidates(void* h) { return (int64_t)static_cast<Scene*>(h)->cand_keys.size(); }
void orc_get_candidates(void* h, uint64_t* keys, int* ids) {
  Scene& s = *static_cast<Scene*>(h);
  if (keys) std::memcpy(keys, s.cand_keys.data(), s.cand_keys.size() * 8);
  if (ids) std::memcpy(ids, s.cand_ids.data(), s.cand_ids.size() * 4);
}
int64_t orc_num_buckets(void* h) {
  Scene& s = *static_cast<Scene*>(h);
  return s.tile_boff.empty() ? 0 : s.tile_boff.back();
}
void orc_get_preprocess(void* h, double* rec, int* radii, uint8_t* valid, uint8_t* gauss_amb, int* rect_area) {
  Scene& s = *static_cast<Scene*>(h);
  if (rec) std::memcpy(rec, s.rec.data(), s.rec.size() * sizeof(double));
  if (radii) std::memcpy(radii, s.radii.data(), s.P * sizeof(int));
  if (valid) std::memcpy(valid, s.valid.data(), s.P);
  if (gauss_amb) std::memcpy(gauss_amb, s.gauss_amb.data(), s.P);
  if (rect_area) std::memcpy(rect_area, s.rect_area.data(), s.P * sizeof(int));
}
void orc_get_pairs(void* h, uint64_t* keys, int* ids, uint8_t* amb, int* ranges) {
  Scene& s = *static_cast<Scene*>(h);
  if (keys) std::memcpy(keys, s.keys.data(), s.keys.size() * 8);
  if (ids) std::memcpy(ids, s.ids.data(), s.ids.size() * 4);
  if (amb) std::memcpy(amb, s.pair_amb.data(), s.pair_amb.size());
  if (ranges) std::memcpy(ranges, s.ranges.data(), s.ranges.size() * 4);
}
void orc_get_image(void* h, double* out_color, double* pix_color, int* last_contrib, double* Ts_final,
                   uint8_t* pix_amb, int* max_contrib) {
  Scene& s = *static_cast<Scene*>(h);
  const size_t HW = (size_t)s.cam.W * s.cam.H;
  if (out_color) std::memcpy(out_color, s.out_color.data(), 3 * HW * 8);
  if (pix_color) std::memcpy(pix_color, s.pix_color.data(), 3 * HW * 8);
  if (last_contrib) std::memcpy(last_contrib, s.last_contrib.data(), HW * 4);
  if (Ts_final) std::memcpy(Ts_final, s.Ts_final.data(), HW * 8);
  if (pix_amb) std::memcpy(pix_amb, s.pix_amb.data(), HW);
  if (max_contrib) std::memcpy(max_contrib, s.max_contrib.data(), s.max_contrib.size() * 4);
}

// Full backward.  dL (3,H,W).  Outputs are float64 and fully overwritten.
void orc_backward(void* h, const double* dL, double* dm2, double* dcn, double* dop, double* dcol, double* dmean,
                  double* dcov, double* ddc, double* dsh, double* dscale, double* drot) {
  Scene& s = *static_cast<Scene*>(h);
  std::fill(dm2, dm2 + 4 * (size_t)s.P, 0.0);
  std::fill(dcn, dcn + 4 * (size_t)s.P, 0.0);
  std::fill(dop, dop + (size_t)s.P, 0.0);
  std::fill(dcol, dcol + 3 * (size_t)s.P, 0.0);
  composite_backward(s, dL, dm2, dcn, dop, dcol);
  preprocess_backward(s, dm2, dcn, dcol, dmean, dcov, ddc, dsh, dscale, drot);
}

// Densification statistics (backward.cu:892-918); each output is optional.
void orc_densify(void* h, const double* dm2, double* grad_accum, double* grad_accum_abs, double* max_radii,
                 double* denom) {
  Scene& s = *static_cast<Scene*>(h);
  for (int i = 0; i < s.P; ++i) {
    if (!(s.radii[i] > 0)) continue;
    const double* g = dm2 + 4 * (size_t)i;
    if (denom) denom[i] += 1;
    if (max_radii) max_radii[i] = std::max(max_radii[i], (double)s.radii[i]);
    if (grad_accum) grad_accum[i] += std::sqrt(g[0] * g[0] + g[1] * g[1]);
    if (grad_accum_abs) grad_accum_abs[i] += std::sqrt(g[2] * g[2] + g[3] * g[3]);
  }
}

// Decision signature of the last composite: (#pairs with alpha >= 1/255,
// #pairs clamped at 0.99) and the per-Gaussian clamp flags.
void orc_get_decisions(void* h, int64_t* counts, uint8_t* gauss_clamped) {
  Scene& s = *static_cast<Scene*>(h);
  if (counts) { counts[0] = s.n_alpha_on; counts[1] = s.n_clamped; }
  if (gauss_clamped) std::memcpy(gauss_clamped, s.gauss_clamped.data(), s.gauss_clamped.size());
}

void orc_render_simp(void* h, double eps_alpha, double eps_T, double eps_w, double* wsum, int* wcnt,
                     double* wmaxcnt, uint8_t* amb) {
  render_simp(*static_cast<Scene*>(h), eps_alpha, eps_T, eps_w, wsum, wcnt, wmaxcnt, amb);
}

void orc_render_depth(void* h, double eps_alpha, double eps_T, double eps_w, double* out_pts, double* out_depth,
                      double* accum_alpha, int* gidx, double* disc, uint8_t* amb) {
  render_depth(*static_cast<Scene*>(h), eps_alpha, eps_T, eps_w, out_pts, out_depth, accum_alpha, gidx, disc, amb);
}

int orc_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

}  // extern "C"

extern "C" {
// Colour of SH degree deg at n unit directions (no +0.5 offset, no clamp),
// for pinning the basis against an independent implementation.
// coeffs: (n, 16, 3) with coefficient 0 the DC term; out: (n, 3).
void orc_eval_sh(int n, int deg, const double* dirs, const double* coeffs, double* out) {
  for (int i = 0; i < n; ++i) {
    double B[16];
    sh_basis(deg, dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2], B, nullptr);
    const int nb = (deg + 1) * (deg + 1);
    for (int ch = 0; ch < 3; ++ch) {
      double v = 0;
      for (int k = 0; k < nb; ++k) v += B[k] * coeffs[(i * 16 + k) * 3 + ch];
      out[3 * i + ch] = v;
    }
  }
}
// Upper-triangular 3D covariance (xx, xy, xz, yy, yz, zz) of n Gaussians.
void orc_cov3d(int n, const double* scales, const double* quats, double smod, double* out) {
  for (int i = 0; i < n; ++i) {
    double R[3][3];
    quat_rot(quats + 4 * i, R, nullptr);
    double s2[3];
    for (int k = 0; k < 3; ++k) s2[k] = (smod * scales[3 * i + k]) * (smod * scales[3 * i + k]);
    int o = 0;
    for (int a = 0; a < 3; ++a)
      for (int b = a; b < 3; ++b) {
        double v = 0;
        for (int k = 0; k < 3; ++k) v += R[a][k] * s2[k] * R[b][k];
        out[6 * i + o++] = v;
      }
  }
}
}  // extern "C"
