"""The FP64 oracle against golden vectors produced by the reference CUDA
backend itself (FB, built for sm_103a from its own sources and run on a GB300;
tests/golden/make_fb_golden.py).  This pins the oracle's restatement of FB's
rasterizer core -- tile test, key emission, sort order, tile ranges, bucket
compositing and merge, backward and densification statistics -- to what FB
computes, on the seeded scenes C1 (10k Gaussians, 256x256, SH 0), C5a (2k,
128x128, SH 1) and c2_small (20k Gaussians of the 1M distribution, 320x208,
SH 3).

Tolerances (FB runs in FP32 with approximate ex2 / lg2 / sqrt; the oracle in
FP64):
  * radii, the bucket count, tile ranges and every tile's sorted id list:
    bit-exact, except entries the oracle flags as within rounding distance of
    a threshold (Gaussians, and tiles holding such a pair);
  * on the pixels outside ``dL_mask`` (flagged pixels and the tiles of
    flagged pairs): last_contributor bit-exact; image and Ts_final max-abs
    1e-5 on C1 and C5a; on c2_small 1e-5 on at least 99.5% of the pixels,
    3e-5 on 99.99% and 2e-3 on all: FB evaluates the alpha
    exponent as con_o.w + con_o.x dx^2 + con_o.y dx dy + con_o.z dy^2 in
    FP32, which loses digits far from the centre of a thin Gaussian (one
    c2_small pixel is 1.4e-3 off FP64 for that reason; this library's
    record form keeps the same pixel within 1e-5);
  * gradients (FB's upstream gradient is zero on ``dL_mask``): per Gaussian
    and tensor, max |FB - oracle| <= 1e-4 max |oracle|.  For the covariance
    path (dL/dcov3D, dL/dscale, dL/drot) the bound is
    (1e-4 + 5e-10 kappa^2) max |oracle|, kappa the condition number of the
    Gaussian's 2D covariance: FB projects dL/dSigma2 on each principal axis
    in FP32, which cancels with kappa^2 (c2_small holds Gaussians with kappa
    near 5000; there FB is ~3e-3 off FP64 while this library's kernels stay
    within 5e-5, see tests/test_gpu_fb_golden.py);
  * densification statistics: denom and max_radii exact, the gradient-norm
    accumulator within 1e-4 of its largest value.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle
from fastergs_gb300 import scenes

HERE = Path(__file__).resolve().parent
GOLDEN = HERE / "golden"
SCENES = {
    "c1": lambda: scenes.scene_c1(),
    "c5a": lambda: scenes.scene_c5a(),
    "c2_small": lambda: scenes.scene_c2(seed=0, P=20000, width=320, height=208),
}
GRADS = ["dmean2D", "dcolor", "dopacity", "dmean3D", "dcov3D", "ddc", "dsh", "dscale", "drot"]
COV_PATH = {"dcov3D", "dscale", "drot"}
KAPPA_COEF = 5e-10


def load(name):
    return dict(np.load(GOLDEN / f"fb_{name}.npz"))


def oracle_run(name):
    s = SCENES[name]()
    m, sc, rot, op, dc, shs = [np.asarray(a, np.float64) for a in s.activated()]
    o = oracle.Oracle().set_scene(m, op, sc, rot, s.camera, dc=dc, shs=shs, sh_degree=s.sh_degree)
    o.preprocess()
    rec = o.records()
    o.emit_sort()
    pr = o.pairs()
    o.render()
    return s, o, rec, pr, o.image()


def kappa_of(rec):
    """Condition number of each Gaussian's 2D covariance (from its conic), 1 for invalid ones."""
    a, b, c = rec["rec"][:, 16], rec["rec"][:, 17], rec["rec"][:, 18]
    half_tr = 0.5 * (a + c)
    disc = np.sqrt(np.maximum(half_tr * half_tr - (a * c - b * b), 0.0))
    with np.errstate(divide="ignore", invalid="ignore"):
        k = (half_tr + disc) / (half_tr - disc)
    return np.where(rec["valid"] & np.isfinite(k), k, 1.0)


@pytest.fixture(scope="module", params=list(SCENES))
def case(request):
    name = request.param
    return (name, load(name)) + oracle_run(name)


def test_pairs_sort_and_ranges_match_fb(case):
    name, g, s, o, rec, pr, im = case
    amb = rec["ambiguous"]
    assert amb.mean() < 0.01
    np.testing.assert_array_equal(g["radii"][~amb], rec["radii"][~amb])
    rg_fb, rg_o = g["ranges"], pr["ranges"]
    assert rg_fb.shape == rg_o.shape
    flagged = 0
    flagged_tiles = set(pr["flagged_tiles"].tolist())
    for t in range(rg_o.shape[0]):
        ids_o = pr["ids"][rg_o[t, 0]:rg_o[t, 1]]
        if t in flagged_tiles:
            flagged += 1
            continue
        np.testing.assert_array_equal(g["vals_sorted"][rg_fb[t, 0]:rg_fb[t, 1]], ids_o, err_msg=f"tile {t}")
        assert rg_fb[t, 1] - rg_fb[t, 0] == rg_o[t, 1] - rg_o[t, 0]
    assert pr["ambiguous"].sum() <= 1e-3 * pr["ids"].size  # flagged pairs
    if flagged == 0:
        np.testing.assert_array_equal(rg_fb, rg_o)
        assert int(g["K"]) == int(pr["ids"].size)
    assert int(g["bucket_sum"]) == im["num_buckets"]


def test_image_matches_fb(case):
    name, g, s, o, rec, pr, im = case
    ok = ~g["dL_mask"]
    assert ok.mean() > 0.95
    np.testing.assert_array_equal(g["last_contributor"][ok], im["last_contributor"][ok])
    for err in (np.abs(g["out_color"] - im["out_color"]).max(0)[ok], np.abs(g["Ts_final"] - im["Ts_final"])[ok]):
        if name in ("c1", "c5a"):
            assert err.max() <= 1e-5, err.max()
        assert (err <= 1e-5).mean() >= 0.995, (err > 1e-5).sum()
        assert (err <= 3e-5).mean() >= 0.9999, (err > 3e-5).sum()
        assert err.max() <= 2e-3, err.max()


def test_gradients_match_fb(case):
    name, g, s, o, rec, pr, im = case
    dL = scenes.upstream_grad(0, s.camera.height, s.camera.width).astype(np.float64)
    dL[:, g["dL_mask"]] = 0.0
    r = o.backward(dL)
    kappa = kappa_of(rec)
    for k in GRADS:
        fb = g[k].astype(np.float64)
        ref = r[k][: fb.shape[0]].reshape(fb.shape)
        fb, ref = fb.reshape(fb.shape[0], -1), ref.reshape(ref.shape[0], -1)
        if k == "dmean2D":
            fb, ref = fb[:, :2], ref[:, :2]
        mx = np.abs(ref).max()
        if mx == 0.0:
            assert np.all(fb == 0.0), k
            continue
        row = np.abs(fb - ref).max(1) / mx
        bound = 1e-4 + (KAPPA_COEF * kappa[: fb.shape[0]] ** 2 if k in COV_PATH else 0.0)
        worst = int(np.argmax(row - bound))
        assert np.all(row <= bound), (k, worst, row[worst], kappa[worst])


def test_densification_statistics_match_fb(case):
    name, g, s, o, rec, pr, im = case
    dL = scenes.upstream_grad(0, s.camera.height, s.camera.width).astype(np.float64)
    dL[:, g["dL_mask"]] = 0.0
    r = o.backward(dL)
    P = s.P
    acc, acc_abs, maxr, den = (np.zeros(P) for _ in range(4))
    acc, acc_abs, maxr, den = o.densify(r["dmean2D"], acc, acc_abs, maxr, den)
    amb = rec["ambiguous"]
    np.testing.assert_array_equal(g["denom"][~amb], den[~amb])
    np.testing.assert_array_equal(g["max_radii"][~amb], maxr[~amb])
    assert np.abs(g["xyz_gradient_accum"] - acc).max() <= 1e-4 * np.abs(acc).max()
