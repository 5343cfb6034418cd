"""The importance pass (render_simp) and the depth pass (render_depth) against
the FP64 oracle replaying the device's own records and sorted lists.

Tolerances: per-Gaussian weight sums within 1e-4 of the largest (FP32 sums
of many weights), counts and max-weight counts exact; per pixel the index of
the largest-weight Gaussian exact, final transmittance within 1e-5, depth and
points within 1e-4 relative.  Gaussians (simp) and pixels (depth) that the
oracle flags as within rounding distance of a different discrete decision
(alpha at the 1/255 cut, a stop test at T = 1e-4, a near-tie for the largest
weight) are excluded.
"""
import numpy as np
import pytest
import torch

from fastergs_gb300 import GaussianRasterizer, _C, scenes
from gpu_util import gpu_records_as_oracle, oracle_scene, run_forward

pytestmark = pytest.mark.gpu

SCENES = {
    "c1": lambda: scenes.scene_c1(),
    "c2_small": lambda: scenes.scene_c2(seed=0, P=20000, width=320, height=208),
    "c2_ragged": lambda: scenes.scene_c2(seed=1, P=8000, width=203, height=77),
}


def _replay(s, fw):
    o = oracle_scene(s)
    rec, radii, _ = gpu_records_as_oracle(fw)
    valid = (radii > 0) | np.isin(np.arange(s.P), fw["vals_sorted"])
    o.set_records(rec, radii, valid)
    o.set_lists(fw["vals_sorted"], fw["ranges"])
    return o


@pytest.mark.parametrize("name", list(SCENES))
def test_render_simp_matches_oracle_replay(cuda_device, name):
    s = SCENES[name]()
    fw = run_forward(s, cuda_device)
    buf, cam = fw["buf"], s.camera
    _, w, cnt, mx = _C.ops.render_simp(s.P, fw["K"], cam.width, cam.height, buf.splat_buffer,
                                       buf.gaussian_keys_sorted, buf.gaussian_values_sorted, buf.ranges)
    torch.cuda.synchronize()
    assert _C.device_errors(cuda_device) == 0
    r = _replay(s, fw).render_simp()
    ok = ~r["ambiguous"]
    assert ok.mean() > 0.95
    w = w.cpu().numpy().astype(np.float64)
    assert np.abs(w - r["weights"])[ok].max() <= 1e-4 * max(r["weights"].max(), 1e-30)
    np.testing.assert_array_equal(cnt.cpu().numpy()[ok], r["counts"][ok])
    np.testing.assert_array_equal(mx.cpu().numpy()[ok], r["max_counts"][ok])
    assert r["counts"].sum() > 0 and r["max_counts"].sum() > 0


@pytest.mark.parametrize("name", list(SCENES))
def test_render_depth_matches_oracle_replay(cuda_device, name):
    s = SCENES[name]()
    fw = run_forward(s, cuda_device)
    buf, cam, T = fw["buf"], s.camera, fw["T"]
    f = lambda a: torch.tensor(np.asarray(a, np.float32), device=cuda_device)
    pts, depth, alpha, gidx, disc = _C.ops.render_depth(
        s.P, fw["K"], cam.width, cam.height, buf.splat_buffer, buf.gaussian_keys_sorted, buf.gaussian_values_sorted,
        buf.ranges, T["means"], T["scales"], T["rotations"], f(cam.projmatrix), f(cam.campos))
    torch.cuda.synchronize()
    assert _C.device_errors(cuda_device) == 0
    assert pts.shape == (3, cam.height, cam.width) and depth.shape == (1, cam.height, cam.width)
    r = _replay(s, fw).render_depth()
    ok = ~r["ambiguous"]
    assert ok.mean() > 0.95
    np.testing.assert_array_equal(gidx.cpu().numpy()[0][ok], r["gidx"][ok])
    assert np.abs(alpha.cpu().numpy()[0] - r["accum_alpha"])[ok].max() <= 1e-5
    d = depth.cpu().numpy()[0].astype(np.float64)
    assert np.abs(d - r["out_depth"])[ok].max() <= 1e-4 * max(np.abs(r["out_depth"]).max(), 1e-30)
    p = pts.cpu().numpy().astype(np.float64)
    assert np.abs(p - r["out_pts"])[:, ok].max() <= 1e-4 * max(np.abs(r["out_pts"]).max(), 1e-30)
    hit = ok & (r["gidx"] >= 0) & (r["out_depth"] > 0)
    dd = disc.cpu().numpy()[0].astype(np.float64)
    assert np.abs(dd - r["discriminants"])[hit].max() <= 1e-3 * max(np.abs(r["discriminants"][hit]).max(), 1e-30)


def test_rasterizer_methods_as_mini_splatting_calls_them(cuda_device):
    """GaussianRasterizer.render_simp / render_depth with the keyword call of
    mini-splatting2/gaussian_renderer/render_faster.py (mult 0.5, culling)."""
    from test_gpu_api import settings_for
    s = SCENES["c2_small"]()
    m, sc, rot, op, dc, shs = s.activated()
    t = lambda a: torch.tensor(np.ascontiguousarray(a), device=cuda_device)
    st = settings_for(s.camera, cuda_device, s.sh_degree)._replace(mult=0.5)
    cull = torch.zeros(s.P, dtype=torch.bool, device=cuda_device)
    cull[::7] = True
    rast = GaussianRasterizer(st)
    radii, w, cnt, mx = rast.render_simp(means3D=t(m), dc=t(dc), shs=t(shs), culling=cull, opacities=t(op),
                                         scales=t(sc), rotations=t(rot))
    assert radii.shape == (s.P,) and w.shape == (s.P,) and cnt.dtype == torch.int32
    assert (radii[cull] == 0).all() and (w[cull] == 0).all() and (cnt[cull] == 0).all()
    assert float(mx.sum()) <= s.camera.width * s.camera.height
    res = rast.render_depth(means3D=t(m), dc=t(dc), shs=t(shs), culling=cull, opacities=t(op), scales=t(sc),
                            rotations=t(rot))
    assert set(res) >= {"out_pts", "accum_alpha", "rendered_depth", "gidx", "discriminants"}
    a = res["accum_alpha"]
    assert a.shape == (1, s.camera.height, s.camera.width) and float(a.min()) >= 0 and float(a.max()) <= 1
    assert not bool(torch.isin(res["gidx"][a < 1], torch.nonzero(cull).flatten()).any())
