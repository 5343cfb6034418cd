"""GPU parity of the backward path against the FP64 oracle.

Tolerance: every gradient tensor within 1e-4 relative, measured as
max |device - oracle| <= 1e-4 * max |oracle| per tensor, and every entry
within 1e-4 of itself plus a floor of 5e-6 of the tensor's largest value
(dL/drot: the per-tensor bound alone; gpu_util.check_gradients).  Upstream gradients are
zeroed at pixels the oracle flags as ambiguous (a discrete decision within
rounding distance of its threshold), in both the device and the oracle run,
so a flipped decision cannot leak into the comparison; against the fully
independent FP64 pipeline also on the tiles whose lists hold a pair whose
tile test is within rounding distance (a pair one side keeps and the other
drops changes every pixel of the tile).
"""
import numpy as np
import pytest
import torch

from fastergs_gb300 import scenes
from gpu_util import ambiguous_tiles_mask, check_gradients, oracle_scene, replay_oracle, run_backward, run_forward

pytestmark = pytest.mark.gpu

KEYS = ["dmean2D", "dopacity", "dcolor", "dmean3D", "ddc", "dsh", "dscale", "drot"]


def _compare(gpu, orc, keys=KEYS, tol=1e-4, per_entry=True):
    check_gradients(gpu, orc, keys=keys, tol=tol, per_entry=per_entry)


def small_c2(seed=0, P=20000, W=320, H=208):
    return scenes.scene_c2(seed=seed, P=P, width=W, height=H)


def deep_tiles():
    from test_gpu_forward import deep_tiles as scene
    return scene()


SCENES = {"c1": lambda: scenes.scene_c1(), "c5a": lambda: scenes.scene_c5a(), "c2_small": lambda: small_c2(),
          "deep": deep_tiles}


@pytest.mark.parametrize("name", list(SCENES))
def test_backward_matches_oracle_replay(cuda_device, name):
    s = SCENES[name]()
    fw = run_forward(s, cuda_device)
    o = replay_oracle(s, fw)
    amb = o.image()["ambiguous"]
    dL = scenes.upstream_grad(1, s.camera.height, s.camera.width)
    dL[:, amb] = 0.0
    g = run_backward(s, fw, dL, cuda_device)
    r = o.backward(dL.astype(np.float64))
    _compare(g, r)


@pytest.mark.parametrize("name", ["c1", "c5a", "c2_small"])
def test_backward_end_to_end_vs_fp64_oracle(cuda_device, name):
    s = SCENES[name]()
    fw = run_forward(s, cuda_device)
    o = oracle_scene(s).preprocess()
    o.emit_sort(eps_pair=1e-4)
    o.render(eps_alpha=1e-4, eps_T=1e-4)
    im = o.image()
    amb = ambiguous_tiles_mask(o, im, s.camera.width) | replay_oracle(s, fw).image()["ambiguous"]
    assert amb.mean() < 0.2
    dL = scenes.upstream_grad(2, s.camera.height, s.camera.width)
    dL[:, amb] = 0.0
    o2 = oracle_scene(s).preprocess()
    o2.emit_sort(eps_pair=1e-4)
    o2.render()
    r = o2.backward(dL.astype(np.float64))
    g = run_backward(s, fw, dL, cuda_device)
    _compare(g, r)


def test_densification_statistics(cuda_device):
    s = scenes.scene_c5a(seed=2)
    fw = run_forward(s, cuda_device)
    dL = scenes.upstream_grad(4, s.camera.height, s.camera.width)
    g = run_backward(s, fw, dL, cuda_device, stats=True)
    accum, accum_abs, max_radii, denom = g["stats"]
    radii = fw["radii"].cpu().numpy()
    vis = radii > 0
    np.testing.assert_array_equal(denom, vis.astype(np.float64))
    np.testing.assert_array_equal(max_radii, np.where(vis, radii, 0).astype(np.float64))
    dm = g["dmean2D"]
    np.testing.assert_allclose(accum, np.where(vis, np.hypot(dm[:, 0], dm[:, 1]), 0), rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(accum_abs, np.where(vis, np.hypot(dm[:, 2], dm[:, 3]), 0), rtol=1e-5, atol=1e-7)


def test_precomputed_colour_gradients(cuda_device):
    s = scenes.scene_c1(seed=4, P=3000)
    colors = np.random.default_rng(9).uniform(0, 1, size=(s.P, 3)).astype(np.float32)
    fw = run_forward(s, cuda_device, colors=colors)
    o = replay_oracle(s, fw, colors=colors)
    amb = o.image()["ambiguous"]
    dL = scenes.upstream_grad(5, s.camera.height, s.camera.width)
    dL[:, amb] = 0.0
    g = run_backward(s, fw, dL, cuda_device)
    r = o.backward(dL.astype(np.float64))
    _compare(g, r, keys=["dmean2D", "dopacity", "dcolor", "dmean3D", "dscale", "drot"])
    assert np.all(g["ddc"] == 0)


def test_zero_gaussians(cuda_device):
    s = scenes.scene_c1(seed=1, P=500)
    fw = run_forward(s, cuda_device, culling=np.ones(s.P, bool))
    g = run_backward(s, fw, scenes.upstream_grad(0, 256, 256), cuda_device)
    for k in KEYS:
        assert np.all(g[k] == 0), k


@pytest.mark.parametrize("WH", [(1, 1), (5, 3), (17, 33), (1031, 9), (640, 480)],
                         ids=lambda wh: f"{wh[0]}x{wh[1]}")
def test_backward_huge_gaussians_and_odd_image_sizes(cuda_device, WH):
    from test_gpu_forward import huge_and_odd
    s = huge_and_odd(*WH)
    fw = run_forward(s, cuda_device, bg=(0.25, 0.5, 0.75))
    o = replay_oracle(s, fw, bg=(0.25, 0.5, 0.75))
    amb = o.image()["ambiguous"]
    dL = scenes.upstream_grad(3, s.camera.height, s.camera.width)
    dL[:, amb] = 0.0
    g = run_backward(s, fw, dL, cuda_device, stats=True)
    r = o.backward(dL.astype(np.float64))
    _compare(g, r, per_entry=WH[0] * WH[1] >= 1000)
    # a Gaussian that no pixel saw has exactly zero gradients
    unseen = ~np.isin(np.arange(s.P), fw["vals_sorted"])
    for k in ("dmean3D", "dopacity", "ddc", "dscale", "drot"):
        assert np.all(g[k][unseen] == 0.0), k
