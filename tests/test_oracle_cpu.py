"""CPU tests: the oracle against the reference's golden fixtures, and the
oracle's own forward/backward consistency (FP64 central differences)."""
import math
from pathlib import Path

import numpy as np
import pytest

import oracle
from fastergs_gb300 import scenes

GOLD = Path(__file__).resolve().parent / "golden"


def test_sh_matches_reference_eval_sh():
    g = np.load(GOLD / "sh_golden.npz")
    for deg in range(4):
        ours = oracle.eval_sh(deg, g["dirs"], g["coeffs"])
        np.testing.assert_allclose(ours, g[f"deg{deg}"], rtol=1e-12, atol=1e-12)


def test_cov3d_matches_reference_build_scaling_rotation():
    g = np.load(GOLD / "cov_golden.npz")
    ours = oracle.cov3d(g["scales"], g["quats"])
    # the reference computes in float32: bound the error by float32 epsilon
    # times the covariance scale (its trace) of each Gaussian
    scale = (g["cov"][:, 0] + g["cov"][:, 3] + g["cov"][:, 5])[:, None]
    assert np.all(np.abs(ours - g["cov"]) <= 4 * np.finfo(np.float32).eps * scale)


def test_camera_matrices_match_reference():
    g = np.load(GOLD / "camera_golden.npz")
    for k in range(g["R"].shape[0]):
        R, T = g["R"][k], g["T"][k]
        w2v = scenes.world_to_view(R, T)
        np.testing.assert_allclose(w2v.T, g["world_view"][k], rtol=1e-5, atol=1e-5)
        P = scenes.projection_matrix(0.01, 100.0, float(g["fovx"][k]), float(g["fovy"][k]))
        np.testing.assert_allclose(P.T, g["proj"][k], rtol=1e-5, atol=1e-6)
        full = w2v.T @ P.T
        np.testing.assert_allclose(full, g["full_proj"][k], rtol=1e-4, atol=1e-4)
        center = np.linalg.inv(w2v.T)[3, :3]
        np.testing.assert_allclose(center, g["center"][k], rtol=1e-4, atol=1e-4)


def test_make_camera_identity_pose():
    cam = scenes.make_camera(256, 256, 60.0, fovy_deg=60.0)
    np.testing.assert_allclose(cam.viewmatrix, np.eye(4), atol=1e-7)
    np.testing.assert_allclose(cam.campos, 0.0, atol=1e-7)
    assert math.isclose(cam.tanfovx, math.tan(math.radians(30)), rel_tol=1e-6)


def _oracle_for(scene, **kw):
    m, sc, rot, op, dc, shs = [np.asarray(a, np.float64) for a in scene.activated()]
    o = oracle.Oracle().set_scene(m, op, sc, rot, scene.camera, dc=dc, shs=shs, sh_degree=scene.sh_degree, **kw)
    return o.preprocess(), (m, sc, rot, op, dc, shs)


def test_oracle_c1_forward_shapes_and_invariants():
    s = scenes.scene_c1()
    o, _ = _oracle_for(s)
    rec = o.records()
    K = o.emit_sort()
    pr = o.pairs()
    assert K == pr["ids"].size > 0
    # ranges partition the sorted list by tile, in tile order
    tiles = (pr["keys"] >> np.uint64(32)).astype(np.int64)
    assert np.all(np.diff(tiles) >= 0)
    counts = pr["ranges"][:, 1] - pr["ranges"][:, 0]
    assert counts.sum() == K
    # every emitted Gaussian is valid and every valid one has radius >= 0
    assert rec["valid"][pr["ids"]].all()
    o.render()
    im = o.image()
    T = im["Ts_final"]
    assert np.all((T >= 0) & (T <= 1))
    assert np.all(im["out_color"] >= 0)
    # colour + T * bg with bg = 0 is the pixel colour
    np.testing.assert_allclose(im["out_color"].transpose(1, 2, 0), im["pixel_colors"], atol=1e-15)


def _loss_and_grads(scene, params, dL, grads=False):
    m, sc, rot, op, dc, shs = params
    o = oracle.Oracle().set_scene(m, op, sc, rot, scene.camera, dc=dc, shs=shs, sh_degree=scene.sh_degree)
    o.preprocess()
    o.emit_sort()
    o.render()
    im = o.image()
    L = float((im["out_color"] * dL).sum())
    return (L, o.backward(dL)) if grads else L


@pytest.mark.parametrize("which", ["means", "scales", "rotations", "opacities", "dc", "shs"])
def test_oracle_backward_matches_central_differences(which):
    s = scenes.scene_c5a(P=300)
    s.camera = scenes.make_camera(64, 64, 60.0, fovy_deg=60.0)
    params = [np.asarray(a, np.float64) for a in s.activated()]
    dL = scenes.upstream_grad(3, 64, 64).astype(np.float64)
    _, g = _loss_and_grads(s, params, dL, grads=True)
    idx = ["means", "scales", "rotations", "opacities", "dc", "shs"].index(which)
    key = ["dmean3D", "dscale", "drot", "dopacity", "ddc", "dsh"][idx]
    ga = g[key].reshape(-1)
    order = np.argsort(-np.abs(ga))[:5]
    for fi in order:
        base = params[idx].reshape(-1)
        h = 1e-6 * max(abs(base[fi]), 1e-2)
        res = []
        for sgn in (1, -1):
            p = [a.copy() for a in params]
            p[idx].reshape(-1)[fi] += sgn * h
            res.append(_loss_and_grads(s, p, dL))
        fd = (res[0] - res[1]) / (2 * h)
        assert abs(fd - ga[fi]) <= 1e-5 * max(abs(fd), 1e-3), (which, fi, fd, ga[fi])
