"""GPU tests of the drop-in Python API: GaussianRasterizer / autograd,
capacity errors, SparseGaussianAdam, and finite differences through the whole
chain (activations + rasterizer) against the FP64 oracle."""
import numpy as np
import pytest
import torch

import oracle
from fastergs_gb300 import (Buffer, GaussianRasterizationSettings, GaussianRasterizer, SparseGaussianAdam,
                            _C, _RasterizeGaussians, scenes)

pytestmark = pytest.mark.gpu


def settings_for(cam, dev, deg, bg=(0.0, 0.0, 0.0)):
    t = lambda a: torch.tensor(np.asarray(a, np.float32), device=dev)
    return GaussianRasterizationSettings(
        image_height=cam.height, image_width=cam.width, tanfovx=cam.tanfovx, tanfovy=cam.tanfovy, bg=t(bg),
        scale_modifier=1.0, viewmatrix=t(cam.viewmatrix), projmatrix=t(cam.projmatrix), sh_degree=deg,
        campos=t(cam.campos), mult=1.0, prefiltered=False, debug=False)


def raw_params(scene, dev):
    t = lambda a: torch.tensor(np.asarray(a, np.float32), device=dev, requires_grad=True)
    return dict(means=t(scene.means), log_scales=t(scene.log_scales), quats=t(scene.quats),
                logits=t(scene.opacity_logits), dc=t(scene.dc), shs=t(scene.shs))


def render(scene, p, dev):
    rast = GaussianRasterizer(settings_for(scene.camera, dev, scene.sh_degree))
    q = p["quats"] / p["quats"].norm(dim=1, keepdim=True)
    return rast(means3D=p["means"], opacities=torch.sigmoid(p["logits"]), dc=p["dc"], shs=p["shs"],
                scales=torch.exp(p["log_scales"]), rotations=q)


def test_autograd_roundtrip_and_radii(cuda_device):
    s = scenes.scene_c1()
    p = raw_params(s, cuda_device)
    img, radii = render(s, p, cuda_device)
    assert img.shape == (3, 256, 256) and radii.dtype == torch.int32
    (img * torch.tensor(scenes.upstream_grad(0, 256, 256), device=cuda_device)).sum().backward()
    for k, v in p.items():
        assert v.grad is not None and torch.isfinite(v.grad).all(), k


def test_argument_validation_mirrors_reference(cuda_device):
    s = scenes.scene_c1(P=100)
    rast = GaussianRasterizer(settings_for(s.camera, cuda_device, 0))
    m = torch.zeros((100, 3), device=cuda_device)
    with pytest.raises(Exception, match="one of either SHs"):
        rast(means3D=m, opacities=m[:, :1])
    with pytest.raises(Exception, match="scale/rotation pair"):
        rast(means3D=m, opacities=m[:, :1], shs=torch.zeros((100, 15, 3), device=cuda_device))


def test_capacity_overflow_raises(cuda_device):
    s = scenes.scene_c1()
    slot = _RasterizeGaussians.__dict__["buffer"]  # the lazily allocated shared Buffer
    old = slot._buf
    try:
        small = Buffer(device=cuda_device, MAX_NUM_RENDERED=1024)
        small.splat_buffer = torch.zeros((s.P, 32), device=cuda_device)  # room for every Gaussian's record
        slot._buf = small
        with pytest.raises(RuntimeError, match="Too many k-v pairs"):
            render(s, raw_params(s, cuda_device), cuda_device)
    finally:
        slot._buf = old
    img, _ = render(s, raw_params(s, cuda_device), cuda_device)
    assert torch.isfinite(img).all()


def test_sparse_adam_matches_masked_adam(cuda_device):
    torch.manual_seed(0)
    N, M = 1000, 3
    param = torch.randn(N, M, device=cuda_device, requires_grad=True)
    ref = param.detach().clone()
    opt = SparseGaussianAdam([param], lr=0.01, eps=1e-15)
    m1 = torch.zeros_like(ref)
    m2 = torch.zeros_like(ref)
    for step in range(1, 4):
        g = torch.randn(N, M, device=cuda_device)
        vis = torch.rand(N, device=cuda_device) < 0.5
        param.grad = g.clone()
        opt.step(vis, N)
        lr = 0.01 * (1 - 0.999 ** step) ** 0.5 / (1 - 0.9 ** step)
        m1n = 0.9 * m1 + 0.1 * g
        m2n = 0.999 * m2 + 0.001 * g * g
        upd = ref - lr * m1n / (m2n.sqrt() + 1e-15)
        v = vis[:, None]
        ref = torch.where(v, upd, ref)
        m1 = torch.where(v, m1n, m1)
        m2 = torch.where(v, m2n, m2)
        torch.testing.assert_close(param.detach(), ref, rtol=1e-5, atol=1e-6)


def _oracle_loss(scene, raw, dL):
    means, ls, q, lg, dc, shs = raw
    qn = q / np.linalg.norm(q, axis=1, keepdims=True)
    o = oracle.Oracle().set_scene(means, 1 / (1 + np.exp(-lg)), np.exp(ls), qn, scene.camera, dc=dc, shs=shs,
                                  sh_degree=scene.sh_degree)
    o.preprocess()
    K = o.emit_sort()
    o.render()
    im = o.image()
    (non, ncl), cl = o.decisions()
    sig = (K, non, ncl, int(im["last_contributor"].sum()))
    return float((im["out_color"] * dL).sum()), sig, cl


def test_gradients_match_fp64_finite_differences(cuda_device):
    """C5a: 2,000 Gaussians, 128x128, SH degree 1; FP64 central differences
    (relative step 1e-4) on 200 seeded entries over means, log-scales,
    quaternions, opacity logits and SH; entries whose +/- evaluations change a
    discrete decision (pair list, alpha cut-off, merge break) or touch an
    alpha clamped at 0.99 (where FB's analytic gradient is not the derivative)
    are skipped and counted.  Tolerance per entry:
    |device - fd| <= 1e-4 * |fd| + 1e-4 * max |fd| of the parameter group."""
    s = scenes.scene_c5a()
    dL = scenes.upstream_grad(0, s.camera.height, s.camera.width).astype(np.float64)
    p = raw_params(s, cuda_device)
    img, _ = render(s, p, cuda_device)
    (img * torch.tensor(dL, dtype=torch.float32, device=cuda_device)).sum().backward()
    grads = [p[k].grad.cpu().numpy().astype(np.float64) for k in ("means", "log_scales", "quats", "logits", "dc",
                                                                   "shs")]
    raw = [np.asarray(a, np.float64) for a in (s.means, s.log_scales, s.quats, s.opacity_logits, s.dc, s.shs)]
    _, sig0, clamped = _oracle_loss(s, raw, dL)
    rng = np.random.default_rng(123)
    groups = [0, 1, 2, 3, 4, 5]
    checked, skipped = 0, 0
    per_group = {g: [] for g in groups}
    for n in range(200):
        gi = groups[n % len(groups)]
        arr = raw[gi]
        if gi == 5:  # SH degree 1 uses the first three rest coefficients
            i = int(rng.integers(s.P))
            flat = np.ravel_multi_index((i, int(rng.integers(3)), int(rng.integers(3))), arr.shape)
        else:
            flat = int(rng.integers(arr.size))
        gauss = np.unravel_index(flat, arr.shape)[0]
        if clamped[gauss]:
            skipped += 1
            continue
        h = 1e-4 * max(abs(arr.reshape(-1)[flat]), 1e-2)
        vals = []
        sigs = []
        for sgn in (1, -1):
            r2 = [a.copy() for a in raw]
            r2[gi].reshape(-1)[flat] += sgn * h
            L, sig, _ = _oracle_loss(s, r2, dL)
            vals.append(L)
            sigs.append(sig)
        if sigs[0] != sig0 or sigs[1] != sig0:
            skipped += 1
            continue
        fd = (vals[0] - vals[1]) / (2 * h)
        per_group[gi].append((fd, grads[gi].reshape(-1)[flat]))
        checked += 1
    assert checked >= 120, (checked, skipped)
    for gi, pairs in per_group.items():
        if not pairs:
            continue
        fd = np.array([a for a, _ in pairs])
        an = np.array([b for _, b in pairs])
        tol = 1e-4 * np.abs(fd) + 1e-4 * np.abs(fd).max()
        assert np.all(np.abs(an - fd) <= tol), (gi, np.max(np.abs(an - fd) / (np.abs(fd) + 1e-12)))


def test_vanilla_rasterize_gaussians_alias(cuda_device):
    """_C.rasterize_gaussians / rasterize_gaussians_backward take the vanilla
    extension's layouts (sh (P, 1 + M, 3) with DC first, dL/dmeans2D (P, 3))
    and give the drop-in path's image, radii and gradients."""
    from fastergs_gb300 import _C
    s = scenes.scene_c5a()
    dev = cuda_device
    st = settings_for(s.camera, dev, s.sh_degree, bg=(0.1, 0.2, 0.3))
    m, sc, rot, op, dc, shs = s.activated()
    t = lambda a: torch.tensor(np.ascontiguousarray(a), device=dev)
    leaves = {k: t(v).requires_grad_(True) for k, v in dict(means=m, scales=sc, rotations=rot, opacities=op, dc=dc,
                                                             shs=shs).items()}
    img, radii = GaussianRasterizer(st)(means3D=leaves["means"], opacities=leaves["opacities"], dc=leaves["dc"],
                                        shs=leaves["shs"], scales=leaves["scales"], rotations=leaves["rotations"])
    dL = t(scenes.upstream_grad(3, s.camera.height, s.camera.width))
    torch.autograd.backward(img, grad_tensors=dL)
    empty = torch.empty(0, device=dev)
    sh_full = torch.cat([t(dc), t(shs)], dim=1)
    R, color, radii2, geom, binning, image = _C.rasterize_gaussians(
        st.bg, t(m), empty, t(op), t(sc), t(rot), 1.0, empty, st.viewmatrix, st.projmatrix, st.tanfovx, st.tanfovy,
        st.image_height, st.image_width, sh_full, s.sh_degree, st.campos, False, False)
    assert R > 0 and color.shape == img.shape
    assert torch.equal(radii2, radii)
    assert (color - img.detach()).abs().max().item() <= 1e-5
    g = _C.rasterize_gaussians_backward(st.bg, t(m), radii2, empty, t(sc), t(rot), 1.0, empty, st.viewmatrix,
                                        st.projmatrix, st.tanfovx, st.tanfovy, dL, sh_full, s.sh_degree, st.campos,
                                        geom, R, binning, image, False)
    dmeans2D, dcolors, dop, dmean3D, dcov3D, dsh, dscale, drot = g
    assert dmeans2D.shape == (s.P, 3) and dsh.shape == sh_full.shape and dop.shape == (s.P, 1)
    rel = lambda a, b: ((a - b).abs().max() / b.abs().max().clamp_min(1e-30)).item()
    assert rel(dmean3D, leaves["means"].grad) <= 1e-5
    assert rel(dscale, leaves["scales"].grad) <= 1e-5
    assert rel(drot, leaves["rotations"].grad) <= 1e-5
    assert rel(dop, leaves["opacities"].grad) <= 1e-5
    assert rel(dsh[:, :1], leaves["dc"].grad) <= 1e-5
    assert rel(dsh[:, 1:], leaves["shs"].grad) <= 1e-5


def test_render_from_ply_file_matches_direct_render(cuda_device, tmp_path):
    """A scene written as a 3DGS PLY, read back and rasterized with settings from
    fastergs_gb300.cameras gives the direct render's radii and image."""
    from fastergs_gb300 import cameras, ply
    s = scenes.scene_c1()
    params = {"xyz": s.means, "f_dc": s.dc, "f_rest": s.shs, "opacity": s.opacity_logits, "scaling": s.log_scales,
              "rotation": s.quats}
    ply.save_ply(tmp_path / "point_cloud.ply", params)
    loaded = ply.load_ply(tmp_path / "point_cloud.ply")  # 15 coefficients stored, rendered at the scene's degree
    assert loaded["f_rest"].shape == s.shs.shape
    model = ply.to_device(loaded, cuda_device)
    rs = cameras.raster_settings(s.camera, sh_degree=s.sh_degree, device=cuda_device)
    with torch.no_grad():
        img, radii = GaussianRasterizer(rs)(**ply.activated(model))
        img_ref, radii_ref = render(s, raw_params(s, cuda_device), cuda_device)
    assert torch.equal(radii, radii_ref)
    assert float((img - img_ref).abs().max()) < 1e-6


def test_expired_wait_reports_timeout_and_context_survives(cuda_device):
    """A bounded device wait on a flag nothing sets gives up, raises the timeout bit that the
    host reads, and the context keeps working (no fault, no hang)."""
    import time
    from fastergs_gb300 import _lib
    assert _C.device_errors(cuda_device) == 0
    flag = torch.zeros(1, dtype=torch.int32, device=cuda_device)
    t0 = time.perf_counter()
    _lib.call("fgs_selftest_wait", flag.data_ptr(), torch.cuda.current_stream(cuda_device).cuda_stream)
    errs = _C.device_errors(cuda_device)  # synchronises, reads and clears
    assert errs & 1, errs
    assert time.perf_counter() - t0 < 30.0
    assert _C.device_errors(cuda_device) == 0
    s = scenes.scene_c1(P=2000)
    img, radii = render(s, raw_params(s, cuda_device), cuda_device)
    assert torch.isfinite(img).all() and int((radii > 0).sum()) > 0
    assert _C.device_errors(cuda_device) == 0


class _Model:
    """The attributes a backbone's GaussianModel hands the rasterizer (3DGS/scene/gaussian_model.py:
    get_xyz, get_opacity = sigmoid, get_scaling = exp, get_rotation = normalize, _features_dc/_rest)."""

    def __init__(self, scene, dev):
        t = lambda a: torch.nn.Parameter(torch.tensor(np.asarray(a, np.float32), device=dev))
        self._xyz, self._scaling, self._rotation = t(scene.means), t(scene.log_scales), t(scene.quats)
        self._opacity, self._features_dc, self._features_rest = t(scene.opacity_logits), t(scene.dc), t(scene.shs)
        self.active_sh_degree = scene.sh_degree

    get_xyz = property(lambda self: self._xyz)
    get_opacity = property(lambda self: torch.sigmoid(self._opacity))
    get_scaling = property(lambda self: torch.exp(self._scaling))
    get_rotation = property(lambda self: torch.nn.functional.normalize(self._rotation))


def test_reference_import_name_runs_the_backbone_call_sequence(cuda_device):
    # the --fastergs render of 3DGS/gaussian_renderer/render_faster.py:16-66, line for line
    import math
    from diff_gaussian_rasterization_faster import GaussianRasterizationSettings as S, GaussianRasterizer as R
    s = scenes.scene_c2(seed=1, P=20000, width=320, height=208)
    pc = _Model(s, cuda_device)
    cam = s.camera
    t = lambda a: torch.tensor(np.asarray(a, np.float32), device=cuda_device)
    raster_settings = S(image_height=int(cam.height), image_width=int(cam.width), tanfovx=math.tan(cam.fovx * 0.5),
                        tanfovy=math.tan(cam.fovy * 0.5), bg=torch.zeros(3, device=cuda_device), scale_modifier=1.0,
                        viewmatrix=t(cam.viewmatrix), projmatrix=t(cam.projmatrix), sh_degree=pc.active_sh_degree,
                        mult=1.0, campos=t(cam.campos), prefiltered=False, debug=False)
    rasterizer = R(raster_settings=raster_settings)
    dc, shs = pc._features_dc, pc._features_rest
    rendered_image, radii = rasterizer(means3D=pc.get_xyz, dc=dc, shs=shs, opacities=pc.get_opacity,
                                       scales=pc.get_scaling, rotations=pc.get_rotation)
    dL = torch.tensor(scenes.upstream_grad(0, cam.height, cam.width), device=cuda_device)
    (rendered_image * dL).sum().backward()
    # the same frame through the ctypes binding of the C ABI (this package's _C.ops)
    from gpu_util import run_backward, run_forward
    T = dict(means=pc.get_xyz.detach(), scales=pc.get_scaling.detach().contiguous(),
             rotations=pc.get_rotation.detach().contiguous(), opacities=pc.get_opacity.detach().contiguous(),
             dc=dc.detach(), shs=shs.detach())
    fw = run_forward(s, cuda_device, T=T)
    assert torch.equal(radii, fw["radii"])
    assert (rendered_image.detach() - fw["out_color"]).abs().max().item() == 0.0
    g = run_backward(s, fw, dL.cpu().numpy(), cuda_device)
    for name, leaf, ref in (("means", pc._xyz, "dmean3D"), ("dc", pc._features_dc, "ddc"),
                            ("shs", pc._features_rest, "dsh")):
        a = leaf.grad.cpu().numpy().astype(np.float64).reshape(g[ref].shape)
        assert np.abs(a - g[ref]).max() <= 1e-6 * max(np.abs(g[ref]).max(), 1e-30), name
    for leaf in (pc._scaling, pc._rotation, pc._opacity):
        assert leaf.grad is not None and torch.isfinite(leaf.grad).all()


def test_backward_after_a_later_forward_raises(cuda_device):
    # the shared Buffer holds one frame; FB would silently differentiate the second frame's lists
    s = scenes.scene_c1(P=2000)
    p = raw_params(s, cuda_device)
    img1, _ = render(s, p, cuda_device)
    with torch.no_grad():
        render(s, p, cuda_device)
    with pytest.raises(RuntimeError, match="later frame"):
        img1.sum().backward()
    img3, _ = render(s, p, cuda_device)
    img3.sum().backward()  # forward then backward: fine
    assert torch.isfinite(p["means"].grad).all()
