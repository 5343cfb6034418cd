"""Sparse Adam fused into the backward (fgs_preprocess_bwd_adam, fgs_render_batched_bwd_adam).

FB's training step writes every per-Gaussian gradient, lets autograd push the
opacity / scale / rotation gradients through sigmoid / exp / normalize, and
runs SparseGaussianAdam.step(radii > 0, N) over the raw tensors
(FB __init__.py:267-298, adam.cu:9-38).  The fused step does all of it in the
preprocess backward.  Each step here starts both paths from the same
parameters and optimiser state and compares them after one step:

* the unfused masked Adam against the oracle's FP32 restatement of FB's step
  (1e-6 relative: the device contracts b m + (1 - b) g into one FMA and forms
  the step with the hardware square root and reciprocal);
* fused against unfused: Adam moments within 1e-5 of their largest value
  (the rasterizer's gradients are the same kernels' output, summed by float
  atomics in a run-dependent order; the normalize backward is formed in
  another order than autograd's), every fused parameter equal to Adam's
  update on its own moments, untouched rows bit-identical, densification
  statistics within 1e-5;
* the same for the batched path (gradients summed over four cameras,
  stepped where any camera saw the Gaussian) and for a CUDA graph of the
  whole training step (activations + forward + fused backward) replayed
  against the eager sequence.
"""
import numpy as np
import pytest
import torch
import torch.nn.functional as F

import oracle
from fastergs_gb300 import (GaussianRasterizationSettings, GaussianRasterizer, SparseGaussianAdam,
                            _RasterizeGaussians, scenes)
from fastergs_gb300.batched import BatchedRasterizer, CapturedStep, rasterize_batched

pytestmark = pytest.mark.gpu

GROUPS = ("xyz", "f_dc", "f_rest", "opacity", "scaling", "rotation")
LRS = {"xyz": 1.6e-4, "f_dc": 2.5e-3, "f_rest": 2.5e-3 / 20, "opacity": 2.5e-2, "scaling": 5e-3, "rotation": 1e-3}


def _settings(cam, dev, deg, bg=(0.0, 0.0, 0.0)):
    t = lambda a: torch.tensor(np.asarray(a, np.float32), device=dev)
    return GaussianRasterizationSettings(
        image_height=cam.height, image_width=cam.width, tanfovx=cam.tanfovx, tanfovy=cam.tanfovy, bg=t(bg),
        scale_modifier=1.0, viewmatrix=t(cam.viewmatrix), projmatrix=t(cam.projmatrix), sh_degree=deg,
        campos=t(cam.campos), mult=1.0, prefiltered=False, debug=False)


def _model(scene, dev):
    """Raw tensors named and laid out as FasterGS's GaussianModel holds them."""
    t = lambda a: torch.tensor(np.asarray(a, np.float32), device=dev).contiguous().requires_grad_(True)
    q = np.asarray(scene.quats, np.float32) * np.float32(1.7)  # not unit length: the normalize backward matters
    return {"xyz": t(scene.means), "f_dc": t(scene.dc), "f_rest": t(scene.shs), "opacity": t(scene.opacity_logits),
            "scaling": t(scene.log_scales), "rotation": t(q)}


def _optimizer(model):
    return SparseGaussianAdam([{"params": [model[n]], "lr": LRS[n], "name": n} for n in GROUPS], lr=0.0, eps=1e-15)


def _copy(model_src, opt_src, model_dst, opt_dst):
    with torch.no_grad():
        for n in GROUPS:
            model_dst[n].copy_(model_src[n])
            s_src = opt_src.state.get(model_src[n], {})
            if s_src:
                opt_dst.state[model_dst[n]] = {"step": s_src["step"].clone(), "exp_avg": s_src["exp_avg"].clone(),
                                               "exp_avg_sq": s_src["exp_avg_sq"].clone()}


def _inputs(model):
    return dict(means3D=model["xyz"], opacities=torch.sigmoid(model["opacity"]), dc=model["f_dc"],
                shs=model["f_rest"], scales=torch.exp(model["scaling"]), rotations=F.normalize(model["rotation"]))


def _stats(P, dev):
    return dict(xyz_gradient_accum=torch.zeros((P, 1), device=dev), xyz_gradient_accum_abs=torch.zeros((P, 1), device=dev),
                max_radii=torch.zeros(P, device=dev), denom=torch.zeros((P, 1), device=dev))


def _tile_mask(tiles, sizes, bx=16, by=16):
    """Pixel masks (per camera) of the given global tile ids."""
    masks, off = [], 0
    for h, w in sizes:
        gx, gy = (w + bx - 1) // bx, (h + by - 1) // by
        m = np.zeros((h, w), bool)
        for t in tiles:
            if off <= t < off + gx * gy:
                ty, tx = divmod(t - off, gx)
                m[ty * by:(ty + 1) * by, tx * bx:(tx + 1) * bx] = True
        masks.append(m)
        off += gx * gy
    return masks


def _tie_tiles(keys):
    """Tiles whose sorted list holds two equal (tile, depth) keys: their order follows the
    run-dependent emission order, so the upstream gradient is zeroed there."""
    keys = keys.cpu().numpy().view(np.uint64)
    return set(((keys[1:][keys[1:] == keys[:-1]]) >> np.uint64(32)).astype(np.int64).tolist())


def _plain_ties(H, W, dev):
    buf = _RasterizeGaussians.buffer
    K = int(buf.curr_offset[0])
    m = _tile_mask(_tie_tiles(buf.gaussian_keys_sorted[:K]), [(H, W)])[0]
    return torch.tensor(m, device=dev)


def _batched_ties(rast, dev):
    st = rast.state()
    masks = _tile_mask(_tie_tiles(st["keys_sorted"]), rast.sizes, rast.tune.block_x, rast.tune.block_y)
    return torch.cat([torch.tensor(m, device=dev).reshape(1, -1).expand(3, -1).reshape(-1) for m in masks])


def _compare(name, before, unfused, fused, opt_u, opt_f, vis):
    """Moments (which carry the gradients) against the unfused step, within 1e-5 of their largest
    value; every fused parameter against Adam's update on its own moments; rows no camera saw
    untouched.  Parameters are not compared with the unfused ones directly: Adam moves a
    parameter by about lr whatever the size of its gradient, so the last-bit differences of
    near-zero gradients (a quaternion gradient nearly parallel to the quaternion, projected out
    by the normalize backward) show up at full size in the move."""
    N = len(vis)
    for key in ("exp_avg", "exp_avg_sq"):
        mu, mf = opt_u.state[unfused][key], opt_f.state[fused][key]
        den = max(float(mu.abs().max()), 1e-30)
        assert float((mf - mu).abs().max()) / den <= 1e-5, (name, key)
    st = opt_f.state[fused]
    step = st["step"]
    assert float(opt_u.state[unfused]["step"]) == float(step)
    lr = [g["lr"] for g in opt_f.param_groups if g["params"][0] is fused][0]
    lr_t = float(lr * (1 - 0.999 ** step) ** 0.5 / (1 - 0.9 ** step))
    want = before + (-lr_t * st["exp_avg"]) / (st["exp_avg_sq"].sqrt() + 1e-15)
    pf = fused.detach()
    v = vis.reshape(N, 1)
    want = torch.where(v, want.reshape(N, -1), before.reshape(N, -1)).reshape(before.shape)
    err = float((pf - want).abs().max())
    move = float((want - before).abs().max())
    # the device forms the step with the hardware square root and reciprocal (~2^-22 relative)
    assert err <= 4e-6 * move + 1e-7 * float(before.abs().max()), (name, err, move)
    hidden = ~vis
    assert torch.equal(pf.reshape(N, -1)[hidden], before.reshape(N, -1)[hidden]), name
    for key in ("exp_avg", "exp_avg_sq"):
        prev = opt_u.state[unfused][key]  # rows no camera saw keep their previous moments in both
        assert torch.equal(st[key].reshape(N, -1)[hidden], prev.reshape(N, -1)[hidden]), (name, key)


@pytest.mark.parametrize("which", ["c1", "c2_small"])
def test_fused_step_matches_unfused(cuda_device, which):
    dev = cuda_device
    s = scenes.scene_c1() if which == "c1" else scenes.scene_c2(P=20000, width=320, height=208)
    P = s.means.shape[0]
    rs = _settings(s.camera, dev, s.sh_degree)
    dL = torch.tensor(scenes.upstream_grad(3, s.camera.height, s.camera.width), device=dev)
    mu, mf = _model(s, dev), _model(s, dev)
    ou, of = _optimizer(mu), _optimizer(mf)
    for step in range(1, 4):
        _copy(mu, ou, mf, of)
        before = {n: mu[n].detach().clone() for n in GROUPS}
        # unfused: FB's step (autograd through the activations, then SparseGaussianAdam.step)
        su, sf = _stats(P, dev), _stats(P, dev)
        img, radii = GaussianRasterizer(rs)(**_inputs(mu), **su)
        ties = _plain_ties(s.camera.height, s.camera.width, dev)
        dLm = dL * ~ties
        (img * dLm).sum().backward()
        vis = radii > 0
        grads = {n: mu[n].grad.detach().clone() for n in GROUPS}
        states = {n: {k: v.clone() for k, v in ou.state[mu[n]].items()} if mu[n] in ou.state else None
                  for n in GROUPS}
        ou.step(vis, P)
        ou.zero_grad(set_to_none=True)
        # the unfused step is FB's step (oracle restatement, FP32)
        for n in GROUPS:
            st = states[n]
            m0 = st["exp_avg"].cpu().numpy() if st else np.zeros(tuple(mu[n].shape), np.float32)
            v0 = st["exp_avg_sq"].cpu().numpy() if st else np.zeros(tuple(mu[n].shape), np.float32)
            p_ref, m_ref, v_ref = oracle.sparse_adam(before[n].cpu().numpy(), grads[n].cpu().numpy(), m0, v0,
                                                     vis.cpu().numpy(), LRS[n], step, 1e-15)
            for got, ref in ((mu[n].detach(), p_ref), (ou.state[mu[n]]["exp_avg"], m_ref),
                             (ou.state[mu[n]]["exp_avg_sq"], v_ref)):
                got = got.cpu().numpy()
                den = max(float(np.abs(ref).max()), 1e-30)
                assert float(np.abs(got - ref).max()) / den <= 1e-6, n
        # fused: the same step inside the backward
        img_f, radii_f = GaussianRasterizer(rs)(**_inputs(mf), **sf, adam=of)
        assert torch.equal(radii_f, radii)
        assert torch.equal(_plain_ties(s.camera.height, s.camera.width, dev), ties)
        assert torch.equal(img_f * ~ties, img.detach() * ~ties)
        (img_f * dLm).sum().backward()
        for n in GROUPS:
            assert mf[n].grad is None, n  # no gradient reached memory
            _compare(n, before[n], mu[n], mf[n], ou, of, vis.cpu().to(dev))
        for k in su:  # float atomics in the composite backward: equal up to summation order
            torch.testing.assert_close(sf[k], su[k], rtol=1e-5, atol=1e-7)


def test_fused_matches_oracle_activation_gradients(cuda_device):
    """The in-kernel activation backward against FP64 sigmoid / exp / normalize derivatives,
    read back from the fused step's first moment (m = (1 - b1) g at step 1)."""
    dev = cuda_device
    s = scenes.scene_c1()
    P = s.means.shape[0]
    rs = _settings(s.camera, dev, s.sh_degree)
    dL = torch.tensor(scenes.upstream_grad(5, s.camera.height, s.camera.width), device=dev)
    ma, mf = _model(s, dev), _model(s, dev)
    of = _optimizer(mf)
    # dL/d(activated) from the plain backward
    inp = _inputs(ma)
    for k in ("opacities", "scales", "rotations"):
        inp[k].retain_grad()
    img, radii = GaussianRasterizer(rs)(**inp)
    dL = dL * ~_plain_ties(s.camera.height, s.camera.width, dev)
    (img * dL).sum().backward()
    img_f, _ = GaussianRasterizer(rs)(**_inputs(mf), adam=of)
    (img_f * dL).sum().backward()
    vis = (radii > 0).cpu().numpy()
    for name, act, key in (("opacity", "sigmoid", "opacities"), ("scaling", "exp", "scales"),
                           ("rotation", "normalize", "rotations")):
        g_ref = oracle.activation_grad(act, ma[name].detach().cpu().numpy(), inp[key].grad.cpu().numpy())
        g_dev = of.state[mf[name]]["exp_avg"].cpu().numpy() / np.float32(0.1)
        den = max(float(np.abs(g_ref[vis]).max()), 1e-30)
        assert float(np.abs(g_dev[vis] - g_ref[vis]).max()) / den <= 1e-5, name
        assert not np.any(g_dev[~vis]), name


def test_fused_argument_checks(cuda_device):
    dev = cuda_device
    s = scenes.scene_c1(P=500)
    rs = _settings(s.camera, dev, s.sh_degree)
    m = _model(s, dev)
    opt = _optimizer(m)
    inp = _inputs(m)
    other = m["xyz"].detach().clone().requires_grad_(True)
    with pytest.raises(ValueError, match="xyz"):
        GaussianRasterizer(rs)(**dict(inp, means3D=other), adam=opt)
    unnamed = SparseGaussianAdam([m["xyz"]], lr=0.01, eps=1e-15)
    with pytest.raises(ValueError, match="named"):
        GaussianRasterizer(rs)(**inp, adam=unnamed)


def _batch_cameras(dev, deg):
    import math
    cams = []
    for k, (w, h) in enumerate([(320, 208), (257, 131), (401, 300), (64, 48)]):
        th = 2 * math.pi * k / 4 + 0.3
        eye = (8 * math.sin(th), 0.5, 7.0 - 8 * math.cos(th))
        cams.append(scenes.make_camera(w, h, 55.0, eye=eye, target=(0.0, 0.0, 7.0)))
    return [_settings(c, dev, deg) for c in cams]


def test_batched_fused_step_matches_unfused(cuda_device):
    dev = cuda_device
    s = scenes.scene_c2(P=20000, width=320, height=208)
    P = s.means.shape[0]
    settings = _batch_cameras(dev, s.sh_degree)
    mu, mf = _model(s, dev), _model(s, dev)
    ou, of = _optimizer(mu), _optimizer(mf)
    rast = BatchedRasterizer(settings, P)
    inp = _inputs(mu)
    rast.fit(inp["means3D"].detach(), inp["opacities"].detach(), inp["dc"].detach(), inp["shs"].detach(), None,
             inp["scales"].detach(), inp["rotations"].detach(), None, s.sh_degree)
    rng = torch.Generator(device="cpu").manual_seed(9)
    dL = torch.randn(rast.out_color.numel(), generator=rng).to(dev)
    for step in range(1, 3):
        _copy(mu, ou, mf, of)
        before = {n: mu[n].detach().clone() for n in GROUPS}
        su, sf = _stats(P, dev), _stats(P, dev)
        imgs, radii = rasterize_batched(rast, **_inputs(mu), sh_degree=s.sh_degree, **su)
        dLm = dL * ~_batched_ties(rast, dev)
        flat = torch.cat([im.reshape(-1) for im in imgs])
        (flat * dLm).sum().backward()
        vis = (radii > 0).any(0)
        ou.step(vis, P)
        ou.zero_grad(set_to_none=True)
        inp_f = {k: v.detach() for k, v in _inputs(mf).items()}
        rast.forward(inp_f["means3D"], inp_f["opacities"], inp_f["dc"], inp_f["shs"], None, inp_f["scales"],
                     inp_f["rotations"], None, s.sh_degree)
        fused, _keep, _ = of._fused_args(P, dev)
        assert torch.equal(dL * ~_batched_ties(rast, dev), dLm)
        rast.backward_adam(dLm, inp_f["means3D"], inp_f["shs"], inp_f["opacities"], inp_f["scales"],
                           inp_f["rotations"], s.sh_degree, fused, **sf)
        torch.cuda.synchronize(dev)
        for n in GROUPS:
            _compare(n, before[n], mu[n], mf[n], ou, of, vis)
        for k in su:
            torch.testing.assert_close(sf[k], su[k], rtol=1e-5, atol=1e-7)


def test_captured_training_step_matches_eager(cuda_device):
    dev = cuda_device
    s = scenes.scene_c2(P=20000, width=320, height=208)
    P = s.means.shape[0]
    settings = _batch_cameras(dev, s.sh_degree)
    mg, me = _model(s, dev), _model(s, dev)
    og, oe = _optimizer(mg), _optimizer(me)
    rg, re = BatchedRasterizer(settings, P), BatchedRasterizer(settings, P)
    inp = {k: v.detach() for k, v in _inputs(mg).items()}
    for r in (rg, re):
        r.fit(inp["means3D"], inp["opacities"], inp["dc"], inp["shs"], None, inp["scales"], inp["rotations"], None,
              s.sh_degree)
    rng = torch.Generator(device="cpu").manual_seed(4)
    dL0 = torch.randn(rg.out_color.numel(), generator=rng).to(dev)
    dL = dL0.clone()  # the graph's static upstream gradient
    sg, se = _stats(P, dev), _stats(P, dev)
    step = CapturedStep(rg, None, dL, sh_degree=s.sh_degree, stats=sg, adam=og)
    for t in range(1, 4):
        _copy(mg, og, me, oe)
        before = {n: mg[n].detach().clone() for n in GROUPS}
        inp_e = {k: v.detach() for k, v in _inputs(me).items()}
        re.forward(inp_e["means3D"], inp_e["opacities"], inp_e["dc"], inp_e["shs"], None, inp_e["scales"],
                   inp_e["rotations"], None, s.sh_degree)
        dL.copy_(dL0 * ~_batched_ties(re, dev))  # same keys in both frames, so the same tie tiles
        step.replay()
        rg.status()
        assert torch.equal(_batched_ties(rg, dev), _batched_ties(re, dev))
        fused, _keep, _ = oe._fused_args(P, dev)
        re.backward_adam(dL, inp_e["means3D"], inp_e["shs"], inp_e["opacities"], inp_e["scales"],
                         inp_e["rotations"], s.sh_degree, fused, **se)
        torch.cuda.synchronize(dev)
        vis = (re.radii > 0).any(0)
        assert torch.equal(rg.radii, re.radii)
        for n in GROUPS:
            _compare(n, before[n], me[n], mg[n], oe, og, vis)
    for k in sg:
        torch.testing.assert_close(sg[k], se[k], rtol=1e-5, atol=1e-7)
