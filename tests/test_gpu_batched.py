"""Batched multi-camera path (fgs_render_batched_fwd/bwd, fastergs_gb300.batched).

The batched path runs the same kernels as the plain path over a table of
cameras, so per camera it must reproduce the plain path: identical radii,
images equal up to the order of equal (tile, depth) keys (1e-6), gradients
summed over cameras within 1e-4 relative of the per-camera sum (the float
reductions into the gradient records run in a different order, and a
Gaussian whose per-pixel conic terms cancel amplifies that rounding).  For launch configurations the plain Python API does not
expose (bucket 16/32/64, 8x32 and 32x8 tiles, packet 2/8) every camera is
checked against the oracle replaying the device's own records and lists
(1e-5 max-abs), and the global sort is checked bit-exact.
"""
import math

import numpy as np
import pytest
import torch

import oracle
from fastergs_gb300 import GaussianRasterizationSettings, GaussianRasterizer, _C, scenes
from fastergs_gb300.batched import BatchedRasterizer, BatchOverflow, CapturedStep, TuneConfig, rasterize_batched
from gpu_util import tensors

pytestmark = pytest.mark.gpu

SIZES = [(320, 208), (257, 131), (64, 48), (401, 300)]  # (W, H), ragged on purpose
CENTER = (0.0, 0.0, 7.0)


def _cameras(sizes=SIZES, seed=0, radius=8.0):
    rng = np.random.default_rng(seed + 77)
    cams = []
    for k, (w, h) in enumerate(sizes):
        th = 2 * math.pi * k / len(sizes) + 0.3
        eye = (CENTER[0] + radius * math.sin(th), CENTER[1] + 0.5, CENTER[2] - radius * math.cos(th))
        cams.append(scenes.make_camera(w, h, float(rng.uniform(40.0, 70.0)), eye=eye, target=CENTER))
    return cams


def _settings(cam, dev, bg=(0.0, 0.0, 0.0), sh_degree=3, smod=1.0, mult=1.0):
    f = lambda a: torch.tensor(np.asarray(a, np.float32), device=dev)
    return GaussianRasterizationSettings(
        image_height=cam.height, image_width=cam.width, tanfovx=cam.tanfovx, tanfovy=cam.tanfovy, bg=f(bg),
        scale_modifier=smod, viewmatrix=f(cam.viewmatrix), projmatrix=f(cam.projmatrix), sh_degree=sh_degree,
        campos=f(cam.campos), mult=mult, prefiltered=False, debug=False)


def _scene(P=20000, seed=0):
    return scenes.scene_c2(seed=seed, P=P, width=320, height=208)


def _bgs(n):
    return [(0.1 * k, 0.05, 0.2 - 0.03 * k) for k in range(n)]


def _rel(a, b):
    den = max(float(np.abs(b).max()), 1e-30)
    return float(np.abs(a - b).max()) / den


@pytest.fixture(scope="module")
def setup(cuda_device):
    s = _scene()
    T = tensors(s, cuda_device)
    cams = _cameras()
    sets = [_settings(c, cuda_device, bg) for c, bg in zip(cams, _bgs(len(cams)))]
    return s, T, cams, sets


def _plain(T, st, dL=None, stats=None):
    """One plain-path camera through the public API; returns image, radii, grads."""
    leaves = {k: T[k].clone().requires_grad_(True) for k in ("means", "opacities", "dc", "shs", "scales",
                                                              "rotations")}
    r = GaussianRasterizer(st)
    kw = {}
    if stats is not None:
        kw = dict(xyz_gradient_accum=stats[0], xyz_gradient_accum_abs=stats[1], max_radii=stats[2], denom=stats[3])
    img, radii = r(means3D=leaves["means"], opacities=leaves["opacities"], dc=leaves["dc"], shs=leaves["shs"],
                   scales=leaves["scales"], rotations=leaves["rotations"], **kw)
    grads = None
    if dL is not None:
        torch.autograd.backward(img, grad_tensors=dL)
        grads = {k: v.grad.detach().clone() for k, v in leaves.items()}
    return img.detach().clone(), radii.clone(), grads


def _batched(T, sets, tune=None, dL=None, stats=None):
    rast = BatchedRasterizer(sets, T["means"].shape[0], tune=tune)
    rast.fit(T["means"], T["opacities"], T["dc"], T["shs"], None, T["scales"], T["rotations"], None, 3)
    rast.forward(T["means"], T["opacities"], T["dc"], T["shs"], None, T["scales"], T["rotations"], None, 3)
    g = None
    if dL is not None:
        kw = {}
        if stats is not None:
            kw = dict(xyz_gradient_accum=stats[0], xyz_gradient_accum_abs=stats[1], max_radii=stats[2],
                      denom=stats[3])
        g = rast.backward(dL, T["means"], T["dc"], T["shs"], T["scales"], T["rotations"], 3, **kw)
    torch.cuda.synchronize()
    assert _C.device_errors(T["means"].device) == 0
    return rast, g


def _tie_masks(rast):
    """Per camera, the pixels of tiles whose sorted list holds two equal keys
    (same tile, bit-identical depth).  Their relative order follows the
    emission order, which atomics make run-dependent in FB and here alike."""
    keys = rast.state()["keys_sorted"].numpy().view(np.uint64)
    tie_tiles = set(((keys[1:][keys[1:] == keys[:-1]]) >> np.uint64(32)).astype(np.int64).tolist())
    bx, by = rast.tune.block_x, rast.tune.block_y
    masks, off = [], 0
    for h, w in rast.sizes:
        gx, gy = (w + bx - 1) // bx, (h + by - 1) // by
        m = np.zeros((h, w), bool)
        for t in tie_tiles:
            if off <= t < off + gx * gy:
                ty, tx = divmod(t - off, gx)
                m[ty * by:(ty + 1) * by, tx * bx:(tx + 1) * bx] = True
        masks.append(m)
        off += gx * gy
    return masks


def test_batched_forward_matches_plain_per_camera(setup):
    s, T, cams, sets = setup
    rast, _ = _batched(T, sets)
    pairs, buckets = rast.status()
    assert pairs > 0 and buckets > 0
    imgs = rast.images()
    ties = _tie_masks(rast)
    for k, st in enumerate(sets):
        img, radii, _ = _plain(T, st)
        assert torch.equal(rast.radii[k], radii), k
        d = (imgs[k] - img).abs().amax(0).cpu().numpy()
        err = d[~ties[k]].max()
        assert err <= 1e-6, (k, err)


def test_batched_backward_matches_sum_of_plain(setup):
    s, T, cams, sets = setup
    dev = T["means"].device
    probe, _ = _batched(T, sets)
    ties = _tie_masks(probe)
    del probe
    dLs = []
    for k, st in enumerate(sets):
        dL = scenes.upstream_grad(10 + k, st.image_height, st.image_width)
        dL[:, ties[k]] = 0.0  # the order of equal keys is run-dependent
        dLs.append(torch.tensor(dL, device=dev))
    P = s.P
    st_plain = [torch.zeros((P, 1), device=dev) for _ in range(4)]
    acc = None
    for st, dL in zip(sets, dLs):
        _, _, g = _plain(T, st, dL, st_plain)
        acc = g if acc is None else {k: acc[k] + g[k] for k in acc}
    st_b = [torch.zeros((P, 1), device=dev) for _ in range(4)]
    flat = torch.cat([d.reshape(-1) for d in dLs])
    rast, g = _batched(T, sets, dL=flat, stats=st_b)
    pairs = {"means": "means3D", "opacities": "opacities", "dc": "dc", "shs": "shs", "scales": "scales",
             "rotations": "rotations"}
    for kp, kb in pairs.items():
        e = _rel(g[kb].cpu().numpy().astype(np.float64), acc[kp].cpu().numpy().astype(np.float64))
        assert e <= 1e-4, (kp, e)
    for a, b, name in zip(st_b, st_plain, ["accum", "accum_abs", "max_radii", "denom"]):
        a, b = a.cpu().numpy().astype(np.float64), b.cpu().numpy().astype(np.float64)
        if name in ("max_radii", "denom"):
            np.testing.assert_array_equal(a, b)
        else:
            assert _rel(a, b) <= 1e-5, name


def _view_replay(s, T, rast, state, k, bg, tune):
    """Oracle compositing of camera k from the device's records and sorted lists."""
    P = s.P
    h, w = rast.sizes[k]
    gx, gy = (w + tune.block_x - 1) // tune.block_x, (h + tune.block_y - 1) // tune.block_y
    tile_off = sum(((ww + tune.block_x - 1) // tune.block_x) * ((hh + tune.block_y - 1) // tune.block_y)
                   for hh, ww in rast.sizes[:k])
    keys = state["keys_sorted"].numpy().view(np.uint64)
    vals = state["vals_sorted"].numpy().view(np.uint32)
    tiles = (keys >> np.uint64(32)).astype(np.int64)
    lo, hi = np.searchsorted(tiles, [tile_off, tile_off + gx * gy])
    ids = vals[lo:hi].astype(np.int64) - k * P
    assert ids.min(initial=0) >= 0 and ids.max(initial=0) < P
    rng = state["ranges"].numpy()[tile_off:tile_off + gx * gy].astype(np.int64)
    nonempty = rng[:, 1] > rng[:, 0]
    rng[nonempty] -= lo
    rng[~nonempty] = 0
    m, sc, rot, op, dc, shs = [np.asarray(a, np.float64) for a in s.activated()]
    o = oracle.Oracle()
    o.set_scene(m, op, sc, rot, rast_cam(rast, k), dc=dc, shs=shs, sh_degree=s.sh_degree,
                block=(tune.block_x, tune.block_y))
    rec = state["records"][k * P:(k + 1) * P].numpy()
    recd = rec.astype(np.float64)
    recd[:, 12:16] = rec.view(np.int32)[:, 12:16]
    radii = rast.radii[k].cpu().numpy()
    valid = (radii > 0) | np.isin(np.arange(P), ids)
    o.set_records(recd, radii, valid)
    o.set_lists(ids.astype(np.uint32), rng.astype(np.uint32))
    o.render(bg=bg, bucket_size=tune.bucket_size, eps_alpha=1e-5, eps_T=1e-5)
    return o


_CAMS = {}


def rast_cam(rast, k):
    return _CAMS[id(rast)][k]


TUNES = [TuneConfig(32, 8, 32, 2), TuneConfig(64, 32, 8, 8), TuneConfig(16, 16, 16, 1),
         TuneConfig(128, 16, 16, 4),  # FB's bucket: composited as two sub-buckets, stop at the full bucket
         # short fold chains: most tiles' later buckets go through the pixel-parallel merge
         TuneConfig(16, 16, 16, 4, chain=1), TuneConfig(32, 8, 32, 2, chain=2)]


@pytest.mark.parametrize("tune", TUNES, ids=lambda t: f"b{t.bucket_size}_{t.block_x}x{t.block_y}_p{t.packet}_c{t.chain}")
def test_tuned_configs_match_oracle_replay(setup, tune):
    s, T, cams, sets = setup
    rast, _ = _batched(T, sets, tune=tune)
    _CAMS[id(rast)] = cams
    state = rast.state()
    K = state["pairs"]
    assert K <= rast.pair_capacity
    # global sort: bit-exact stable sort of the emitted pairs
    ku = state["keys_unsorted"].numpy().view(np.uint64)
    vu = state["vals_unsorted"].numpy().view(np.uint32)
    order = np.argsort(ku, kind="stable")
    np.testing.assert_array_equal(state["keys_sorted"].numpy().view(np.uint64), ku[order])
    np.testing.assert_array_equal(state["vals_sorted"].numpy().view(np.uint32), vu[order])
    # ranges bit-exact
    tiles = (ku[order] >> np.uint64(32)).astype(np.int64)
    T_all = state["ranges"].shape[0]
    starts = np.searchsorted(tiles, np.arange(T_all), side="left")
    ends = np.searchsorted(tiles, np.arange(T_all), side="right")
    ref = np.stack([np.where(ends > starts, starts, 0), np.where(ends > starts, ends, 0)], 1)
    np.testing.assert_array_equal(state["ranges"].numpy().astype(np.int64), ref)
    imgs = rast.images()
    for k, bg in enumerate(_bgs(len(sets))):
        im = _view_replay(s, T, rast, state, k, bg, tune).image()
        ok = ~im["ambiguous"]
        assert ok.mean() > 0.99
        g = imgs[k].cpu().numpy().astype(np.float64)
        err = np.abs(g - im["out_color"])[:, ok].max()
        assert err <= 1e-5, (k, err)


def _flat_mask(rast, masks):
    return torch.tensor(np.concatenate([np.broadcast_to(m, (3,) + m.shape).reshape(-1) for m in masks]),
                        device=rast.device)


def test_captured_step_replays_and_follows_parameter_updates(setup):
    s, T, cams, sets = setup
    dev = T["means"].device
    params = {"means3D": T["means"].clone(), "opacities": T["opacities"].clone(), "dc": T["dc"].clone(),
              "shs": T["shs"].clone(), "scales": T["scales"].clone(), "rotations": T["rotations"].clone()}
    rast = BatchedRasterizer(sets, s.P)
    rast.fit(params["means3D"], params["opacities"], params["dc"], params["shs"], None, params["scales"],
             params["rotations"], None, 3)
    tie = _flat_mask(rast, _tie_masks(rast))  # pixels whose equal-key order is run-dependent
    dL = torch.randn(rast.out_color.numel(), device=dev, generator=torch.Generator(device=dev).manual_seed(3))
    dL[tie] = 0.0
    step = CapturedStep(rast, params, dL, sh_degree=3)
    step.replay()
    torch.cuda.synchronize()
    img1 = rast.out_color.clone()
    g1 = {k: v.clone() for k, v in step.grads.items()}
    # eager reference on the same parameters
    rast.forward(params["means3D"], params["opacities"], params["dc"], params["shs"], None, params["scales"],
                 params["rotations"], None, 3)
    ge = rast.backward(dL, params["means3D"], params["dc"], params["shs"], params["scales"], params["rotations"], 3)
    torch.cuda.synchronize()
    assert (rast.out_color - img1).abs()[~tie].max().item() <= 1e-6
    for k in ("means3D", "opacities", "dc", "shs", "scales", "rotations"):
        assert _rel(g1[k].cpu().numpy(), ge[k].cpu().numpy()) <= 1e-4, k
    # move the scene in place; the graph must see the new values
    params["means3D"].add_(torch.tensor([0.05, -0.02, 0.0], device=dev))
    step.replay()
    torch.cuda.synchronize()
    img2 = rast.out_color.clone()
    tie2 = _flat_mask(rast, _tie_masks(rast))
    assert (img2 - img1).abs().max().item() > 1e-3
    rast.forward(params["means3D"], params["opacities"], params["dc"], params["shs"], None, params["scales"],
                 params["rotations"], None, 3)
    torch.cuda.synchronize()
    assert (rast.out_color - img2).abs()[~tie2].max().item() <= 1e-6
    rast.status()  # no overflow
    assert _C.device_errors(dev) == 0


def test_overflow_is_reported_not_written(setup):
    s, T, cams, sets = setup
    dev = T["means"].device
    rast = BatchedRasterizer(sets, s.P, pair_capacity=1000)
    rast.forward(T["means"], T["opacities"], T["dc"], T["shs"], None, T["scales"], T["rotations"], None, 3)
    with pytest.raises(BatchOverflow) as ei:
        rast.status()
    assert ei.value.pairs > 1000
    assert _C.device_errors(dev) != 0  # capacity bit latched, and cleared by the read
    need = rast.fit(T["means"], T["opacities"], T["dc"], T["shs"], None, T["scales"], T["rotations"], None, 3)
    assert need == ei.value.pairs
    rast.forward(T["means"], T["opacities"], T["dc"], T["shs"], None, T["scales"], T["rotations"], None, 3)
    assert rast.status()[0] == need
    assert _C.device_errors(dev) == 0


def test_captured_step_reports_overflow_without_synchronising(setup):
    s, T, cams, sets = setup
    dev = T["means"].device
    rast = BatchedRasterizer(sets, s.P, pair_capacity=1000)
    params = {"means3D": T["means"], "opacities": T["opacities"], "dc": T["dc"], "shs": T["shs"],
              "scales": T["scales"], "rotations": T["rotations"]}
    dL = torch.zeros(rast.out_color.numel(), device=dev)
    step = CapturedStep(rast, params, dL, sh_degree=3, with_backward=False)
    step.replay()  # nothing has completed yet that could report
    with pytest.raises(BatchOverflow) as ei:
        step.check()
    assert ei.value.pairs > 1000 and ei.value.capacity == 1000
    with pytest.raises(BatchOverflow):  # the next replay raises before it launches
        step.replay()
    assert _C.device_errors(dev) != 0  # capacity bit latched by the kernels, cleared by the read
    # a fitted workspace replays without a report
    rast.fit(T["means"], T["opacities"], T["dc"], T["shs"], None, T["scales"], T["rotations"], None, 3)
    step = CapturedStep(rast, params, dL, sh_degree=3, with_backward=False)
    step.replay()
    step.replay()
    step.check()
    assert _C.device_errors(dev) == 0


def test_autograd_batched_matches_direct_backward(setup):
    s, T, cams, sets = setup
    dev = T["means"].device
    rast = BatchedRasterizer(sets, s.P)
    rast.fit(T["means"], T["opacities"], T["dc"], T["shs"], None, T["scales"], T["rotations"], None, 3)
    leaves = {k: T[k].clone().requires_grad_(True) for k in ("means", "opacities", "dc", "shs", "scales",
                                                              "rotations")}
    imgs, radii = rasterize_batched(rast, leaves["means"], leaves["opacities"], dc=leaves["dc"], shs=leaves["shs"],
                                    scales=leaves["scales"], rotations=leaves["rotations"], sh_degree=3)
    assert len(imgs) == len(sets) and radii.shape == (len(sets), s.P)
    loss = sum((im * (k + 1)).sum() for k, im in enumerate(imgs))
    loss.backward()
    dL = torch.cat([torch.full((3 * h * w,), float(k + 1), device=dev) for k, (h, w) in enumerate(rast.sizes)])
    rast.forward(T["means"], T["opacities"], T["dc"], T["shs"], None, T["scales"], T["rotations"], None, 3)
    g = rast.backward(dL, T["means"], T["dc"], T["shs"], T["scales"], T["rotations"], 3)
    torch.cuda.synchronize()
    for kp, kb in {"means": "means3D", "opacities": "opacities", "scales": "scales", "rotations": "rotations",
                   "dc": "dc", "shs": "shs"}.items():
        assert _rel(leaves[kp].grad.cpu().numpy(), g[kb].cpu().numpy()) <= 1e-5, kp


@pytest.mark.parametrize("tune", TUNES[:2] + TUNES[-1:],
                         ids=lambda t: f"b{t.bucket_size}_{t.block_x}x{t.block_y}_p{t.packet}_c{t.chain}")
def test_tuned_backward_matches_oracle_replay(setup, tune):
    """Gradients summed over cameras against the oracle's per-camera replay
    backward (dL zeroed at ambiguous pixels), 1e-4 relative."""
    s, T, cams, sets = setup
    dev = T["means"].device
    rast, _ = _batched(T, sets, tune=tune)
    _CAMS[id(rast)] = cams
    state = rast.state()
    dLs, ref = [], {}
    for k, bg in enumerate(_bgs(len(sets))):
        o = _view_replay(s, T, rast, state, k, bg, tune)
        h, w = rast.sizes[k]
        dL = scenes.upstream_grad(20 + k, h, w)
        dL[:, o.image()["ambiguous"]] = 0.0
        dLs.append(dL)
        r = o.backward(dL.astype(np.float64))
        for key in ("dmean3D", "dopacity", "ddc", "dsh", "dscale", "drot"):
            ref[key] = r[key] if key not in ref else ref[key] + r[key]
    flat = torch.tensor(np.concatenate([d.reshape(-1) for d in dLs]), device=dev)
    g = rast.backward(flat, T["means"], T["dc"], T["shs"], T["scales"], T["rotations"], 3)
    torch.cuda.synchronize()
    names = {"dmean3D": "means3D", "dopacity": "opacities", "ddc": "dc", "dsh": "shs", "dscale": "scales",
             "drot": "rotations"}
    errs = {}
    for key, gk in names.items():
        a = g[gk].cpu().numpy().astype(np.float64).reshape(s.P, -1)
        b = ref[key].reshape(s.P, -1)
        errs[key] = _rel(a, b)
    assert max(errs.values()) <= 1e-4, errs


@pytest.mark.parametrize("tune", [TuneConfig(128, 16, 16, 4, True), TuneConfig(32, 8, 32, 2, True)],
                         ids=["b128_16x16", "b32_8x32"])
def test_recompute_mode_matches_store_mode(setup, tune):
    """Recompute mode keeps one running prefix per tile and rebuilds every
    bucket's prefix in the backward: the same images (the forward folds the
    same values) and the same gradients up to the order of float reductions,
    from a workspace smaller by ~4 KB per bucket."""
    s, T, cams, sets = setup
    dev = T["means"].device
    store_cfg = TuneConfig(tune.bucket_size, tune.block_x, tune.block_y, tune.packet, False)
    r_store, _ = _batched(T, sets, tune=store_cfg)
    ties = _flat_mask(r_store, _tie_masks(r_store))
    dL = torch.randn(r_store.out_color.numel(), device=dev, generator=torch.Generator(device=dev).manual_seed(5))
    dL[ties] = 0.0
    st = [torch.zeros((s.P, 1), device=dev) for _ in range(4)]
    rr = [torch.zeros((s.P, 1), device=dev) for _ in range(4)]
    kw = lambda x: dict(xyz_gradient_accum=x[0], xyz_gradient_accum_abs=x[1], max_radii=x[2], denom=x[3])
    g_store = r_store.backward(dL, T["means"], T["dc"], T["shs"], T["scales"], T["rotations"], 3, **kw(st))
    img_store = r_store.out_color.clone()
    r_rec, _ = _batched(T, sets, tune=tune)
    assert r_rec.workspace.numel() < r_store.workspace.numel()
    g_rec = r_rec.backward(dL, T["means"], T["dc"], T["shs"], T["scales"], T["rotations"], 3, **kw(rr))
    torch.cuda.synchronize()
    assert _C.device_errors(dev) == 0
    assert (r_rec.out_color - img_store).abs()[~ties].max().item() == 0.0
    for k in ("means3D", "opacities", "dc", "shs", "scales", "rotations"):
        assert _rel(g_rec[k].cpu().numpy(), g_store[k].cpu().numpy()) <= 1e-5, k
    for a, b in zip(rr, st):
        assert _rel(a.cpu().numpy(), b.cpu().numpy()) <= 1e-5


def test_batched_colours_culling_and_per_camera_settings(cuda_device):
    """Precomputed colours, a culling mask and a different scale modifier and
    mult per camera: every camera must match the drop-in path with the same
    settings, and the colour gradient must be the per-camera sum."""
    dev = cuda_device
    s = _scene(P=12000, seed=3)
    T = tensors(s, dev)
    cams = _cameras(sizes=[(200, 136), (97, 61), (256, 256)], seed=5)
    smods, mults = [0.8, 1.0, 1.3], [1.0, 1.4, 0.7]
    sets = [_settings(c, dev, bg, sh_degree=0, smod=sm, mult=mu)
            for c, bg, sm, mu in zip(cams, _bgs(3), smods, mults)]
    rng = np.random.default_rng(9)
    colors = torch.tensor(rng.uniform(0.0, 1.5, size=(s.P, 3)).astype(np.float32), device=dev)
    cull = torch.tensor(rng.random(s.P) < 0.2, device=dev)
    dLs = [torch.tensor(scenes.upstream_grad(40 + k, st.image_height, st.image_width), device=dev)
           for k, st in enumerate(sets)]
    rast = BatchedRasterizer(sets, s.P)
    rast.fit(T["means"], T["opacities"], None, None, colors, T["scales"], T["rotations"], cull, 0)
    rast.forward(T["means"], T["opacities"], None, None, colors, T["scales"], T["rotations"], cull, 0)
    ties = _tie_masks(rast)
    for k in range(3):
        dLs[k][:, torch.tensor(ties[k], device=dev)] = 0.0
    g = rast.backward(torch.cat([d.reshape(-1) for d in dLs]), T["means"], None, None, T["scales"], T["rotations"], 0)
    torch.cuda.synchronize()
    assert _C.device_errors(dev) == 0
    imgs = rast.images()
    acc = None
    for k, st in enumerate(sets):
        leaves = {"means": T["means"].clone().requires_grad_(True), "colors": colors.clone().requires_grad_(True),
                  "opacities": T["opacities"].clone().requires_grad_(True)}
        img, radii = GaussianRasterizer(st)(means3D=leaves["means"], opacities=leaves["opacities"],
                                            colors_precomp=leaves["colors"], scales=T["scales"],
                                            rotations=T["rotations"], culling=cull)
        assert torch.equal(rast.radii[k], radii), k
        assert (radii[cull] == 0).all()
        d = (imgs[k] - img.detach()).abs().amax(0).cpu().numpy()
        assert d[~ties[k]].max(initial=0.0) <= 1e-6, k
        torch.autograd.backward(img, grad_tensors=dLs[k])
        gk = {n: v.grad.detach().clone() for n, v in leaves.items()}
        acc = gk if acc is None else {n: acc[n] + gk[n] for n in acc}
    assert _rel(g["colors"].cpu().numpy(), acc["colors"].cpu().numpy()) <= 1e-4
    assert _rel(g["means3D"].cpu().numpy(), acc["means"].cpu().numpy()) <= 1e-4
    assert _rel(g["opacities"].cpu().numpy(), acc["opacities"].cpu().numpy()) <= 1e-4


def test_batched_many_tiny_and_ragged_cameras(cuda_device):
    """32 cameras (the most one batch takes), down to 1x1 pixel images."""
    dev = cuda_device
    s = _scene(P=5000, seed=4)
    T = tensors(s, dev)
    sizes = [(1, 1), (17, 3), (5, 40), (33, 17), (64, 64), (15, 16), (16, 15), (129, 7)] * 4
    cams = _cameras(sizes=sizes, seed=6)
    sets = [_settings(c, dev) for c in cams]
    rast, _ = _batched(T, sets)
    imgs = rast.images()
    ties = _tie_masks(rast)
    assert len(imgs) == 32 and imgs[0].shape == (3, 1, 1)
    for k, st in enumerate(sets):
        img, radii = _plain(T, st)[:2]
        assert torch.equal(rast.radii[k], radii), k
        d = (imgs[k] - img).abs().amax(0).cpu().numpy()
        assert d[~ties[k]].max(initial=0.0) <= 1e-6, k
    with pytest.raises(ValueError):
        BatchedRasterizer(sets + sets[:1], s.P)  # 33 cameras


def test_batched_zero_gaussians_gives_background(cuda_device):
    dev = cuda_device
    cams = _cameras(sizes=[(40, 30), (16, 16)])
    sets = [_settings(c, dev, bg) for c, bg in zip(cams, _bgs(2))]
    e = torch.empty((0, 3), device=dev)
    rast = BatchedRasterizer(sets, 0, pair_capacity=1024)
    rast.forward(e, torch.empty((0, 1), device=dev), torch.empty((0, 1, 3), device=dev), torch.empty((0, 15, 3), device=dev),
                 None, e, torch.empty((0, 4), device=dev), None, 3)
    g = rast.backward(torch.ones(rast.out_color.numel(), device=dev), e, torch.empty((0, 1, 3), device=dev),
                      torch.empty((0, 15, 3), device=dev), e, torch.empty((0, 4), device=dev), 3)
    torch.cuda.synchronize()
    assert _C.device_errors(dev) == 0
    for k, im in enumerate(rast.images()):
        bg = torch.tensor(_bgs(2)[k], device=dev, dtype=torch.float32).view(3, 1, 1)
        assert torch.equal(im, bg.expand_as(im)), k
    assert rast.status() == (0, 0)
    assert g["means3D"].numel() == 0


def test_native_autotuner_times_candidates_and_picks_the_fastest(setup):
    """fgs_tune (through tune.autotune_native): every candidate that fits is timed, the fastest
    is returned; a pair capacity too small for the frame marks every candidate -2 and reports
    FGS_ERR_CAPACITY without touching memory past the buffers."""
    import ctypes as C
    from fastergs_gb300 import _lib
    from fastergs_gb300.tune import autotune_native
    s, T, cams, sets = setup
    params = {"means3D": T["means"], "opacities": T["opacities"], "dc": T["dc"], "shs": T["shs"],
              "scales": T["scales"], "rotations": T["rotations"]}
    cands = [TuneConfig(), TuneConfig(32, 16, 16, 4), TuneConfig(64, 8, 32, 2), TuneConfig(16, 16, 16, 8, True)]
    for backward in (False, True):
        best, table = autotune_native(sets, params, sh_degree=3, candidates=cands, backward=backward, reps=2)
        ms = [r["ms"] for r in table]
        assert all(m > 0 for m in ms), ms
        assert best == cands[int(np.argmin(ms))]
    assert _C.device_errors(T["means"].device) == 0
    # capacity far below the frame's pairs: every candidate overflows
    rast = BatchedRasterizer(sets, T["means"].shape[0], pair_capacity=1 << 10)
    arr = (_lib.TuneConfig * 2)(cands[0].as_c(), cands[1].as_c())
    ms = (C.c_float * 2)()
    best = C.c_int(5)
    st = _lib.load().fgs_tune(T["means"].shape[0], 3, T["shs"].shape[1], T["means"].data_ptr(), None,
                              T["dc"].data_ptr(), T["shs"].data_ptr(), T["opacities"].data_ptr(),
                              T["scales"].data_ptr(), T["rotations"].data_ptr(), None, rast.V, rast._cams, arr, 2,
                              rast.pair_capacity, rast.workspace.data_ptr(), rast.workspace.numel(),
                              rast.out_color.data_ptr(), rast.radii.data_ptr(), None, None, 0, 1, C.byref(best),
                              ms, torch.cuda.current_stream().cuda_stream)
    assert st == 2 and best.value == -1
    assert ms[0] == -2.0 or ms[0] == -1.0
    _C.device_errors(T["means"].device)  # clears the capacity bit the skipped writes latched
    assert _C.device_errors(T["means"].device) == 0
