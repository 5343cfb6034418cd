"""GPU parity at the benchmark's full sizes, against the FP64 oracle replaying
the device's own records and pair lists.

Workloads (the ones the bench times):
  C2   1,000,000 Gaussians, 1297x840, SH degree 3: forward and backward;
  C3   3,000,000 Gaussians in 64 Zipf(1.2) clusters, 1920x1080: forward;
  C4   the C2 scene through three of the sixteen C4 cameras (1920x1080,
       1297x840, 640x360) in one batched launch at the autotuner's choice
       (bucket 64, 16x16 tiles): forward and backward;
  C5b  6,000,000 clustered Gaussians at 3840x2160, one batched view with the
       bucket prefixes stored and recomputed: forward.

Checks and tolerances:
  * sort: the sorted pairs are a stable sort of the emitted pairs, bit for bit;
    tile ranges bit-exact;
  * pair sets: equal to the oracle's tile test on the device's records except
    pairs the oracle flags: a nudge of 1e-4 relative in the power or of 0.01 px
    of the centre changes the outcome, or a comparison of the test lies within
    its FP32 rounding bound (the discriminant cancels for thin footprints);
    flagged pairs, including the ones the FP64 test rejects, at most 0.5%;
  * images: max-abs 1e-5 on pixels the oracle does not flag as ambiguous (an
    alpha within 1e-5 relative of 1/255, or a bucket-end transmittance within
    1e-5 relative of 1e-4); at most 1% of the pixels may be flagged;
    last_contributor bit-exact and Ts_final within 1e-5 there; the bucket
    count equal;
  * gradients (upstream gradient zeroed at flagged pixels): per tensor
    max |device - oracle| <= 1e-4 max |oracle|, and per entry
    |device - oracle| <= 1e-4 |oracle| + floor max |oracle| with floor 5e-6
    (dL/drot: the per-tensor bound): entries are sums of many terms that can
    cancel to a small value (gpu_util.check_gradients).
"""
import numpy as np
import pytest
import torch

from fastergs_gb300 import _C, scenes
from fastergs_gb300.batched import TuneConfig
from gpu_util import check_gradients, gpu_records_as_oracle, oracle_scene, replay_oracle, run_backward, run_forward

pytestmark = pytest.mark.gpu


def check_forward(s, fw, bg=(0.0, 0.0, 0.0)):
    """Sort, ranges, pair set and image of one plain-path frame against the oracle replay."""
    keys = fw["keys_unsorted"].view(np.uint64)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(fw["keys_sorted"].view(np.uint64), keys[order])
    np.testing.assert_array_equal(fw["vals_sorted"], fw["vals_unsorted"][order])
    tiles = (keys[order] >> np.uint64(32)).astype(np.int64)
    T = fw["ranges"].shape[0]
    starts = np.searchsorted(tiles, np.arange(T), side="left")
    ends = np.searchsorted(tiles, np.arange(T), side="right")
    ref = np.stack([np.where(ends > starts, starts, 0), np.where(ends > starts, ends, 0)], 1)
    np.testing.assert_array_equal(fw["ranges"].astype(np.int64), ref)
    # pair set: the oracle's tile test on the device's records
    oe = oracle_scene(s)
    rec, radii, _ = gpu_records_as_oracle(fw)
    oe.set_records(rec, radii, radii > 0)
    oe.emit_sort(eps_pair=1e-4)
    pr = oe.pairs()
    code = lambda t, i: (np.asarray(t, np.uint64) << np.uint64(32)) | np.asarray(i, np.uint64)
    gpu = code(keys >> np.uint64(32), fw["vals_unsorted"].astype(np.uint64))
    assert np.unique(gpu).size == gpu.size, "duplicate pairs emitted"
    orc = code(pr["keys"] >> np.uint64(32), pr["ids"].astype(np.uint64))
    diff = np.setxor1d(gpu, orc)
    amb = np.union1d(orc[pr["ambiguous"]], code(pr["cand_keys"] >> np.uint64(32), pr["cand_ids"].astype(np.uint64)))
    assert np.isin(diff, amb).all(), f"{int((~np.isin(diff, amb)).sum())} pairs differ outside the flagged ones"
    assert amb.size <= 5e-3 * max(orc.size, 1), amb.size
    # image
    o = replay_oracle(s, fw, bg=bg)
    im = o.image()
    ok = ~im["ambiguous"]
    assert ok.mean() > 0.99, f"{1 - ok.mean():.4f} of the pixels flagged"
    gimg = fw["out_color"].cpu().numpy().astype(np.float64)
    err = np.abs(gimg - im["out_color"])[:, ok].max()
    assert err <= 1e-5, err
    lc = fw["last_contrib"].cpu().numpy()[..., 0]
    np.testing.assert_array_equal(lc[ok], im["last_contributor"][ok])
    tf = fw["Ts_final"].cpu().numpy()[..., 0]
    assert np.abs(tf - im["Ts_final"])[ok].max() <= 1e-5
    assert fw["bucket_sum"] == im["num_buckets"]
    return o, im


def test_c2_full_forward_and_backward(cuda_device):
    s = scenes.scene_c2(seed=0)
    fw = run_forward(s, cuda_device, cap=1 << 23)
    assert fw["K"] > 3_000_000
    o, im = check_forward(s, fw)
    dL = scenes.upstream_grad(0, s.camera.height, s.camera.width)
    dL[:, im["ambiguous"]] = 0.0
    g = run_backward(s, fw, dL, cuda_device, stats=True)
    r = o.backward(dL.astype(np.float64))
    check_gradients(g, r)


def test_c3_full_forward(cuda_device):
    s = scenes.scene_c3(seed=0)
    bg = (0.1, 0.2, 0.3)
    fw = run_forward(s, cuda_device, bg=bg, cap=1 << 22)
    assert fw["K"] > 1_000_000
    check_forward(s, fw, bg=bg)


def _batched_replay(s, rast, state, k, cam, tune, bg):
    """Oracle compositing of camera k of a batched frame from the device's records and lists."""
    from test_gpu_batched import _CAMS, _view_replay
    _CAMS[id(rast)] = {k: cam}
    return _view_replay(s, None, rast, state, k, bg, tune)


def test_c4_cameras_batched_at_the_tuned_config(cuda_device):
    from fastergs_gb300.batched import BatchedRasterizer
    from test_gpu_batched import _settings
    s = scenes.scene_c2(seed=0)
    c4 = scenes.cameras_c4(seed=0)
    cams = [c4[7], c4[1], c4[6]]
    assert [(c.width, c.height) for c in cams] == [(1920, 1080), (1297, 840), (640, 360)]
    tune = TuneConfig(64, 16, 16, 4)
    bgs = [(0.0, 0.0, 0.0), (0.2, 0.3, 0.4), (1.0, 1.0, 1.0)]
    sets = [_settings(c, cuda_device, bg) for c, bg in zip(cams, bgs)]
    m, sc, rot, op, dc, shs = s.activated()
    t = lambda a: torch.tensor(np.ascontiguousarray(a), device=cuda_device)
    T = dict(means=t(m), scales=t(sc), rotations=t(rot), opacities=t(op), dc=t(dc), shs=t(shs))
    rast = BatchedRasterizer(sets, s.P, tune=tune)
    rast.fit(T["means"], T["opacities"], T["dc"], T["shs"], None, T["scales"], T["rotations"], None, 3)
    rast.forward(T["means"], T["opacities"], T["dc"], T["shs"], None, T["scales"], T["rotations"], None, 3)
    torch.cuda.synchronize()
    assert _C.device_errors(cuda_device) == 0
    state = rast.state()
    ku = state["keys_unsorted"].numpy().view(np.uint64)
    order = np.argsort(ku, kind="stable")
    np.testing.assert_array_equal(state["keys_sorted"].numpy().view(np.uint64), ku[order])
    np.testing.assert_array_equal(state["vals_sorted"].numpy().view(np.uint32),
                                  state["vals_unsorted"].numpy().view(np.uint32)[order])
    imgs = rast.images()
    dLs, refs = [], []
    for k, (cam, bg) in enumerate(zip(cams, bgs)):
        o = _batched_replay(s, rast, state, k, cam, tune, bg)
        im = o.image()
        ok = ~im["ambiguous"]
        assert ok.mean() > 0.99, (k, 1 - ok.mean())
        err = np.abs(imgs[k].cpu().numpy().astype(np.float64) - im["out_color"])[:, ok].max()
        assert err <= 1e-5, (k, err)
        dL = scenes.upstream_grad(30 + k, cam.height, cam.width)
        dL[:, im["ambiguous"]] = 0.0
        dLs.append(torch.tensor(dL, device=cuda_device))
        refs.append(o.backward(dL.astype(np.float64)))
    g = rast.backward(torch.cat([d.reshape(-1) for d in dLs]), T["means"], T["dc"], T["shs"], T["scales"],
                      T["rotations"], 3)
    torch.cuda.synchronize()
    summed = {k: sum(r[k] for r in refs) for k in ("dmean3D", "ddc", "dsh", "dscale", "drot", "dopacity")}
    dev = {"dmean3D": g["means3D"], "ddc": g["dc"], "dsh": g["shs"], "dscale": g["scales"], "drot": g["rotations"],
           "dopacity": g["opacities"]}
    check_gradients({k: v.cpu().numpy() for k, v in dev.items()}, summed, keys=list(summed))


def test_c5b_forward_store_and_recompute(cuda_device):
    from fastergs_gb300.batched import BatchedRasterizer
    from test_gpu_batched import _settings
    s = scenes.scene_c5b(seed=0)
    cam = s.camera
    m, sc, rot, op, dc, shs = s.activated()
    t = lambda a: torch.tensor(np.ascontiguousarray(a), device=cuda_device)
    T = dict(means=t(m), scales=t(sc), rotations=t(rot), opacities=t(op), dc=t(dc), shs=t(shs))
    del m, sc, rot, op, dc, shs
    st = _settings(cam, cuda_device, (0.0, 0.0, 0.0))
    imgs = {}
    for name, rec in (("store", False), ("recompute", True)):
        tune = TuneConfig(recompute=rec)
        rast = BatchedRasterizer([st], s.P, tune=tune)
        rast.fit(T["means"], T["opacities"], T["dc"], T["shs"], None, T["scales"], T["rotations"], None, 3,
                 headroom=1.05)
        rast.forward(T["means"], T["opacities"], T["dc"], T["shs"], None, T["scales"], T["rotations"], None, 3)
        torch.cuda.synchronize()
        assert _C.device_errors(cuda_device) == 0
        imgs[name] = rast.images()[0].cpu().numpy()
        if name == "store":
            state = rast.state()
            o = _batched_replay(s, rast, state, 0, cam, tune, (0.0, 0.0, 0.0))
            im = o.image()
            ok = ~im["ambiguous"]
            assert ok.mean() > 0.99, 1 - ok.mean()
            err = np.abs(imgs[name].astype(np.float64) - im["out_color"])[:, ok].max()
            assert err <= 1e-5, err
            del state, o
        del rast
        torch.cuda.empty_cache()
    np.testing.assert_array_equal(imgs["store"], imgs["recompute"])
