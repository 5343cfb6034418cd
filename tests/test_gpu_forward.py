"""GPU parity of the forward path (preprocess, key emission, sort, tile
ranges, bucket compositing + merge) against the FP64 oracle.

Tolerances (FP32 device vs FP64 oracle):
  * radii, tile rectangles, clamp flags, (tile, Gaussian) pair sets, sorted
    lists, tile ranges, last_contributor: bit-exact, except entries the
    oracle flags as within rounding distance of a discrete threshold;
  * images: max-abs 1e-5 when the oracle composites the device's own
    records and lists (replay), excluding pixels the oracle flags as
    ambiguous (an alpha within 1e-5 relative of the 1/255 cut-off or a
    bucket-end transmittance within 1e-5 relative of 1e-4);
  * images against the oracle's own FP64 records (compositing the device's
    pair lists, or fully independent lists for the small scenes): max-abs
    1e-5.
"""
import numpy as np
import pytest
import torch

from fastergs_gb300 import _C, _lib, scenes
from gpu_util import gpu_records_as_oracle, oracle_scene, replay_oracle, run_forward

pytestmark = pytest.mark.gpu


def small_c2(seed=0, P=20000, W=320, H=208):
    return scenes.scene_c2(seed=seed, P=P, width=W, height=H)


def deep_tiles():
    """Dense Zipf clusters on a small frame: five tiles need more than the
    forward's chain of 8 sub-buckets (up to 41), so their later buckets go
    through the deep-tile merge."""
    return scenes.scene_clusters(seed=3, P=60000, width=256, height=192, name="deep")


SCENES = {
    "c1": lambda: scenes.scene_c1(),
    "c5a": lambda: scenes.scene_c5a(),
    "c2_small": lambda: small_c2(),
    "deep": deep_tiles,
}


@pytest.mark.parametrize("name", list(SCENES))
def test_preprocess_records_match_oracle(cuda_device, name):
    s = SCENES[name]()
    fw = run_forward(s, cuda_device)
    o = oracle_scene(s).preprocess()
    r = o.records()
    radii = fw["radii"].cpu().numpy()
    amb = r["ambiguous"]
    assert (~amb).mean() > 0.99, amb.sum()  # the flagged entries are few
    assert np.array_equal(radii[~amb], r["radii"][~amb])
    valid = r["valid"] & ~amb
    g = fw["rec"].astype(np.float64)
    gi = fw["rec"].view(np.int32)
    ref = r["rec"]
    v = valid
    np.testing.assert_allclose(g[v, 0:2], ref[v, 0:2], atol=1e-4, rtol=0)              # FP32 pixel xy
    # full-precision position: floor(float x) + fraction (FP64 projection)
    gpos = np.floor(g[v, 0:2]) + g[v, 10:12]
    opos = np.floor(ref[v, 0:2].astype(np.float32).astype(np.float64)) + ref[v, 10:12]
    np.testing.assert_allclose(gpos, opos, atol=1e-6, rtol=0)
    np.testing.assert_allclose(g[v, 2:5], ref[v, 2:5], atol=1e-5, rtol=0)               # rgb
    np.testing.assert_allclose(g[v, 5], ref[v, 5], rtol=1e-6)                           # depth
    np.testing.assert_allclose(g[v, 6], ref[v, 6], rtol=2e-5)                           # A1
    assert np.all(np.abs(g[v, 7] - ref[v, 7]) <= 2e-5 * (np.abs(ref[v, 7]) + 1))        # P
    np.testing.assert_allclose(g[v, 8], ref[v, 8], rtol=2e-5)                           # C1
    np.testing.assert_allclose(g[v, 9], ref[v, 9], atol=2e-6)                           # log2 opacity
    np.testing.assert_array_equal(gi[v, 12:16], ref[v, 12:16].astype(np.int32))        # tile rect
    cn = np.linalg.norm(ref[v, 16:19], axis=1, keepdims=True)
    assert np.all(np.abs(g[v, 16:19] - ref[v, 16:19]) <= 2e-5 * cn)                    # conic
    np.testing.assert_allclose(g[v, 19], ref[v, 19], rtol=2e-6, atol=2e-6)             # power
    tr = (ref[v, 23] + ref[v, 26] + ref[v, 28])[:, None]
    assert np.all(np.abs(g[v, 23:29] - ref[v, 23:29]) <= 1e-6 * tr)                     # cov3D
    pre = ref[v, 2:5]  # clamp flags are exact away from a zero crossing
    sure = np.all(np.abs(pre) > 1e-5, axis=1) | (ref[v, 20:23].sum(1) == 0)
    np.testing.assert_array_equal(g[v][sure, 20:23], ref[v][sure, 20:23])


@pytest.mark.parametrize("name", list(SCENES))
def test_emitted_pairs_match_oracle_replay(cuda_device, name):
    s = SCENES[name]()
    fw = run_forward(s, cuda_device)
    o = oracle_scene(s)
    rec, radii, _ = gpu_records_as_oracle(fw)
    o.set_records(rec, radii, radii > 0)
    o.emit_sort(eps_pair=1e-5)
    pr = o.pairs()
    gtile = (fw["keys_unsorted"].view(np.uint64) >> np.uint64(32)).astype(np.int64)
    gpu = set(zip(gtile.tolist(), fw["vals_unsorted"].tolist()))
    assert len(gpu) == fw["K"], "duplicate pairs emitted"
    otile = (pr["keys"] >> np.uint64(32)).astype(np.int64)
    orc = set(zip(otile.tolist(), pr["ids"].tolist()))
    amb = set(zip(otile[pr["ambiguous"]].tolist(), pr["ids"][pr["ambiguous"]].tolist()))
    amb |= set(zip((pr["cand_keys"] >> np.uint64(32)).astype(np.int64).tolist(), pr["cand_ids"].tolist()))
    assert len(amb) <= 0.01 * len(orc), len(amb)  # the flagged pairs are few
    assert (gpu ^ orc) <= amb, f"{len(gpu - orc)} extra / {len(orc - gpu)} missing pairs"
    # depth bits of every key are the record's depth
    depth_bits = (fw["keys_unsorted"].view(np.uint64) & np.uint64(0xffffffff)).astype(np.uint32)
    rec_depth = fw["rec"][fw["vals_unsorted"], 5].view(np.uint32)
    np.testing.assert_array_equal(depth_bits, rec_depth)


def test_sorted_list_is_stable_sort_of_emitted_pairs(cuda_device):
    s = small_c2()
    fw = run_forward(s, cuda_device)
    keys = fw["keys_unsorted"].view(np.uint64)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(fw["keys_sorted"].view(np.uint64), keys[order])
    np.testing.assert_array_equal(fw["vals_sorted"], fw["vals_unsorted"][order])


def _sort_via_cabi(keys_np, vals_np, W, H, dev):
    lib = _lib.load()
    K = keys_np.size
    k_in = torch.tensor(keys_np.view(np.int64), device=dev)
    v_in = torch.tensor(vals_np.view(np.int32), device=dev)
    k_out = torch.empty(max(K, 1), dtype=torch.int64, device=dev)
    v_out = torch.empty(max(K, 1), dtype=torch.int32, device=dev)
    tmp = torch.empty(int(lib.fgs_sort_temp_bytes(K)), dtype=torch.uint8, device=dev)
    _lib.call("fgs_sort", K, W, H, 16, 16, tmp.data_ptr(), tmp.numel(), k_in.data_ptr() if K else 0,
              v_in.data_ptr() if K else 0, k_out.data_ptr(), v_out.data_ptr(),
              torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert _C.device_errors(dev) == 0
    np.testing.assert_array_equal(k_in.cpu().numpy().view(np.uint64), keys_np)  # input untouched
    return k_out[:K].cpu().numpy().view(np.uint64), v_out[:K].cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("K", [0, 1, 31, 4095, 4096, 4097, 123457, 3_000_001])
@pytest.mark.parametrize("WH", [(256, 256), (1297, 840), (3840, 2160)])
def test_radix_sort_bit_exact(cuda_device, K, WH):
    W, H = WH
    T = ((W + 15) // 16) * ((H + 15) // 16)
    rng = np.random.default_rng(K + W)
    tiles = rng.integers(0, T, K, dtype=np.uint64)
    # few distinct depths -> many equal keys, which checks stability
    depth = rng.choice(rng.uniform(0.2, 50.0, size=max(K // 8, 1)).astype(np.float32), size=K).view(np.uint32)
    keys = (tiles << np.uint64(32)) | depth.astype(np.uint64)
    vals = np.arange(K, dtype=np.uint32)
    ks, vs = _sort_via_cabi(keys, vals, W, H, cuda_device)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(ks, keys[order])
    np.testing.assert_array_equal(vs, vals[order])


def test_tile_ranges_bit_exact(cuda_device):
    s = small_c2()
    fw = run_forward(s, cuda_device)
    tiles = (fw["keys_sorted"].view(np.uint64) >> np.uint64(32)).astype(np.int64)
    T = fw["ranges"].shape[0]
    ref = np.zeros((T, 2), np.int64)
    starts = np.searchsorted(tiles, np.arange(T), side="left")
    ends = np.searchsorted(tiles, np.arange(T), side="right")
    ref[:, 0] = np.where(ends > starts, starts, 0)
    ref[:, 1] = np.where(ends > starts, ends, 0)
    np.testing.assert_array_equal(fw["ranges"].astype(np.int64), ref)


@pytest.mark.parametrize("name", list(SCENES))
@pytest.mark.parametrize("bg", [(0.0, 0.0, 0.0), (0.3, 0.6, 0.9)])
def test_render_matches_oracle_replay(cuda_device, name, bg):
    s = SCENES[name]()
    fw = run_forward(s, cuda_device, bg=bg)
    o = replay_oracle(s, fw, bg=bg)
    im = o.image()
    ok = ~im["ambiguous"]
    assert ok.mean() > 0.99
    gimg = fw["out_color"].cpu().numpy().astype(np.float64)
    err = np.abs(gimg - im["out_color"])[:, ok]
    assert err.max() <= 1e-5, err.max()
    lc = fw["last_contrib"].cpu().numpy()[..., 0]
    np.testing.assert_array_equal(lc[ok], im["last_contributor"][ok])
    tf = fw["Ts_final"].cpu().numpy()[..., 0]
    assert np.abs(tf - im["Ts_final"])[ok].max() <= 1e-5
    assert fw["bucket_sum"] == im["num_buckets"]


@pytest.mark.parametrize("name", list(SCENES))
def test_render_vs_fp64_records(cuda_device, name):
    """Images against the oracle's own FP64 preprocess, compositing the
    device's (tile, Gaussian) lists: 1e-5 max-abs."""
    s = SCENES[name]()
    fw = run_forward(s, cuda_device)
    o = oracle_scene(s).preprocess()
    o.set_lists(fw["vals_sorted"], fw["ranges"])
    o.render(eps_alpha=1e-4, eps_T=1e-4)
    im = o.image()
    ok = ~im["ambiguous"]
    assert ok.mean() > 0.99
    gimg = fw["out_color"].cpu().numpy().astype(np.float64)
    assert np.abs(gimg - im["out_color"])[:, ok].max() <= 1e-5


@pytest.mark.parametrize("name", ["c1", "c5a"])
def test_render_end_to_end_vs_fp64_oracle(cuda_device, name):
    """Fully independent FP64 pipeline (own pair lists and sort)."""
    s = SCENES[name]()
    fw = run_forward(s, cuda_device)
    o = oracle_scene(s).preprocess()
    o.emit_sort(eps_pair=1e-4)
    o.render(eps_alpha=1e-4, eps_T=1e-4)
    im = o.image()
    ok = ~im["ambiguous"]
    gimg = fw["out_color"].cpu().numpy().astype(np.float64)
    assert np.abs(gimg - im["out_color"])[:, ok].max() <= 1e-5


def test_ragged_image_and_culling(cuda_device):
    s = scenes.scene_c1(seed=3, P=4000)
    s.camera = scenes.make_camera(250, 170, 60.0)
    rng = np.random.default_rng(5)
    cull = rng.random(s.P) < 0.3
    fw = run_forward(s, cuda_device, culling=cull, bg=(0.2, 0.1, 0.0), mult=1.3, smod=0.8)
    assert np.all(fw["radii"].cpu().numpy()[cull] == 0)
    assert not np.isin(np.flatnonzero(cull), fw["vals_unsorted"]).any()
    o = replay_oracle(s, fw, bg=(0.2, 0.1, 0.0), culling=cull, mult=1.3, smod=0.8)
    im = o.image()
    ok = ~im["ambiguous"]
    gimg = fw["out_color"].cpu().numpy().astype(np.float64)
    assert np.abs(gimg - im["out_color"])[:, ok].max() <= 1e-5
    o2 = oracle_scene(s, culling=cull, mult=1.3, smod=0.8).preprocess()
    r = o2.records()
    a = r["ambiguous"]
    np.testing.assert_array_equal(fw["radii"].cpu().numpy()[~a], r["radii"][~a])


def test_precomputed_colours(cuda_device):
    s = scenes.scene_c1(seed=4, P=3000)
    colors = np.random.default_rng(9).uniform(0, 1, size=(s.P, 3)).astype(np.float32)
    fw = run_forward(s, cuda_device, colors=colors)
    o = replay_oracle(s, fw, colors=colors)
    im = o.image()
    ok = ~im["ambiguous"]
    gimg = fw["out_color"].cpu().numpy().astype(np.float64)
    assert np.abs(gimg - im["out_color"])[:, ok].max() <= 1e-5


def test_everything_culled_gives_background(cuda_device):
    s = scenes.scene_c1(seed=1, P=500)
    fw = run_forward(s, cuda_device, culling=np.ones(s.P, bool), bg=(0.1, 0.2, 0.3))
    assert fw["K"] == 0 and fw["bucket_sum"] == 0
    img = fw["out_color"].cpu().numpy()
    np.testing.assert_allclose(img[:, 0, 0], [0.1, 0.2, 0.3], rtol=1e-7)
    assert np.all(fw["Ts_final"].cpu().numpy() == 1.0)


def huge_and_odd(W, H, seed=7, P=600, n_huge=20):
    """C1-like scene on a W x H image with n_huge Gaussians large enough
    (tile rectangle of 128 tiles or more on the larger images) to take the
    large-footprint sub-task path of the preprocess."""
    s = scenes.scene_c1(seed=seed, P=P)
    rng = np.random.default_rng(seed + 1)
    s.means[:n_huge] = np.stack([rng.uniform(-0.6, 0.6, n_huge), rng.uniform(-0.4, 0.4, n_huge),
                                 rng.uniform(3.0, 5.0, n_huge)], axis=1).astype(np.float32)
    s.log_scales[:n_huge] = np.log(rng.uniform(0.25, 0.5, (n_huge, 3))).astype(np.float32)
    s.opacity_logits[:n_huge] = rng.uniform(-3.0, -1.0, (n_huge, 1)).astype(np.float32)
    s.camera = scenes.make_camera(W, H, 60.0)
    return s


ODD_SIZES = [(1, 1), (5, 3), (17, 33), (1031, 9), (640, 480)]


@pytest.mark.parametrize("WH", ODD_SIZES, ids=lambda wh: f"{wh[0]}x{wh[1]}")
def test_huge_gaussians_and_odd_image_sizes(cuda_device, WH):
    W, H = WH
    s = huge_and_odd(W, H)
    fw = run_forward(s, cuda_device, bg=(0.25, 0.5, 0.75))
    tiles = ((W + 15) // 16) * ((H + 15) // 16)
    rect = fw["rec"].view(np.int32)[:, 12:16].astype(np.int64)
    radii = fw["radii"].cpu().numpy()
    area = np.where(radii > 0, (rect[:, 2] - rect[:, 0]) * (rect[:, 3] - rect[:, 1]), 0)
    if tiles >= 128:
        assert (area >= 128).sum() >= 5  # the sub-task path is exercised
    # (tile, Gaussian) pairs: the large-footprint sub-tasks emit exactly the
    # pairs the oracle's per-tile test emits, once each
    oe = oracle_scene(s)
    rec, _, _ = gpu_records_as_oracle(fw)
    oe.set_records(rec, radii, radii > 0)
    oe.emit_sort(eps_pair=1e-5)
    pr = oe.pairs()
    gtile = (fw["keys_unsorted"].view(np.uint64) >> np.uint64(32)).astype(np.int64)
    gpu = set(zip(gtile.tolist(), fw["vals_unsorted"].tolist()))
    assert len(gpu) == fw["K"], "duplicate pairs emitted"
    otile = (pr["keys"] >> np.uint64(32)).astype(np.int64)
    orc = set(zip(otile.tolist(), pr["ids"].tolist()))
    amb = set(zip(otile[pr["ambiguous"]].tolist(), pr["ids"][pr["ambiguous"]].tolist()))
    amb |= set(zip((pr["cand_keys"] >> np.uint64(32)).astype(np.int64).tolist(), pr["cand_ids"].tolist()))
    assert len(amb) <= 0.01 * max(len(orc), 100), len(amb)  # the flagged pairs are few
    assert (gpu ^ orc) <= amb, f"{len(gpu - orc)} extra / {len(orc - gpu)} missing pairs"
    o2 = oracle_scene(s).preprocess()
    r = o2.records()
    a = r["ambiguous"]
    np.testing.assert_array_equal(radii[~a], r["radii"][~a])
    o = replay_oracle(s, fw, bg=(0.25, 0.5, 0.75))
    im = o.image()
    ok = ~im["ambiguous"]
    gimg = fw["out_color"].cpu().numpy().astype(np.float64)
    assert gimg.shape == (3, H, W)
    if ok.any():
        assert np.abs(gimg - im["out_color"])[:, ok].max() <= 1e-5
    lc = fw["last_contrib"].cpu().numpy()[..., 0]
    np.testing.assert_array_equal(lc[ok], im["last_contributor"][ok])
    assert fw["bucket_sum"] == im["num_buckets"]
    np.testing.assert_array_equal(fw["ranges"].shape, (tiles, 2))


def test_sort_flags_keys_that_are_not_tile_depth_keys(cuda_device):
    # keys are (tile << 32) | bits of a positive float depth; bit 31 set is a
    # negative depth, which the sort does not order and reports
    keys = np.array([(1 << 32) | 0x3f800000, (0 << 32) | 0xbf800000, (2 << 32) | 0x40000000], np.uint64)
    lib = _lib.load()
    k_in = torch.tensor(keys.view(np.int64), device=cuda_device)
    v_in = torch.arange(3, dtype=torch.int32, device=cuda_device)
    k_out, v_out = torch.empty_like(k_in), torch.empty_like(v_in)
    tmp = torch.empty(int(lib.fgs_sort_temp_bytes(3)), dtype=torch.uint8, device=cuda_device)
    _lib.call("fgs_sort", 3, 64, 64, 16, 16, tmp.data_ptr(), tmp.numel(), k_in.data_ptr(), v_in.data_ptr(),
              k_out.data_ptr(), v_out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert _C.device_errors(cuda_device) & 2  # the capacity bit, cleared by the read
    assert _C.device_errors(cuda_device) == 0
