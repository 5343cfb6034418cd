"""Helpers shared by the GPU parity tests: run the plain path through the
C-ABI (``fastergs_gb300._C.ops``) and set up the oracle on the same inputs."""
from __future__ import annotations

import numpy as np
import torch

import oracle
from fastergs_gb300 import Buffer, _C


def tensors(scene, dev):
    m, sc, rot, op, dc, shs = scene.activated()
    t = lambda a: torch.tensor(np.ascontiguousarray(a), device=dev)
    return dict(means=t(m), scales=t(sc), rotations=t(rot), opacities=t(op), dc=t(dc), shs=t(shs))


_BUFFERS = {}


def buffer(dev, cap=2**21, buffer_cls=None):
    cls = Buffer if buffer_cls is None else buffer_cls
    key = (str(dev), cap, cls)
    if key not in _BUFFERS:
        _BUFFERS.clear()
        torch.cuda.empty_cache()
        _BUFFERS[key] = cls(device=dev, MAX_NUM_RENDERED=cap)
    return _BUFFERS[key]


def run_forward(scene, dev, bg=(0.0, 0.0, 0.0), culling=None, colors=None, mult=1.0, smod=1.0, cap=2**21,
                shs_override="keep", ops=None, buffer_cls=None, T=None):
    """One forward through ``ops`` (this library's ``_C.ops`` by default, or the reference
    backend's, which takes the same arguments) in FB's call order (FB ``__init__.py:98-140``).
    ``T`` overrides the scene's activated parameter tensors."""
    ours = ops is None
    ops = _C.ops if ours else ops
    cam = scene.camera
    T = tensors(scene, dev) if T is None else T
    buf = buffer(dev, cap, buffer_cls)
    f = lambda a: torch.tensor(np.asarray(a, np.float32), device=dev)
    empty = torch.tensor([])
    shs = T["shs"] if shs_override == "keep" else shs_override
    cull = empty.bool() if culling is None else torch.tensor(culling, device=dev)
    col = empty if colors is None else f(colors)
    buf.curr_offset.fill_(0)
    radii = ops.preprocess(scene.sh_degree, T["means"], col, T["dc"] if colors is None else empty,
                              shs if colors is None else empty, T["opacities"], T["scales"], T["rotations"], smod,
                              cam.width, cam.height, 16, 16, f(cam.campos), f(cam.viewmatrix), f(cam.projmatrix),
                              cam.tanfovx, cam.tanfovy, 100.0, 0.01, buf.gaussian_keys_unsorted,
                              buf.gaussian_values_unsorted, buf.gaussian_values_sorted, buf.curr_offset, mult,
                              buf.splat_buffer, cull)
    K = int(buf.curr_offset.cpu()[0])
    assert K < buf.MAX_NUM_RENDERED
    assert not ours or _C.device_errors(dev) == 0
    keys_u = buf.gaussian_keys_unsorted[:K].clone()
    vals_u = buf.gaussian_values_unsorted[:K].clone()
    ops.sort_gaussian(K, cam.width, cam.height, 16, 16, buf.list_sorting_space, buf.gaussian_keys_unsorted,
                         buf.gaussian_values_unsorted, buf.gaussian_keys_sorted, buf.gaussian_values_sorted)
    H, W = cam.height, cam.width
    lc = torch.zeros((H, W, 1), device=dev, dtype=torch.int32)
    Tf = torch.zeros((H, W, 1), device=dev, dtype=torch.float32)
    bsum, out, img_buf, smp_buf = ops.render_16x16(scene.P, K, W, H, buf.splat_buffer,
                                                      buf.gaussian_keys_sorted, buf.gaussian_values_sorted,
                                                      buf.ranges, f(bg), lc, Tf)
    torch.cuda.synchronize()
    assert not ours or _C.device_errors(dev) == 0
    P = scene.P
    return dict(
        K=K, bucket_sum=bsum, radii=radii, out_color=out, last_contrib=lc, Ts_final=Tf, img_buf=img_buf,
        smp_buf=smp_buf, keys_unsorted=keys_u.cpu().numpy(), vals_unsorted=vals_u.cpu().numpy(),
        keys_sorted=buf.gaussian_keys_sorted[:K].cpu().numpy(), vals_sorted=buf.gaussian_values_sorted[:K].cpu().numpy(),
        ranges=buf.ranges[: ((W + 15) // 16) * ((H + 15) // 16)].cpu().numpy(),
        rec=buf.splat_buffer[:P].cpu().numpy(), T=T, buf=buf, bg=f(bg), culling=cull, colors=col, shs=shs,
        mult=mult, smod=smod, ops=ops)


def run_backward(scene, fw, dL, dev, stats=False):
    cam = scene.camera
    T = fw["T"]
    buf = fw["buf"]
    f = lambda a: torch.tensor(np.asarray(a, np.float32), device=dev)
    empty = torch.tensor([])
    P = scene.P
    accum = [torch.zeros((P, 1), device=dev) for _ in range(4)] if stats else [empty] * 4
    colors = fw["colors"].numel() > 0
    res = fw["ops"].backward(scene.sh_degree, fw["bucket_sum"], T["means"], fw["radii"],
                          T["dc"] if not colors else empty, fw["shs"] if not colors else empty, T["opacities"],
                          T["scales"], T["rotations"], fw["smod"], cam.width, cam.height, 16, 16, cam.tanfovx,
                          cam.tanfovy, 100.0, 0.01, f(cam.campos), f(cam.viewmatrix), f(cam.projmatrix),
                          fw["img_buf"], fw["smp_buf"], buf.splat_buffer, buf.gaussian_values_sorted, buf.ranges,
                          fw["bg"], fw["last_contrib"], fw["Ts_final"], f(dL), *accum)
    torch.cuda.synchronize()
    names = ["dmean2D", "dcolor", "dopacity", "dmean3D", "dcov3D", "ddc", "dsh", "dscale", "drot"]
    out = {k: v.cpu().numpy().astype(np.float64) for k, v in zip(names, res)}
    if stats:
        out["stats"] = [a.cpu().numpy()[:, 0].astype(np.float64) for a in accum]
    return out


def oracle_scene(scene, culling=None, colors=None, mult=1.0, smod=1.0, with_shs=True):
    m, sc, rot, op, dc, shs = [np.asarray(a, np.float64) for a in scene.activated()]
    o = oracle.Oracle()
    o.set_scene(m, op, sc, rot, scene.camera, dc=None if colors is not None else dc,
                shs=(shs if with_shs else None) if colors is None else None, colors=colors,
                sh_degree=scene.sh_degree, culling=culling, scale_modifier=smod, mult=mult)
    return o


def gpu_records_as_oracle(fw):
    """The device's float32 records as float64, rect ints decoded."""
    rec = fw["rec"].astype(np.float64)
    raw = fw["rec"].view(np.int32)
    rec[:, 12:16] = raw[:, 12:16]  # tile rect (int bits)
    radii = fw["radii"].cpu().numpy()
    valid = np.zeros(rec.shape[0], bool)
    valid[np.unique(fw["vals_sorted"])] = True
    return rec, radii, valid


def replay_oracle(scene, fw, bg=(0.0, 0.0, 0.0), eps_alpha=1e-5, eps_T=1e-5, **kw):
    """Oracle compositing on the device's own records and sorted lists."""
    o = oracle_scene(scene, **kw)
    rec, radii, _ = gpu_records_as_oracle(fw)
    valid = (radii > 0) | np.isin(np.arange(scene.P), fw["vals_sorted"])
    o.set_records(rec, radii, valid)
    o.set_lists(fw["vals_sorted"], fw["ranges"])
    o.render(bg=bg, eps_alpha=eps_alpha, eps_T=eps_T)
    return o


GRAD_KEYS = ["dmean2D", "dopacity", "dcolor", "dmean3D", "ddc", "dsh", "dscale", "drot"]
# Per-entry floor of the gradient check, as a fraction of the tensor's largest
# value: entries are sums over many pixels whose terms can cancel to a small
# value, and the rounding of those terms stays behind.  dL/drot of a thin
# footprint (condition number in the thousands) is a small difference of
# large products: its entries are held to the per-tensor bound alone (on the
# full-size C2 frame the worst needs 1.3e-5 of the largest value, summed over
# three C4 views 7e-5).
ELEM_FLOOR = {"drot": 1e-4}
ELEM_FLOOR_DEFAULT = 5e-6


def check_gradients(g, r, keys=GRAD_KEYS, tol=1e-4, per_entry=True):
    """Per tensor max |g - r| <= tol max |r|, and (per_entry) every entry |g - r| <= tol |r| + floor max |r|.
    The floor is relative to the tensor's largest value, which only sets a scale when the frame has
    many pixels: tests of frames of a few pixels check the per-tensor bound alone."""
    bad = {}
    for k in keys:
        a = np.asarray(g[k], np.float64).reshape(len(g[k]), -1)
        b = np.asarray(r[k], np.float64).reshape(len(r[k]), -1)
        if k == "dmean2D":  # [:, 2:] are the |dL/dmean2D| sums, compared where a test asks for them
            a, b = a[:, :2], b[:, :2]
        mx = float(np.abs(b).max())
        if mx == 0.0:
            if not np.all(a == 0.0):
                bad[k] = "non-zero where the oracle is zero"
            continue
        e = np.abs(a - b)
        msg = []
        if e.max() > tol * mx:
            msg.append(f"norm-relative {e.max() / mx:.2e}")
        over = e > tol * np.abs(b) + ELEM_FLOOR.get(k, ELEM_FLOOR_DEFAULT) * mx
        if per_entry and over.any():
            i = np.flatnonzero(over.ravel())[:3]
            msg.append(f"{int(over.sum())} entries above the per-entry bound (device {a.ravel()[i]}, "
                       f"oracle {b.ravel()[i]}, max {mx:.3e})")
        if msg:
            bad[k] = ", ".join(msg)
    assert not bad, bad


def ambiguous_tiles_mask(o, im, width):
    """(H, W) bool: the oracle's flagged pixels plus every pixel of a tile whose list holds a pair
    whose tile test is within rounding distance of its threshold."""
    pr = o.pairs()
    mask = im["ambiguous"].copy()
    gx = (width + 15) // 16
    for t in pr["flagged_tiles"].tolist():
        ty, tx = divmod(t, gx)
        mask[ty * 16:(ty + 1) * 16, tx * 16:(tx + 1) * 16] = True
    return mask
