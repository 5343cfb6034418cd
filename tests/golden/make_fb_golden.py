"""Golden vectors produced by the reference CUDA backend itself (FB).

FB is ``gs_submodules/diff-gaussian-rasterization_faster``, built for sm_103a
from its own sources by ``oracle/fb_ref.py``.  This script runs FB's forward
and backward through FB's own ``_C.ops``, in the call order of FB's
``_RasterizeGaussians`` (FB ``__init__.py:98-187``), on the seeded scenes
below, and writes what FB returns to ``tests/golden/fb_<scene>.npz``:

  radii, bucket_sum, pair count K, sorted Gaussian ids, tile ranges,
  out_color, last_contributor, Ts_final, the nine backward tensors
  (FB ``pybind.cpp:210-339``; for c2_small dL/dsh of the first
  ``DSH_ROWS`` Gaussians only, to keep the fixture small) and the four
  densification statistics.

The scene inputs are not stored: ``fastergs_gb300.scenes`` regenerates them
bit for bit from their seeds.  The upstream gradient is
``scenes.upstream_grad(0, H, W)`` with zeros on ``dL_mask``: the pixels the
FP64 oracle flags as ambiguous (an alpha or a bucket-end transmittance within
rounding distance of FB's 1/255 and 1e-4 thresholds) and every pixel of a
tile holding a pair whose tile test is within rounding distance of its
threshold.  There a discrete decision may go either way in FP32, and a
flipped decision changes the gradient of every Gaussian of the tile; the
mask is stored so that tests use the same upstream gradient.

Run on a machine with a GB300 after staging and building FB:

    FASTERGS_REF=<FasterGS checkout> python oracle/fb_ref.py stage
    python oracle/fb_ref.py build
    python tests/golden/make_fb_golden.py [out_dir]

(``out_dir`` defaults to this directory.)
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
for p in (ROOT, ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

from fastergs_gb300 import scenes  # noqa: E402

# name -> scene factory; the same scenes the product's parity tests use
SCENES = {
    "c1": lambda: scenes.scene_c1(),
    "c5a": lambda: scenes.scene_c5a(),
    "c2_small": lambda: scenes.scene_c2(seed=0, P=20000, width=320, height=208),
}
GRADS = ["dmean2D", "dcolor", "dopacity", "dmean3D", "dcov3D", "ddc", "dsh", "dscale", "drot"]
DSH_ROWS = {"c2_small": 4000}


def upstream_mask(scene):
    """(H, W) bool: where the oracle says a discrete decision of the forward is within rounding."""
    import oracle
    m, sc, rot, op, dc, shs = [np.asarray(a, np.float64) for a in scene.activated()]
    o = oracle.Oracle().set_scene(m, op, sc, rot, scene.camera, dc=dc, shs=shs, sh_degree=scene.sh_degree)
    o.preprocess()
    o.emit_sort()
    pr = o.pairs()
    o.render()
    mask = o.image()["ambiguous"].copy()
    W = scene.camera.width
    gx = (W + 15) // 16
    rg = pr["ranges"]
    for t in range(rg.shape[0]):
        if pr["ambiguous"][rg[t, 0]:rg[t, 1]].any():
            ty, tx = divmod(t, gx)
            mask[ty * 16:(ty + 1) * 16, tx * 16:(tx + 1) * 16] = True
    return mask


def run(name: str, dev, fb) -> dict:
    import torch
    from gpu_util import run_backward, run_forward
    s = SCENES[name]()
    cam = s.camera
    fw = run_forward(s, dev, ops=fb._C.ops, buffer_cls=fb.Buffer)
    mask = upstream_mask(s)
    dL = scenes.upstream_grad(0, cam.height, cam.width)
    dL[:, mask] = 0.0
    g = run_backward(s, fw, dL, dev, stats=True)
    out = dict(dL_mask=mask,
        P=np.int64(s.P), W=np.int64(cam.width), H=np.int64(cam.height), K=np.int64(fw["K"]),
        bucket_sum=np.int64(fw["bucket_sum"]),
        radii=fw["radii"].cpu().numpy().astype(np.int32),
        vals_sorted=fw["vals_sorted"].astype(np.int32),
        ranges=fw["ranges"].astype(np.int32),
        out_color=fw["out_color"].cpu().numpy().astype(np.float32),
        last_contributor=fw["last_contrib"].cpu().numpy()[..., 0].astype(np.int32),
        Ts_final=fw["Ts_final"].cpu().numpy()[..., 0].astype(np.float32),
    )
    for k in GRADS:
        out[k] = g[k].astype(np.float32)
    if name in DSH_ROWS:
        out["dsh"] = out["dsh"][:DSH_ROWS[name]]
    for k, a in zip(("xyz_gradient_accum", "xyz_gradient_accum_abs", "max_radii", "denom"), g["stats"]):
        out[k] = a.astype(np.float32)
    torch.cuda.synchronize()
    return out


def main(out_dir: Path) -> None:
    import torch
    from oracle import fb_ref
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    fb = fb_ref.load()
    out_dir.mkdir(parents=True, exist_ok=True)
    for name in SCENES:
        res = run(name, dev, fb)
        np.savez_compressed(out_dir / f"fb_{name}.npz", **res)
        print(f"{name}: P={int(res['P'])} K={int(res['K'])} buckets={int(res['bucket_sum'])} -> "
              f"{out_dir / f'fb_{name}.npz'}", flush=True)


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else HERE)
