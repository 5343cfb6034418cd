"""Batched multi-camera rasterization over ``fgs_render_batched_fwd/bwd``.

FB renders one camera per call and reads the pair and bucket counts back to
the host three times per step (FB diff_gaussian_rasterization_faster/__init__.py:106-132),
so a training step that sees many cameras is a sequence of small, host-bound
launches.  ``BatchedRasterizer`` renders up to 32 cameras of different
resolutions with one launch per stage and no host synchronisation, which
makes the whole forward + backward capturable in a CUDA graph
(``CapturedStep``).

Capacities are fixed when the rasterizer is planned.  ``fit()`` renders one
frame with a generous pair capacity, reads the count and re-plans with
headroom; a later frame that needs more pairs than planned skips the extra
writes on the device and is reported by ``status()`` (``BatchOverflow``).

Image layout: camera k's (3, H_k, W_k) image starts at float offset
3 * sum_{j<k} H_j W_j of the flat colour buffer; ``images()`` returns views.
Gradients are summed over cameras; densification statistics are accumulated
once per camera, as FB's per-camera backward does.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Sequence

import torch

from . import _lib
from ._C import _f32, _ptr, _stream

MAX_VIEWS = 32
MAX_PAIRS = (1 << 30) - 2  # the sort's look-back words carry 30-bit counts


@dataclass(frozen=True)
class TuneConfig:
    """Launch configuration (``fgs_tune_config``); FB's fixed choice is the default."""

    bucket_size: int = 128
    block_x: int = 16
    block_y: int = 16
    packet: int = 1  # small-footprint candidate tiles per lane and step of the preprocess (FB: 1)
    recompute: bool = False  # rebuild bucket prefixes in the backward instead of storing them
    chain: int = 8  # forward fold-chain length per tile, in (sub-)buckets (results identical for any length)

    def as_c(self) -> _lib.TuneConfig:
        return _lib.TuneConfig(self.bucket_size, self.block_x, self.block_y, self.packet, int(self.recompute),
                               self.chain)


class BatchOverflow(RuntimeError):
    """The last batched frame needed more pairs than the workspace was planned for."""

    def __init__(self, pairs: int, capacity: int):
        super().__init__(f"batched frame needs {pairs} pairs, workspace planned for {capacity}")
        self.pairs = pairs
        self.capacity = capacity


def _mat(t, dev) -> torch.Tensor:
    return t.detach().to(device=dev, dtype=torch.float32).contiguous().reshape(-1)


class BatchedRasterizer:
    """Renders ``len(settings)`` cameras of one scene per call.

    settings: sequence of ``GaussianRasterizationSettings`` (one per camera);
    their matrices are copied into device tables owned here, so
    ``set_cameras`` can move cameras between graph replays.
    """

    def __init__(self, settings: Sequence, num_points: int, tune: TuneConfig | None = None,
                 pair_capacity: int | None = None, device=None):
        V = len(settings)
        if not 1 <= V <= MAX_VIEWS:
            raise ValueError(f"1..{MAX_VIEWS} cameras per batch, got {V}")
        self.device = torch.device(device) if device is not None else settings[0].viewmatrix.device
        if self.device.type != "cuda":
            raise ValueError("BatchedRasterizer needs a CUDA device")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.V = V
        self.P = int(num_points)
        self.tune = tune or TuneConfig()
        self.sizes = [(int(s.image_height), int(s.image_width)) for s in settings]
        self.pix_off = [0]
        for h, w in self.sizes:
            self.pix_off.append(self.pix_off[-1] + h * w)
        f = dict(dtype=torch.float32, device=self.device)
        self._view = torch.zeros((V, 16), **f)
        self._proj = torch.zeros((V, 16), **f)
        self._campos = torch.zeros((V, 4), **f)
        self._bg = torch.zeros((V, 4), **f)
        self._scalars = [None] * V
        self._cams = (_lib.Camera * V)()
        self.set_cameras(settings)
        self._cfg = self.tune.as_c()
        self.out_color = torch.zeros(3 * self.pix_off[-1], **f)
        self.radii = torch.zeros((V, self.P), dtype=torch.int32, device=self.device)
        self.workspace = None
        self.pair_capacity = 0
        self.plan(pair_capacity or self._default_capacity())

    # -- cameras --------------------------------------------------------------------------------
    def set_cameras(self, settings: Sequence) -> None:
        """Copy camera matrices into the device tables (sizes must not change)."""
        if len(settings) != self.V:
            raise ValueError("set_cameras: the number of cameras is fixed at construction")
        for k, s in enumerate(settings):
            if (int(s.image_height), int(s.image_width)) != self.sizes[k]:
                raise ValueError("set_cameras: camera resolutions are fixed at construction")
            self._view[k].copy_(_mat(s.viewmatrix, self.device))
            self._proj[k].copy_(_mat(s.projmatrix, self.device))
            self._campos[k, :3].copy_(_mat(s.campos, self.device))
            self._bg[k, :3].copy_(_mat(s.bg, self.device))
            c = self._cams[k]
            c.viewmatrix = self._view[k].data_ptr()
            c.projmatrix = self._proj[k].data_ptr()
            c.campos = self._campos[k].data_ptr()
            c.bg = self._bg[k].data_ptr()
            c.height, c.width = self.sizes[k]
            c.tan_fovx, c.tan_fovy = float(s.tanfovx), float(s.tanfovy)
            c.scale_modifier, c.mult = float(s.scale_modifier), float(s.mult)

    # -- capacity -------------------------------------------------------------------------------
    def _default_capacity(self) -> int:
        # about 4 pairs per Gaussian and camera at 1 MP, scaled by pixel count; fit() refines it
        mp = self.pix_off[-1] / 1e6
        return int(max(1 << 20, min(MAX_PAIRS, 4 * self.P * max(mp, 1.0))))

    def workspace_bytes(self, pair_capacity: int) -> int:
        out = C.c_size_t(0)
        _lib.call("fgs_batch_workspace_bytes", self.P, self.V, self._cams, C.byref(self._cfg), int(pair_capacity),
                  C.byref(out))
        return int(out.value)

    def plan(self, pair_capacity: int) -> None:
        """(Re)allocate the workspace for up to pair_capacity pairs per frame."""
        pair_capacity = int(min(max(pair_capacity, 1), MAX_PAIRS))
        nbytes = self.workspace_bytes(pair_capacity)
        self.workspace = None
        self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        self.pair_capacity = pair_capacity

    def status(self, raise_on_overflow: bool = True) -> tuple[int, int]:
        """(pairs, buckets) of the last forward; synchronises the stream."""
        pairs, buckets = C.c_int64(0), C.c_int64(0)
        st = _lib.load().fgs_batch_status(self.P, self.V, self._cams, C.byref(self._cfg), self.pair_capacity,
                                          _ptr(self.workspace), C.byref(pairs), C.byref(buckets),
                                          _stream(self.device))
        if st == 2 and raise_on_overflow:  # FGS_ERR_CAPACITY
            raise BatchOverflow(int(pairs.value), self.pair_capacity)
        if st not in (0, 2):
            _lib.check("fgs_batch_status", st)
        return int(pairs.value), int(buckets.value)

    def fit(self, means3D, opacities, dc=None, shs=None, colors_precomp=None, scales=None, rotations=None,
            culling=None, sh_degree=0, headroom: float = 1.25) -> int:
        """Render once, then re-plan the workspace for the pairs seen times headroom.  Returns the pairs.

        The re-planned workspace is rendered into once more, so that after fit() the frame state
        (sorted lists, ranges, per-pixel state for backward(), state()) belongs to these inputs."""
        for _ in range(3):
            self.forward(means3D, opacities, dc, shs, colors_precomp, scales, rotations, culling, sh_degree)
            pairs, _ = self.status(raise_on_overflow=False)
            if pairs <= self.pair_capacity:
                break
            self.plan(int(pairs * headroom) + (1 << 16))
        from . import _C
        _C.device_errors(self.device)  # clear a capacity flag left by an undersized attempt
        self.plan(int(pairs * headroom) + (1 << 16))
        self.forward(means3D, opacities, dc, shs, colors_precomp, scales, rotations, culling, sh_degree)
        return pairs

    def pair_count_word(self) -> torch.Tensor:
        """Device view (1,) int32 of the workspace word that holds the last frame's pair count (the
        pairs the frame needed, also when they exceeded the capacity)."""
        offs = (C.c_int64 * 10)()
        _lib.call("fgs_batch_offsets", self.P, self.V, self._cams, C.byref(self._cfg), self.pair_capacity, offs, 10)
        return self.workspace[offs[0]:offs[0] + 4].view(torch.int32)

    def tile_ranges(self) -> torch.Tensor:
        """Device view (tiles, 2) int32 of the last frame's per-tile [start, end) in the sorted pair
        list, cameras in order (no copy)."""
        offs = (C.c_int64 * 10)()
        _lib.call("fgs_batch_offsets", self.P, self.V, self._cams, C.byref(self._cfg), self.pair_capacity, offs, 10)
        tiles = sum(((w + self.tune.block_x - 1) // self.tune.block_x) * ((h + self.tune.block_y - 1) // self.tune.block_y)
                    for h, w in self.sizes)
        return self.workspace[offs[6]:offs[6] + 8 * tiles].view(torch.int32).view(tiles, 2)

    def state(self) -> dict:
        """Host copies of the last frame's records, pairs, sorted lists and ranges (for tests)."""
        offs = (C.c_int64 * 10)()
        _lib.call("fgs_batch_offsets", self.P, self.V, self._cams, C.byref(self._cfg), self.pair_capacity, offs, 10)
        torch.cuda.synchronize(self.device)
        ws = self.workspace
        K = int(ws[offs[0]:offs[0] + 4].view(torch.int32).item())
        n = min(K, self.pair_capacity)
        R = self.V * self.P
        tiles = sum(((w + self.tune.block_x - 1) // self.tune.block_x) * ((h + self.tune.block_y - 1) // self.tune.block_y)
                    for h, w in self.sizes)
        sl = lambda i, nbytes: ws[offs[i]:offs[i] + nbytes]
        return dict(
            pairs=K,
            records=sl(1, 128 * R).view(torch.float32).view(R, 32).cpu(),
            keys_unsorted=sl(2, 8 * n).view(torch.int64).cpu(),
            vals_unsorted=sl(3, 4 * n).view(torch.int32).cpu(),
            keys_sorted=sl(4, 8 * n).view(torch.int64).cpu(),
            vals_sorted=sl(5, 4 * n).view(torch.int32).cpu(),
            ranges=sl(6, 8 * tiles).view(torch.int32).view(tiles, 2).cpu(),
            last_contrib=sl(7, 4 * self.pix_off[-1]).view(torch.int32).cpu(),
            Ts_final=sl(8, 4 * self.pix_off[-1]).view(torch.float32).cpu(),
        )

    # -- frames ---------------------------------------------------------------------------------
    def images(self, flat: torch.Tensor | None = None) -> list[torch.Tensor]:
        flat = self.out_color if flat is None else flat
        out = []
        for k, (h, w) in enumerate(self.sizes):
            out.append(flat[3 * self.pix_off[k]:3 * self.pix_off[k + 1]].view(3, h, w))
        return out

    def _check_points(self, means3D):
        if means3D.shape[0] != self.P:
            raise ValueError(f"planned for {self.P} Gaussians, got {means3D.shape[0]}")

    def forward(self, means3D, opacities, dc=None, shs=None, colors_precomp=None, scales=None, rotations=None,
                culling=None, sh_degree=0) -> torch.Tensor:
        """Renders every camera into self.out_color (returned) and self.radii (V, P)."""
        self._check_points(means3D)
        dev = self.device
        means = _f32("means3D", means3D, dev)
        opac = _f32("opacities", opacities, dev)
        sc = _f32("scales", scales, dev)
        ro = _f32("rotations", rotations, dev)
        cp = _f32("colors_precomp", colors_precomp, dev)
        dcc = _f32("dc", dc, dev)
        shc = _f32("shs", shs, dev)
        M = shc.size(1) if shc.numel() else 0
        cull = 0
        if culling is not None and culling.numel():
            cull_t = culling.to(device=dev, dtype=torch.uint8).contiguous()
            self._cull = cull_t  # keep alive for graph replays
            cull = cull_t.data_ptr()
        _lib.call("fgs_render_batched_fwd", self.P, int(sh_degree), int(M), _ptr(means), _ptr(cp), _ptr(dcc),
                  _ptr(shc), _ptr(opac), _ptr(sc), _ptr(ro), cull, self.V, self._cams, C.byref(self._cfg),
                  self.pair_capacity, _ptr(self.workspace), self.workspace.numel(), _ptr(self.out_color),
                  _ptr(self.radii), _stream(dev))
        return self.out_color

    def alloc_grads(self, sh_coeffs: int) -> dict:
        """Gradient tensors for backward(out=...), shaped like FB's outputs."""
        f = dict(dtype=torch.float32, device=self.device)
        P = self.P
        return dict(means3D=torch.zeros((P, 3), **f), dc=torch.zeros((P, 1, 3), **f),
                    shs=torch.zeros((P, sh_coeffs, 3), **f), opacities=torch.zeros((P, 1), **f),
                    scales=torch.zeros((P, 3), **f), rotations=torch.zeros((P, 4), **f),
                    colors=torch.zeros((P, 3), **f), cov3D=torch.zeros((P, 6), **f))

    def backward(self, dL_dpixels, means3D, dc=None, shs=None, scales=None, rotations=None, sh_degree=0,
                 xyz_gradient_accum=None, xyz_gradient_accum_abs=None, max_radii=None, denom=None,
                 out: dict | None = None) -> dict:
        """Backward of the last forward; returns (or fills) the gradient dict of alloc_grads."""
        self._check_points(means3D)
        dev = self.device
        dL = _f32("dL_dpixels", dL_dpixels, dev)
        if dL.numel() != self.out_color.numel():
            raise ValueError("dL_dpixels must match the flat colour buffer")
        means = _f32("means3D", means3D, dev)
        dcc = _f32("dc", dc, dev)
        shc = _f32("shs", shs, dev)
        sc = _f32("scales", scales, dev)
        ro = _f32("rotations", rotations, dev)
        M = shc.size(1) if shc.numel() else 0
        g = out if out is not None else self.alloc_grads(M)
        stats = xyz_gradient_accum is not None and xyz_gradient_accum.numel() != 0
        _lib.call("fgs_render_batched_bwd", self.P, int(sh_degree), int(M), _ptr(means), _ptr(dcc), _ptr(shc),
                  _ptr(sc), _ptr(ro), self.V, self._cams, C.byref(self._cfg), self.pair_capacity,
                  _ptr(self.workspace), self.workspace.numel(), _ptr(self.radii), _ptr(dL), _ptr(g["means3D"]),
                  _ptr(g["dc"]), _ptr(g["shs"]), _ptr(g["opacities"]), _ptr(g["scales"]), _ptr(g["rotations"]),
                  _ptr(g["colors"]), _ptr(g["cov3D"]),
                  _ptr(xyz_gradient_accum) if stats else 0, _ptr(xyz_gradient_accum_abs) if stats else 0,
                  _ptr(max_radii) if stats else 0, _ptr(denom) if stats else 0, _stream(dev))
        return g


    def backward_adam(self, dL_dpixels, means3D, shs, opacities, scales, rotations, sh_degree, fused,
                      xyz_gradient_accum=None, xyz_gradient_accum_abs=None, max_radii=None, denom=None) -> None:
        """Backward of the last forward with the sparse Adam step fused (``fused``: an
        ``_lib.AdamFused`` from ``SparseGaussianAdam``): gradients summed over the cameras step the
        raw parameters of every Gaussian some camera saw; no gradient tensor is written."""
        self._check_points(means3D)
        dev = self.device
        dL = _f32("dL_dpixels", dL_dpixels, dev)
        if dL.numel() != self.out_color.numel():
            raise ValueError("dL_dpixels must match the flat colour buffer")
        means = _f32("means3D", means3D, dev)
        shc = _f32("shs", shs, dev)
        op = _f32("opacities", opacities, dev)
        sc = _f32("scales", scales, dev)
        ro = _f32("rotations", rotations, dev)
        M = shc.size(1) if shc.numel() else 0
        stats = xyz_gradient_accum is not None and xyz_gradient_accum.numel() != 0
        _lib.call("fgs_render_batched_bwd_adam", self.P, int(sh_degree), int(M), _ptr(means), _ptr(shc), _ptr(op),
                  _ptr(sc), _ptr(ro), self.V, self._cams, C.byref(self._cfg), self.pair_capacity,
                  _ptr(self.workspace), self.workspace.numel(), _ptr(self.radii), _ptr(dL), C.byref(fused),
                  _ptr(xyz_gradient_accum) if stats else 0, _ptr(xyz_gradient_accum_abs) if stats else 0,
                  _ptr(max_radii) if stats else 0, _ptr(denom) if stats else 0, _stream(dev))


class _RasterizeBatched(torch.autograd.Function):
    """Autograd over one batched frame: returns the flat colour buffer and radii (V, P)."""

    @staticmethod
    def forward(ctx, rast, sh_degree, means3D, dc, shs, colors_precomp, opacities, scales, rotations, culling,
                xyz_gradient_accum, xyz_gradient_accum_abs, max_radii, denom):
        rast.forward(means3D, opacities, dc, shs, colors_precomp, scales, rotations, culling, sh_degree)
        ctx.rast = rast
        ctx.sh_degree = sh_degree
        ctx.precomp = colors_precomp is not None and colors_precomp.numel() != 0
        ctx.save_for_backward(means3D, dc, shs, scales, rotations, xyz_gradient_accum, xyz_gradient_accum_abs,
                              max_radii, denom)
        return rast.out_color.clone(), rast.radii.clone()

    @staticmethod
    def backward(ctx, grad_color, _):
        means3D, dc, shs, scales, rotations, acc, acc_abs, mr, den = ctx.saved_tensors
        g = ctx.rast.backward(grad_color.contiguous(), means3D, dc, shs, scales, rotations, ctx.sh_degree, acc,
                              acc_abs, mr, den)
        gc = g["colors"] if ctx.precomp else None
        gdc = None if ctx.precomp else g["dc"]
        gsh = None if ctx.precomp else g["shs"]
        return (None, None, g["means3D"], gdc, gsh, gc, g["opacities"], g["scales"], g["rotations"], None, None,
                None, None, None)


def rasterize_batched(rast: BatchedRasterizer, means3D, opacities, dc=None, shs=None, colors_precomp=None,
                      scales=None, rotations=None, culling=None, sh_degree=0, xyz_gradient_accum=None,
                      xyz_gradient_accum_abs=None, max_radii=None, denom=None):
    """Differentiable batched render: (list of (3,H_k,W_k) images, radii (V, P))."""
    empty = torch.empty(0, device=means3D.device)
    flat, radii = _RasterizeBatched.apply(
        rast, sh_degree, means3D, empty if dc is None else dc, empty if shs is None else shs,
        empty if colors_precomp is None else colors_precomp, opacities, scales, rotations, culling,
        empty if xyz_gradient_accum is None else xyz_gradient_accum,
        empty if xyz_gradient_accum_abs is None else xyz_gradient_accum_abs,
        empty if max_radii is None else max_radii, empty if denom is None else denom)
    return rast.images(flat), radii


class CapturedStep:
    """One forward + backward of a BatchedRasterizer captured in a CUDA graph.

    The parameter tensors, dL_dpixels and the statistics tensors are static:
    update them in place between ``replay()`` calls.  Gradients land in
    ``self.grads`` (summed over cameras), images in ``rast.out_color``.

    With ``adam`` (a SparseGaussianAdam whose groups are named xyz, f_dc,
    f_rest, opacity, scaling, rotation) the graph is a whole training step on
    the optimiser's raw tensors: the activations (sigmoid, exp, normalize)
    into static buffers, the forward, and the backward with the sparse Adam
    step fused; ``params`` may then be None.  Each ``replay()`` advances the
    optimiser's step counts and writes the new step sizes into the graph's
    step-size table first.  Re-capture after densification (new tensors).

    Overflow: the graph keeps the largest pair count of its replays on the
    device and copies it to pinned host memory at the end of every replay, so
    no replay synchronises.  ``replay()`` raises ``BatchOverflow`` when an
    earlier replay that has completed needed more pairs than the workspace
    holds (its extra pairs were dropped, nothing was written past a buffer);
    ``check()`` waits for the last replay and raises the same way.  Recover
    with ``rast.fit(...)`` and a new CapturedStep.
    """

    def __init__(self, rast: BatchedRasterizer, params: dict | None, dL_dpixels: torch.Tensor, sh_degree: int = 0,
                 stats: dict | None = None, with_backward: bool = True, adam=None):
        self.rast = rast
        self.dL = dL_dpixels
        self.sh_degree = sh_degree
        self.stats = stats or {}
        self.with_backward = with_backward
        self.adam = adam
        if adam is not None:
            self._bind_adam(adam)
        else:
            self.params = params
        shs = self.params.get("shs")
        self.grads = rast.alloc_grads(shs.size(1) if shs is not None and shs.numel() else 0) if adam is None else {}
        self._pairs_word = rast.pair_count_word()
        self._pairs_max = torch.zeros(1, dtype=torch.int32, device=rast.device)
        self._pairs_host = torch.zeros(1, dtype=torch.int32).pin_memory()
        self._capacity = rast.pair_capacity
        # Warm up on a side stream (first-call runtime setup must not be captured);
        # the warm-up never steps the optimiser.
        side = torch.cuda.Stream(device=rast.device)
        side.wait_stream(torch.cuda.current_stream(rast.device))
        with torch.cuda.stream(side):
            self._body(warmup=True)
        torch.cuda.current_stream(rast.device).wait_stream(side)
        torch.cuda.synchronize(rast.device)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._body()

    def _bind_adam(self, adam):
        named = adam._named()
        missing = {"xyz", "opacity", "scaling", "rotation"} - set(named)
        if missing:
            raise ValueError(f"the optimiser has no group named {sorted(missing)}")
        raw = {n: g["params"][0] for n, g in named.items()}
        self._raw = raw
        P, dev = self.rast.P, self.rast.device
        self.params = dict(means3D=raw["xyz"], dc=raw.get("f_dc"), shs=raw.get("f_rest"),
                           opacities=torch.empty((P, 1), dtype=torch.float32, device=dev),
                           scales=torch.empty((P, 3), dtype=torch.float32, device=dev),
                           rotations=torch.empty((P, 4), dtype=torch.float32, device=dev))
        adam._check_fused(raw["xyz"], raw.get("f_dc"), raw.get("f_rest"), None)
        # step sizes: pinned host slots copied into a device table the graph reads;
        # a slot is rewritten only after its previous copy has completed
        self._lr = torch.zeros(6, dtype=torch.float32, device=dev)
        self._lr_host = [torch.zeros(6, dtype=torch.float32).pin_memory() for _ in range(4)]
        self._lr_done = [None] * 4
        self._replays = 0
        self._fused = adam._fused_args(P, dev, advance=False, lr_device=self._lr)[0]

    @torch.no_grad()
    def _activations(self):
        p, raw, acts = self.params, self._raw, self.adam.activations
        op, sc, ro = raw["opacity"], raw["scaling"], raw["rotation"]
        if acts["opacity"] == "sigmoid":
            torch.sigmoid(op, out=p["opacities"])
        else:
            p["opacities"].copy_(op)
        if acts["scaling"] == "exp":
            torch.exp(sc, out=p["scales"])
        else:
            p["scales"].copy_(sc)
        if acts["rotation"] == "normalize":
            torch.nn.functional.normalize(ro, dim=-1, out=p["rotations"])
        else:
            p["rotations"].copy_(ro)

    def _body(self, warmup: bool = False):
        p = self.params
        if self.adam is not None:
            self._activations()
        self.rast.forward(p["means3D"], p["opacities"], p.get("dc"), p.get("shs"), p.get("colors_precomp"),
                          p["scales"], p["rotations"], p.get("culling"), self.sh_degree)
        if not warmup:  # sticky largest pair count, read by the host without a synchronisation
            torch.maximum(self._pairs_max, self._pairs_word, out=self._pairs_max)
            self._pairs_host.copy_(self._pairs_max, non_blocking=True)
        if not self.with_backward:
            return
        st = self.stats
        if self.adam is None:
            self.rast.backward(self.dL, p["means3D"], p.get("dc"), p.get("shs"), p["scales"], p["rotations"],
                               self.sh_degree, st.get("xyz_gradient_accum"), st.get("xyz_gradient_accum_abs"),
                               st.get("max_radii"), st.get("denom"), out=self.grads)
        elif warmup:  # the fused kernel with no group to step and no statistics: sets up, changes nothing
            self.rast.backward_adam(self.dL, p["means3D"], p.get("shs"), p["opacities"], p["scales"],
                                    p["rotations"], self.sh_degree, _lib.AdamFused())
        else:
            self.rast.backward_adam(self.dL, p["means3D"], p.get("shs"), p["opacities"], p["scales"],
                                    p["rotations"], self.sh_degree, self._fused, st.get("xyz_gradient_accum"),
                                    st.get("xyz_gradient_accum_abs"), st.get("max_radii"), st.get("denom"))

    def _raise_if_overflowed(self) -> None:
        pairs = int(self._pairs_host[0])
        if pairs > self._capacity:
            raise BatchOverflow(pairs, self._capacity)

    def check(self) -> None:
        """Wait for the last replay; raise BatchOverflow if any replay so far overflowed."""
        torch.cuda.current_stream(self.rast.device).synchronize()
        self._raise_if_overflowed()

    def replay(self):
        self._raise_if_overflowed()
        if self.adam is not None:
            fused, _, lrs = self.adam._fused_args(self.rast.P, self.rast.device, lr_device=self._lr)
            for g in range(6):
                if fused.param[g] != self._fused.param[g] or fused.exp_avg[g] != self._fused.exp_avg[g]:
                    raise RuntimeError("the optimiser's tensors changed since capture: build a new CapturedStep")
            slot = self._replays % len(self._lr_host)
            if self._lr_done[slot] is not None:
                self._lr_done[slot].synchronize()
            self._lr_host[slot].copy_(lrs)
            self._lr.copy_(self._lr_host[slot], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(torch.cuda.current_stream(self.rast.device))
            self._lr_done[slot] = ev
            self._replays += 1
        self.graph.replay()
