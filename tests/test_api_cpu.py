"""CPU tests of the Python surface: names, settings fields, validation and
the no-fallback contract."""
import numpy as np
import pytest
import torch

import fastergs_gb300 as fgs
from fastergs_gb300 import _C, scenes


def test_public_names_mirror_the_reference():
    for name in ("GaussianRasterizationSettings", "GaussianRasterizer", "rasterize_gaussians", "Buffer",
                 "SparseGaussianAdam", "_RasterizeGaussians"):
        assert hasattr(fgs, name)
    for op in ("preprocess", "sort_gaussian", "get_sort_buffer_size", "render_16x16", "backward", "adamUpdate",
               "render_simp", "render_depth"):
        assert callable(getattr(_C.ops, op))
    assert fgs.GaussianRasterizationSettings._fields == (
        "image_height", "image_width", "tanfovx", "tanfovy", "bg", "scale_modifier", "viewmatrix", "projmatrix",
        "sh_degree", "campos", "mult", "prefiltered", "debug")


def test_validation_raises_like_the_reference():
    r = fgs.GaussianRasterizer(None)
    m = torch.zeros(4, 3)
    with pytest.raises(Exception, match="one of either SHs"):
        r(means3D=m, opacities=m[:, :1])
    with pytest.raises(Exception, match="one of either SHs"):
        r(means3D=m, opacities=m[:, :1], shs=m, colors_precomp=m)
    with pytest.raises(Exception, match="scale/rotation pair"):
        r(means3D=m, opacities=m[:, :1], shs=m)


def test_cpu_tensors_are_refused_not_emulated():
    t = torch.zeros(4, 1)
    with pytest.raises(ValueError, match="CUDA"):
        _C.ops.preprocess(0, t, t, t, t, t, t, t, 1.0, 16, 16, 16, 16, t, t, t, 1.0, 1.0, 100.0, 0.01, t, t, t, t,
                          1.0, t, t)


def test_auxiliary_passes_are_bound_with_fb_signatures():
    import inspect
    assert list(inspect.signature(_C.ops.render_simp).parameters) == [
        "P", "num_rendered", "width", "height", "splat_buffer", "gaussian_keys_sorted", "gaussian_values_sorted",
        "ranges"]
    assert list(inspect.signature(_C.ops.render_depth).parameters)[-5:] == [
        "means3D", "scales", "rotations", "proj_matrix", "campos"]
    from fastergs_gb300 import GaussianRasterizer
    assert callable(GaussianRasterizer.render_simp) and callable(GaussianRasterizer.render_depth)


def test_scenes_are_seeded_and_shaped():
    a, b = scenes.scene_c1(seed=0), scenes.scene_c1(seed=0)
    assert np.array_equal(a.means, b.means) and a.P == 10_000
    c = scenes.scene_c2(P=1000)
    assert c.shs.shape == (1000, 15, 3) and c.camera.width == 1297 and c.camera.height == 840
    assert c.means[:, 2].min() >= 2 and c.means[:, 2].max() <= 12
    cams = scenes.cameras_c4()
    assert len(cams) == 16
    assert {(k.width, k.height) for k in cams} <= set(scenes.C4_RESOLUTIONS)
    m, sc, rot, op, dc, shs = c.activated()
    np.testing.assert_allclose(np.linalg.norm(rot, axis=1), 1, rtol=1e-6)
    assert np.all((op > 0) & (op < 1))


def test_reference_import_name_loads_the_compiled_extension():
    # every backbone's --fastergs path does exactly this import (3DGS/gaussian_renderer/render_faster.py:16)
    import __graft_entry__
    __graft_entry__.build()
    import diff_gaussian_rasterization_faster as drf
    from diff_gaussian_rasterization_faster import GaussianRasterizationSettings, GaussianRasterizer  # noqa: F401
    assert drf.GaussianRasterizer is fgs.GaussianRasterizer
    assert drf._RasterizeGaussians is fgs._RasterizeGaussians
    assert drf._C.__file__.endswith(".so"), "the _C of the drop-in package is the compiled extension"
    for op in ("preprocess", "sort_gaussian", "get_sort_buffer_size", "render_16x16", "backward", "adamUpdate",
               "render_simp", "render_depth"):
        assert callable(getattr(drf._C.ops, op))
    assert drf._C.ops.get_sort_buffer_size(1 << 20) == _C.ops.get_sort_buffer_size(1 << 20)
    t = torch.zeros(4, 1)
    with pytest.raises(ValueError, match="CUDA"):
        drf._C.ops.preprocess(0, t, t, t, t, t, t, t, 1.0, 16, 16, 16, 16, t, t, t, 1.0, 1.0, 100.0, 0.01, t, t, t,
                              t, 1.0, t, t)
    out = drf.cpu_deep_copy_tuple((t, 3, "x"))
    assert out[1:] == (3, "x") and out[0] is not t
