"""The rasterizer under the reference backend's own import name.

``from diff_gaussian_rasterization_faster import GaussianRasterizationSettings,
GaussianRasterizer`` is what every FasterGS backbone's ``--fastergs`` path
does (e.g. ``3DGS/gaussian_renderer/render_faster.py``); with this repository
on ``sys.path`` (or installed) those lines load this GB300 rasterizer
unchanged.  The Python classes are ``fastergs_gb300``'s; ``_C`` is the
compiled PyTorch extension (``fastergs_gb300/csrc/torch_ops.cpp``) whose
``ops`` carry the reference binding's names and arguments
(FB ``csrc/pybind.cpp:371-416``) over the C ABI of ``libfgs.so``.
"""
from fastergs_gb300 import (Buffer, GaussianRasterizationSettings, GaussianRasterizer, SparseGaussianAdam,
                            _RasterizeGaussians, cpu_deep_copy_tuple, rasterize_gaussians)

from . import _C

__all__ = ["Buffer", "GaussianRasterizationSettings", "GaussianRasterizer", "SparseGaussianAdam",
           "_RasterizeGaussians", "cpu_deep_copy_tuple", "rasterize_gaussians", "_C"]
