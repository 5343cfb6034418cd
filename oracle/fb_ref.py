"""The reference CUDA backend (FB), built out of tree for sm_103a -- TEST AND BENCH INFRASTRUCTURE ONLY.

FB is ``gs_submodules/diff-gaussian-rasterization_faster`` of FasterGS: the
rasterizer this repository replaces.  It is built here only to pin the oracle
and the product against FB's own outputs, and to time FB beside the product
on the same GPU.  Nothing under ``fastergs_gb300/`` imports this module.

Recipe (no use of FB's own ``setup.py``):

* ``stage()``   copies FB's ``csrc/`` and its Python package from the FasterGS
  checkout named by the ``FASTERGS_REF`` environment variable (required) into
  ``oracle/_ref/fb_src`` and applies the one change CUDA 13 needs:
  ``cub::Max()`` -> ``cuda::maximum<>()`` in ``csrc/cuda_rasterizer/render.cu:387``
  (CCCL 3 removed ``cub::Max``).  ``oracle/_ref`` is git-ignored; the staged
  copy is a build input that never enters the history.
* ``build()``   compiles every ``csrc/cuda_rasterizer/*.cu`` with nvcc
  (``-gencode arch=compute_103a,code=sm_103a -O3``, FB's own nvcc flags minus
  ``-Xptxas=-v``) and ``csrc/pybind.cpp`` with g++ in parallel, against the
  installed torch's headers, and links ``_C`` as a Python extension into
  ``oracle/_ref/fb/diff_gaussian_rasterization_faster/``.  It works on any host
  with nvcc, g++ and torch; the object files are per-machine, so a host of
  another architecture rebuilds from the staged sources.
* ``load()``    imports FB's unmodified Python package under the module name
  ``fb_reference`` (so it never shadows the product's drop-in package of the
  same import name).  Importing it allocates FB's class-wide ``Buffer``
  (2^24 pairs, about 2.6 GB) on the current CUDA device, as FB does.

FB writes past its pair buffer when a frame needs 2^24 or more (tile, Gaussian)
pairs (FB ``__init__.py:117-119`` checks only after ``preprocess`` wrote them);
callers run it only on frames whose pair count stays below that.

Usage: ``FASTERGS_REF=<FasterGS checkout> python oracle/fb_ref.py stage`` (here),
then ``python oracle/fb_ref.py build`` (on the machine that runs it).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import importlib.util
import os
import platform
import shutil
import subprocess
import sys
import sysconfig
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF = HERE / "_ref"
SRC = REF / "fb_src"
OUT = REF / "fb"
PKG = OUT / "diff_gaussian_rasterization_faster"
OBJ = REF / "fb_obj"
FB_SUBDIR = Path("gs_submodules") / "diff-gaussian-rasterization_faster"
SHIM_FILE = Path("csrc") / "cuda_rasterizer" / "render.cu"
SHIM_FROM = "cub::Max()"
SHIM_TO = "cuda::maximum<>()"
MODULE = "fb_reference"

_mod = None


def _ext_suffix() -> str:
    return sysconfig.get_config_var("EXT_SUFFIX") or ".so"


def lib_path() -> Path:
    return PKG / ("_C" + _ext_suffix())


def staged() -> bool:
    return (SRC / "csrc" / "pybind.cpp").exists() and (SRC / "diff_gaussian_rasterization_faster").exists()


def stage(ref: str | None = None) -> Path:
    """Copy FB's sources from the FasterGS checkout into oracle/_ref/fb_src, shim applied."""
    ref = ref or os.environ.get("FASTERGS_REF")
    if not ref:
        raise RuntimeError("set FASTERGS_REF to the FasterGS checkout that holds " + str(FB_SUBDIR))
    src = Path(ref) / FB_SUBDIR
    if not (src / "csrc" / "pybind.cpp").exists():
        raise RuntimeError(f"{src} does not hold FB's sources")
    if SRC.exists():
        shutil.rmtree(SRC)
    SRC.mkdir(parents=True)
    shutil.copytree(src / "csrc", SRC / "csrc")
    shutil.copytree(src / "diff_gaussian_rasterization_faster", SRC / "diff_gaussian_rasterization_faster")
    for p in SRC.rglob("*"):
        if p.is_file():
            p.chmod(0o644)
    f = SRC / SHIM_FILE
    text = f.read_text()
    if text.count(SHIM_FROM) != 1:
        raise RuntimeError(f"expected one {SHIM_FROM} in {SHIM_FILE}, found {text.count(SHIM_FROM)}")
    f.write_text(text.replace(SHIM_FROM, SHIM_TO))
    return SRC


def _stamp() -> str:
    h = hashlib.sha256()
    for p in sorted(SRC.rglob("*")):
        if p.is_file() and p.suffix in (".cu", ".h", ".cpp", ".py", ".hpp", ".inl"):
            h.update(p.relative_to(SRC).as_posix().encode())
            h.update(p.read_bytes())
    h.update(platform.machine().encode())
    h.update(Path(__file__).read_bytes())
    return h.hexdigest()


def built() -> bool:
    st = PKG / ".stamp"
    return lib_path().exists() and st.exists() and staged() and st.read_text() == _stamp()


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile FB for sm_103a from the staged sources (see the module docstring)."""
    if not staged():
        raise RuntimeError("FB sources are not staged (run oracle/fb_ref.py stage with FASTERGS_REF set)")
    if not force and built():
        return lib_path()
    import torch.utils.cpp_extension as ce

    nvcc = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cuda_home = ce.CUDA_HOME or "/usr/local/cuda"
    incs = [*ce.include_paths(), sysconfig.get_paths()["include"], str(SRC / "csrc"), str(Path(cuda_home) / "include")]
    abi = getattr(ce, "_get_pybind11_abi_build_flags", lambda: [])()
    import torch
    defs = ["-DTORCH_EXTENSION_NAME=_C", "-DTORCH_API_INCLUDE_EXTENSION_H",
            f"-D_GLIBCXX_USE_CXX11_ABI={int(torch._C._GLIBCXX_USE_CXX11_ABI)}", *abi]
    inc_flags = [f"-I{p}" for p in incs]
    nv_flags = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
                *ce.COMMON_NVCC_FLAGS, "-Xcompiler", "-fPIC", *defs, *inc_flags]
    cxx_flags = ["-O1", "-std=c++17", "-fPIC", *defs, *inc_flags]

    if OBJ.exists():
        shutil.rmtree(OBJ)
    OBJ.mkdir(parents=True)
    units = sorted((SRC / "csrc" / "cuda_rasterizer").glob("*.cu")) + [SRC / "csrc" / "pybind.cpp"]

    def compile_one(src: Path) -> Path:
        obj = OBJ / (src.stem + ".o")
        cmd = ([nvcc, *nv_flags] if src.suffix == ".cu" else [cxx, *cxx_flags]) + ["-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"FB: compiling {src.name} failed:\n{r.stdout[-4000:]}\n{r.stderr[-4000:]}")
        if verbose:
            print(f"compiled {src.name}", flush=True)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(len(units), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, units))

    if PKG.exists():
        shutil.rmtree(PKG)
    shutil.copytree(SRC / "diff_gaussian_rasterization_faster", PKG)
    libdirs = [*ce.library_paths(), str(Path(cuda_home) / "lib64")]
    tmp = lib_path().with_suffix(".tmp")
    cmd = [cxx, "-shared", "-o", str(tmp), *map(str, objs), *[f"-L{d}" for d in libdirs],
           *[f"-Wl,-rpath,{d}" for d in libdirs],
           "-lc10", "-ltorch", "-ltorch_cpu", "-ltorch_python", "-lc10_cuda", "-ltorch_cuda", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"FB: link failed:\n{r.stdout[-4000:]}\n{r.stderr[-4000:]}")
    os.replace(tmp, lib_path())
    (PKG / ".stamp").write_text(_stamp())
    return lib_path()


def load():
    """FB's Python package (``GaussianRasterizer``, ``Buffer``, ``_C.ops`` ...), imported as ``fb_reference``."""
    global _mod
    if _mod is not None:
        return _mod
    if not built():
        raise RuntimeError("FB is not built for this machine (oracle/fb_ref.py build)")
    import torch  # noqa: F401  (FB's extension links against the loaded torch)
    spec = importlib.util.spec_from_file_location(MODULE, PKG / "__init__.py", submodule_search_locations=[str(PKG)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[MODULE] = mod
    try:
        spec.loader.exec_module(mod)
    except BaseException:
        sys.modules.pop(MODULE, None)
        raise
    _mod = mod
    return mod


if __name__ == "__main__":
    cmd = sys.argv[1] if len(sys.argv) > 1 else "build"
    if cmd == "stage":
        print(stage())
    elif cmd == "build":
        print(build(force="--force" in sys.argv, verbose=True))
    else:
        raise SystemExit(f"usage: {sys.argv[0]} stage|build [--force]")
