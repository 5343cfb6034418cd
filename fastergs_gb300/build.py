"""Builds libfgs.so, the sm_103a CUDA library behind the C ABI in include/fgs.h,
and the compiled ``_C`` of the drop-in package ``diff_gaussian_rasterization_faster``.

Every CUDA translation unit is compiled in parallel with one ``-gencode`` for
sm_103a and linked into ``fastergs_gb300/libfgs.so`` next to this file.
``csrc/torch_ops.cpp`` (the PyTorch extension over the C ABI, no CUDA code) is
compiled with g++ alongside them against the installed torch and linked to
libfgs.so as ``diff_gaussian_rasterization_faster/_C<ext suffix>``.  Each
build is skipped when the stamp written beside the library matches: a hash
of every source and header, the machine architecture and the nvcc version
(a library built on another machine, or by another toolkit, is rebuilt).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess
import sysconfig
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libfgs.so"
STAMP = PKG / "libfgs.so.stamp"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["preprocess.cu", "sort.cu", "render.cu", "backward.cu", "batched.cu", "aux_passes.cu", "ssim.cu",
           "capi.cu"]
EXT_SRC = CSRC / "torch_ops.cpp"
EXT_PKG = ROOT / "diff_gaussian_rasterization_faster"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libfgs.so")


def _sources() -> list[Path]:
    return [CSRC / s for s in SOURCES if (CSRC / s).exists()]


def _deps() -> list[Path]:
    return _sources() + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "fgs.h", Path(__file__)]


def _nvcc_version(cc: str) -> str:
    r = subprocess.run([cc, "--version"], capture_output=True, text=True)
    return r.stdout.strip().splitlines()[-1] if r.returncode == 0 and r.stdout.strip() else "unknown"


def stamp(cc: str | None = None) -> str:
    """Hash of the sources, headers and build script, the machine and the nvcc version."""
    h = hashlib.sha256()
    for p in sorted(_deps()):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(platform.machine().encode())
    h.update(_nvcc_version(cc or nvcc()).encode())
    return h.hexdigest()


def up_to_date() -> bool:
    if not LIB.exists() or not STAMP.exists():
        return False
    try:
        return STAMP.read_text() == stamp()
    except (OSError, RuntimeError):
        return False


def ext_path() -> Path:
    return EXT_PKG / ("_C" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))


def _ext_stamp() -> str:
    import torch
    h = hashlib.sha256()
    for p in (EXT_SRC, ROOT / "include" / "fgs.h", Path(__file__)):
        h.update(p.read_bytes())
    h.update(f"{platform.machine()} {torch.__version__} {torch._C._GLIBCXX_USE_CXX11_ABI}".encode())
    return h.hexdigest()


def _ext_stamp_path() -> Path:
    return ext_path().with_name(ext_path().name + ".stamp")


def ext_up_to_date() -> bool:
    st = _ext_stamp_path()
    try:
        return ext_path().exists() and st.exists() and st.read_text() == _ext_stamp()
    except (OSError, ImportError):
        return False


def _ext_flags():
    """Include paths, defines and libraries of a torch extension (no CUDA code)."""
    import torch
    import torch.utils.cpp_extension as ce
    cuda_home = ce.CUDA_HOME or "/usr/local/cuda"
    incs = [*ce.include_paths(), sysconfig.get_paths()["include"], str(Path(cuda_home) / "include"),
            str(ROOT / "include")]
    defs = ["-DTORCH_EXTENSION_NAME=_C", "-DTORCH_API_INCLUDE_EXTENSION_H",
            f"-D_GLIBCXX_USE_CXX11_ABI={int(torch._C._GLIBCXX_USE_CXX11_ABI)}"]
    libdirs = [*ce.library_paths(), str(Path(cuda_home) / "lib64")]
    return [f"-I{p}" for p in incs] + defs, libdirs


def _compile_ext(verbose: bool) -> Path:
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cflags, _ = _ext_flags()
    obj = OBJ / "torch_ops.o"
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-fPIC", *cflags, "-c", str(EXT_SRC), "-o", str(obj)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed on {EXT_SRC.name}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout, r.stderr)
    return obj


def _link_ext(obj: Path) -> Path:
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    _, libdirs = _ext_flags()
    out = ext_path()
    tmp = out.with_name(out.name + ".tmp")
    # libfgs.so is found next to the package at run time ($ORIGIN-relative), torch's libraries by path
    cmd = [cxx, "-shared", "-o", str(tmp), str(obj), f"-L{PKG}", "-lfgs", *[f"-L{d}" for d in libdirs],
           "-Wl,-rpath,$ORIGIN/../fastergs_gb300", *[f"-Wl,-rpath,{d}" for d in libdirs],
           "-lc10", "-ltorch", "-ltorch_cpu", "-ltorch_python", "-lc10_cuda", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of {out.name} failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    _ext_stamp_path().write_text(_ext_stamp())
    return out


def build(force: bool = False, verbose: bool = False) -> Path:
    lib_ok = not force and up_to_date()
    ext_ok = lib_ok and not force and ext_up_to_date()
    if lib_ok and ext_ok:
        return LIB
    OBJ.mkdir(exist_ok=True)
    if lib_ok:
        _link_ext(_compile_ext(verbose))
        return LIB
    cc = nvcc()
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(ROOT / "include")]

    def compile_one(src: Path) -> Path:
        obj = OBJ / (src.stem + ".o")
        cmd = [cc, *flags, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs) + 1, os.cpu_count() or 4)) as ex:
        ext_obj = ex.submit(_compile_ext, verbose)
        objs = list(ex.map(compile_one, srcs))
        ext_obj = ext_obj.result()
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of libfgs.so failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    STAMP.write_text(stamp(cc))
    _link_ext(ext_obj)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
