"""3DGS point-cloud files: read and write the PLY layout FasterGS's backbones
save trained models in, so that a trained scene can be rendered and
benchmarked here directly.

Layout (3DGS/scene/gaussian_model.py:177-208 construct_list_of_attributes /
save_ply, read back by load_ply :215-256): one ``vertex`` element, float32
properties in the order

    x y z  nx ny nz  f_dc_0..2  f_rest_0..3M-1  opacity  scale_0..2  rot_0..3

with f_dc / f_rest channel-major (f_rest_{c M + k} is coefficient k of colour
channel c; the model holds them as (P, M, 3)), opacity the pre-sigmoid logit,
scale the log scale and rot the raw quaternion (w, x, y, z); the normals are
zero.  The reader accepts binary little- or big-endian and ASCII bodies and
any scalar property types; the writer emits binary little-endian float32,
as plyfile does for the reference.
"""
from __future__ import annotations

import os
from pathlib import Path

import numpy as np

_PLY_TYPES = {"char": "i1", "int8": "i1", "uchar": "u1", "uint8": "u1", "short": "i2", "int16": "i2",
              "ushort": "u2", "uint16": "u2", "int": "i4", "int32": "i4", "uint": "u4", "uint32": "u4",
              "float": "f4", "float32": "f4", "double": "f8", "float64": "f8"}


def attribute_names(sh_rest: int) -> list[str]:
    """Property names for sh_rest = 3 M f_rest values (construct_list_of_attributes)."""
    names = ["x", "y", "z", "nx", "ny", "nz", "f_dc_0", "f_dc_1", "f_dc_2"]
    names += [f"f_rest_{i}" for i in range(sh_rest)]
    names += ["opacity", "scale_0", "scale_1", "scale_2", "rot_0", "rot_1", "rot_2", "rot_3"]
    return names


def _read_header(f):
    if f.readline().strip() != b"ply":
        raise ValueError("not a PLY file")
    fmt, elements, cur = None, [], None
    while True:
        line = f.readline()
        if not line:
            raise ValueError("PLY header has no end_header")
        tok = line.decode("ascii", "replace").split()
        if not tok or tok[0] in ("comment", "obj_info"):
            continue
        if tok[0] == "format":
            fmt = tok[1]
        elif tok[0] == "element":
            cur = {"name": tok[1], "count": int(tok[2]), "props": []}
            elements.append(cur)
        elif tok[0] == "property":
            if cur is None:
                raise ValueError("PLY property outside an element")
            if tok[1] == "list":
                cur["props"].append((tok[-1], None))  # list property: unsupported for vertices
            else:
                if tok[1] not in _PLY_TYPES:
                    raise ValueError(f"unknown PLY property type {tok[1]}")
                cur["props"].append((tok[2], _PLY_TYPES[tok[1]]))
        elif tok[0] == "end_header":
            break
    if fmt not in ("binary_little_endian", "binary_big_endian", "ascii"):
        raise ValueError(f"unsupported PLY format {fmt}")
    return fmt, elements


def read_vertices(path: str | os.PathLike) -> np.ndarray:
    """The vertex element of a PLY file as a structured array (native byte order)."""
    with open(path, "rb") as f:
        fmt, elements = _read_header(f)
        if not elements or elements[0]["name"] != "vertex":
            raise ValueError("the first PLY element must be 'vertex'")
        el = elements[0]
        if any(t is None for _, t in el["props"]):
            raise ValueError("list properties in the vertex element are not supported")
        n = el["count"]
        if fmt == "ascii":
            dt = np.dtype([(name, t) for name, t in el["props"]])
            rows = [f.readline().split() for _ in range(n)]
            out = np.empty(n, dtype=dt)
            for j, (name, t) in enumerate(el["props"]):
                out[name] = np.array([r[j] for r in rows], dtype=t)
            return out
        order = "<" if fmt == "binary_little_endian" else ">"
        dt = np.dtype([(name, order + t) for name, t in el["props"]])
        data = np.fromfile(f, dtype=dt, count=n)
        if data.shape[0] != n:
            raise ValueError("PLY body is shorter than its header says")
        return data.astype(dt.newbyteorder("="))


def _read_float_matrix(path):
    """(property names, (P, F) float32 body) when the vertex element is the file's only element
    and all its properties are float32 in a binary body (what 3DGS writes), else None."""
    with open(path, "rb") as f:
        fmt, elements = _read_header(f)
        if fmt == "ascii" or len(elements) != 1 or elements[0]["name"] != "vertex":
            return None
        el = elements[0]
        if any(t != "f4" for _, t in el["props"]):
            return None
        n, F = el["count"], len(el["props"])
        body = np.fromfile(f, dtype=("<f4" if fmt == "binary_little_endian" else ">f4"), count=n * F)
        if body.size != n * F:
            raise ValueError("PLY body is shorter than its header says")
        return [name for name, _ in el["props"]], body.reshape(n, F).astype(np.float32, copy=False)


def load_ply(path: str | os.PathLike, max_sh_degree: int | None = None) -> dict:
    """Raw parameters of a 3DGS PLY file, laid out as GaussianModel holds them after load_ply
    (gaussian_model.py:215-256): xyz (P,3), f_dc (P,1,3), f_rest (P,M,3), opacity (P,1) logits,
    scaling (P,3) log scales, rotation (P,4) raw quaternions, all float32; plus sh_degree.
    With max_sh_degree the f_rest count must be 3 (max_sh_degree + 1)^2 - 3, as the reference
    asserts."""
    fast = _read_float_matrix(path)
    if fast is not None:
        names, mat = fast
        col = {n: i for i, n in enumerate(names)}
        P = mat.shape[0]

        def f32(cols):
            if not cols:
                return np.zeros((P, 0), np.float32)
            idx = [col[c] for c in cols]
            if idx == list(range(idx[0], idx[0] + len(idx))):  # contiguous columns: one slice
                return np.ascontiguousarray(mat[:, idx[0]:idx[0] + len(idx)])
            return np.ascontiguousarray(mat[:, idx])
    else:
        v = read_vertices(path)
        names = v.dtype.names
        P = v.shape[0]

        def f32(cols):
            if not cols:
                return np.zeros((P, 0), np.float32)
            return np.stack([np.asarray(v[c], np.float32) for c in cols], axis=1)

    def sorted_prefix(prefix):
        return sorted((n for n in names if n.startswith(prefix)), key=lambda s: int(s.split("_")[-1]))

    rest = sorted_prefix("f_rest_")
    if len(rest) % 3:
        raise ValueError("f_rest count is not a multiple of 3")
    M = len(rest) // 3
    deg = int(round((M + 1) ** 0.5)) - 1
    if (deg + 1) ** 2 - 1 != M:
        raise ValueError(f"{len(rest)} f_rest values do not match any SH degree")
    if max_sh_degree is not None and len(rest) != 3 * (max_sh_degree + 1) ** 2 - 3:
        raise ValueError(f"file holds SH degree {deg}, expected {max_sh_degree}")
    return {
        "xyz": f32(["x", "y", "z"]),
        "f_dc": f32(["f_dc_0", "f_dc_1", "f_dc_2"]).reshape(P, 1, 3),
        "f_rest": np.ascontiguousarray(f32(rest).reshape(P, 3, M).transpose(0, 2, 1)),
        "opacity": f32(["opacity"]),
        "scaling": f32(sorted_prefix("scale_")),
        "rotation": f32(sorted_prefix("rot")),
        "sh_degree": deg,
    }


def save_ply(path: str | os.PathLike, params: dict) -> None:
    """Writes raw parameters (the dict load_ply returns; arrays or tensors) in the 3DGS layout,
    binary little-endian float32 (gaussian_model.py:191-208)."""
    def arr(k):
        a = params[k]
        if hasattr(a, "detach"):
            a = a.detach().cpu().numpy()
        return np.asarray(a, np.float32)

    xyz = arr("xyz")
    P = xyz.shape[0]
    f_dc = arr("f_dc").reshape(P, -1, 3).transpose(0, 2, 1).reshape(P, -1)
    f_rest = arr("f_rest").reshape(P, -1, 3).transpose(0, 2, 1).reshape(P, -1)
    cols = [xyz, np.zeros_like(xyz), f_dc, f_rest, arr("opacity").reshape(P, 1), arr("scaling").reshape(P, 3),
            arr("rotation").reshape(P, 4)]
    body = np.ascontiguousarray(np.concatenate(cols, axis=1), dtype="<f4")
    names = attribute_names(f_rest.shape[1])
    if body.shape[1] != len(names):
        raise ValueError("parameter shapes do not form a 3DGS vertex")
    header = ["ply", "format binary_little_endian 1.0", f"element vertex {P}"]
    header += [f"property float {n}" for n in names]
    header.append("end_header")
    path = Path(path)
    if path.parent and not path.parent.exists():
        path.parent.mkdir(parents=True, exist_ok=True)
    tmp = path.with_suffix(path.suffix + ".tmp")
    with open(tmp, "wb") as f:
        f.write(("\n".join(header) + "\n").encode("ascii"))
        body.tofile(f)
    os.replace(tmp, path)


def to_device(params: dict, device="cuda", requires_grad: bool = False) -> dict:
    """torch tensors of the raw parameters on device (the GaussianModel fields after load_ply)."""
    import torch
    out = {}
    for k in ("xyz", "f_dc", "f_rest", "opacity", "scaling", "rotation"):
        t = torch.tensor(np.ascontiguousarray(params[k]), dtype=torch.float32, device=device)
        out[k] = t.requires_grad_(requires_grad)
    return out


def activated(model: dict) -> dict:
    """Rasterizer inputs from raw tensors, with the 3DGS activations (get_xyz, get_opacity =
    sigmoid, get_scaling = exp, get_rotation = normalize; gaussian_model.py:33-41)."""
    import torch
    return dict(means3D=model["xyz"], opacities=torch.sigmoid(model["opacity"]), dc=model["f_dc"],
                shs=model["f_rest"], scales=torch.exp(model["scaling"]),
                rotations=torch.nn.functional.normalize(model["rotation"], dim=-1))
