"""PLY files and camera construction (fastergs_gb300.ply, fastergs_gb300.cameras)
against the reference's own code: tests/golden/ply_golden.npz holds the vertex
array 3DGS's GaussianModel.save_ply hands to plyfile and the tensors its
load_ply builds back (SH degrees 1 and 3); camera_golden.npz and
camera_ts_golden.npz hold getWorld2View2 / getProjectionMatrix composed as
3DGS/scene/cameras.py:54-57, without and with a translate / scale.  The PLY
layout must match bit for bit; camera matrices within 1e-6."""
from pathlib import Path

import numpy as np
import pytest

from fastergs_gb300 import cameras, ply

GOLD = Path(__file__).resolve().parent / "golden"
PG = np.load(GOLD / "ply_golden.npz")


def _model(deg):
    return {k: PG[f"{k}{deg}"] for k in ("xyz", "f_dc", "f_rest", "opacity", "scaling", "rotation")}


@pytest.mark.parametrize("deg", [1, 3])
def test_property_names_match_reference(deg):
    M = (deg + 1) ** 2 - 1
    assert ply.attribute_names(3 * M) == list(PG[f"names{deg}"])


@pytest.mark.parametrize("deg", [1, 3])
def test_saved_vertices_match_reference_bit_for_bit(tmp_path, deg):
    path = tmp_path / "point_cloud.ply"
    ply.save_ply(path, _model(deg))
    v = ply.read_vertices(path)
    assert list(v.dtype.names) == list(PG[f"names{deg}"])
    got = np.stack([v[n] for n in v.dtype.names], axis=1)
    assert got.dtype == np.float32
    assert np.array_equal(got.view(np.uint32), PG[f"vertex{deg}"].view(np.uint32))
    assert path.read_bytes().startswith(b"ply\nformat binary_little_endian 1.0\nelement vertex 37\n")


@pytest.mark.parametrize("deg", [1, 3])
def test_loaded_tensors_match_reference(tmp_path, deg):
    path = tmp_path / "point_cloud.ply"
    ply.save_ply(path, _model(deg))
    got = ply.load_ply(path, max_sh_degree=deg)
    assert got["sh_degree"] == deg
    for k in ("xyz", "f_dc", "f_rest", "opacity", "scaling", "rotation"):
        ref = PG[f"loaded_{k}{deg}"]
        assert got[k].shape == ref.shape and got[k].dtype == np.float32, k
        assert np.array_equal(got[k], ref), k


def _write_variant(path, names, data, fmt):
    head = ["ply", f"format {fmt} 1.0", "comment written by the test", f"element vertex {data.shape[0]}"]
    head += [f"property float {n}" for n in names] + ["end_header"]
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode())
        if fmt == "ascii":
            for row in data:
                f.write((" ".join(repr(float(x)) for x in row) + "\n").encode())
        else:
            np.ascontiguousarray(data, dtype=">f4" if fmt == "binary_big_endian" else "<f4").tofile(f)


@pytest.mark.parametrize("fmt", ["binary_big_endian", "ascii"])
def test_other_encodings_read_the_same(tmp_path, fmt):
    names, data = list(PG["names1"]), PG["vertex1"]
    _write_variant(tmp_path / "v.ply", names, data, fmt)
    got = ply.load_ply(tmp_path / "v.ply")
    for k in ("xyz", "f_rest", "rotation"):
        assert np.array_equal(got[k], PG[f"loaded_{k}1"]), k


def test_bad_files_are_rejected(tmp_path):
    names = list(PG["names1"])
    _write_variant(tmp_path / "a.ply", names[:-9] + names[-8:], np.delete(PG["vertex1"], len(names) - 9, axis=1),
                   "binary_little_endian")  # one f_rest value short
    with pytest.raises(ValueError):
        ply.load_ply(tmp_path / "a.ply")
    ply.save_ply(tmp_path / "b.ply", _model(1))
    with pytest.raises(ValueError):
        ply.load_ply(tmp_path / "b.ply", max_sh_degree=3)
    (tmp_path / "c.ply").write_bytes(b"not a ply\n")
    with pytest.raises(ValueError):
        ply.read_vertices(tmp_path / "c.ply")
    data = PG["vertex1"]
    _write_variant(tmp_path / "d.ply", names, data, "binary_little_endian")
    raw = (tmp_path / "d.ply").read_bytes()
    (tmp_path / "d.ply").write_bytes(raw[:-16])  # truncated body
    with pytest.raises(ValueError):
        ply.read_vertices(tmp_path / "d.ply")


def test_camera_construction_matches_reference():
    g = np.load(GOLD / "camera_golden.npz")
    for i in range(g["R"].shape[0]):
        cam = cameras.camera_from_rt(g["R"][i], g["T"][i], float(g["fovx"][i]), float(g["fovy"][i]), 640, 480)
        np.testing.assert_allclose(cam.viewmatrix, g["world_view"][i], rtol=0, atol=1e-6)
        np.testing.assert_allclose(cam.projmatrix, g["full_proj"][i], rtol=0, atol=2e-6)
        np.testing.assert_allclose(cam.campos, g["center"][i], rtol=0, atol=2e-6)
    t = np.load(GOLD / "camera_ts_golden.npz")
    for i in range(t["R"].shape[0]):
        cam = cameras.camera_from_rt(t["R"][i], t["T"][i], float(t["fovx"][i]), float(t["fovy"][i]), 640, 480,
                                     translate=t["translate"][i], scale=float(t["scale"][i]))
        np.testing.assert_allclose(cam.viewmatrix, t["world_view"][i], rtol=0, atol=1e-5)
        np.testing.assert_allclose(cam.projmatrix, t["full_proj"][i], rtol=0, atol=1e-5)
        np.testing.assert_allclose(cam.campos, t["center"][i], rtol=0, atol=1e-5)
