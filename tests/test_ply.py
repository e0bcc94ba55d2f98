"""The binary PLY writer: header and element layout of the file plyfile
writes for i3d/meshing.py:316-384 (vertex x, y, z float32 plus optional
attributes; face vertex_indices as a uchar-counted int list)."""

import numpy as np


def _read(path):
    data = open(path, "rb").read()
    end = data.index(b"end_header\n") + len(b"end_header\n")
    return data[:end].decode("ascii").splitlines(), data[end:]


def test_save_ply_layout_round_trip(tmp_path):
    from mplicits_gb300.meshing import save_ply
    rng = np.random.default_rng(0)
    verts = rng.standard_normal((7, 3)).astype(np.float32)
    faces = rng.integers(0, 7, (5, 3)).astype(np.int64)
    p = tmp_path / "m.ply"
    save_ply(verts, faces, str(p))
    header, body = _read(p)
    assert header == ["ply", "format binary_little_endian 1.0", "element vertex 7",
                      "property float x", "property float y", "property float z",
                      "element face 5", "property list uchar int vertex_indices", "end_header"]
    v = np.frombuffer(body[:7 * 12], "<f4").reshape(7, 3)
    assert np.array_equal(v, verts)
    f = np.frombuffer(body[7 * 12:], dtype=[("n", "u1"), ("v", "<i4", (3,))])
    assert len(f) == 5 and (f["n"] == 3).all() and np.array_equal(f["v"], faces)


def test_save_ply_vertex_attributes(tmp_path):
    from mplicits_gb300.meshing import save_ply
    verts = np.array([[0, 0, 0, 0, 0, 1], [1, 0, 0, 0, 0, 1], [0, 1, 0, 0, 0, 1]], np.float32)
    faces = np.array([[0, 1, 2]])
    p = tmp_path / "n.ply"
    save_ply(verts, faces, str(p), vertex_attributes=[("nx", "f4"), ("ny", "f4"), ("nz", "f4")])
    header, body = _read(p)
    assert header[3:9] == ["property float x", "property float y", "property float z",
                           "property float nx", "property float ny", "property float nz"]
    v = np.frombuffer(body[:3 * 24], "<f4").reshape(3, 6)
    assert np.array_equal(v, verts)


def test_save_ply_integer_and_double_attributes(tmp_path):
    """Each attribute's header type matches the bytes written for it, so a
    PLY reader recovers the values (uchar colour, int label, double weight)."""
    from mplicits_gb300.meshing import save_ply
    from mplicits_gb300.reconstruct import read_ply_points
    verts = np.array([[0.5, 0, 0, 200, -7, 0.25], [1, 0.25, 0, 3, 9, 1e-9],
                      [0, 1, -0.75, 255, 0, -2.5]], np.float64)
    faces = np.array([[0, 1, 2]])
    p = tmp_path / "a.ply"
    attrs = [("red", "u1"), ("label", "i4"), ("weight", "f8")]
    save_ply(verts, faces, str(p), vertex_attributes=attrs)
    header, body = _read(p)
    assert header[6:9] == ["property uchar red", "property int label", "property double weight"]
    dt = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("red", "u1"), ("label", "<i4"),
                   ("weight", "<f8")])
    v = np.frombuffer(body[:3 * dt.itemsize], dtype=dt)
    assert np.array_equal(v["red"], [200, 3, 255])
    assert np.array_equal(v["label"], [-7, 9, 0])
    assert np.array_equal(v["weight"], verts[:, 5])
    assert np.array_equal(read_ply_points(str(p)), verts[:, :3].astype(np.float32))


def test_save_ply_rejects_types_ply_cannot_name(tmp_path):
    import pytest
    from mplicits_gb300.meshing import save_ply
    with pytest.raises(ValueError):
        save_ply(np.zeros((3, 4)), np.array([[0, 1, 2]]), str(tmp_path / "b.ply"),
                 vertex_attributes=[("t", "i8")])
