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
