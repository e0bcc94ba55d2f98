"""The calc_deltas oracle against the reference's own loop (golden vectors)
and its point-triangle distance against float64 geometry."""

import os

import numpy as np
import pytest

from oracle import deltas as od

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "calc_deltas.npz")


def _golden():
    g = np.load(GOLDEN)
    for name in g["cases"]:
        yield str(name), {k.split("__", 1)[1]: g[k] for k in g.files if k.startswith(f"{name}__")}


@pytest.mark.parametrize("cell,fast,bvh", [(0.0, False, False), (0.03, False, False),
                                           (0.11, False, False), (0.03, True, False),
                                           (0.11, True, False), (0.004, True, False),
                                           (0.0, False, True)])
def test_oracle_equals_reference_loop(cell, fast, bvh):
    for name, c in _golden():
        # a Python float, or the float32 value of the reference's tensor
        md = float(c["max_delta"]) if str(c["max_delta_kind"]) == "float" \
            else np.float32(c["max_delta"])
        out, it = od.calc_deltas(c["vertices"], c["positions"], c["faces"], md,
                                 int(c["n_iters"]), cell=cell, fast=fast, bvh=bvh)
        assert it == int(c["iterations"]), name
        np.testing.assert_array_equal(out, c["out"], err_msg=name)


def _seg_dist(p, a, b):
    ab = b - a
    t = np.clip(np.sum((p - a) * ab, -1) / np.maximum(np.sum(ab * ab, -1), 1e-300), 0.0, 1.0)
    return np.linalg.norm(p - (a + t[..., None] * ab), axis=-1)


def _tri_dist64(p, a, b, c):
    """float64: distance to the plane where the projection falls inside,
    else the nearest of the three edges."""
    n = np.cross(b - a, c - a)
    n = n / np.linalg.norm(n, axis=-1, keepdims=True)
    h = np.sum((p - a) * n, -1)
    q = p - h[..., None] * n
    inside = True
    for u, v in ((a, b), (b, c), (c, a)):
        inside = inside & (np.sum(np.cross(v - u, q - u) * n, -1) >= 0)
    edge = np.minimum(np.minimum(_seg_dist(p, a, b), _seg_dist(p, b, c)), _seg_dist(p, c, a))
    return np.where(inside, np.abs(h), edge)


def test_triangle_distance_against_float64():
    rng = np.random.default_rng(3)
    n = 4000
    a, b, c = (rng.uniform(-1, 1, (n, 3)) for _ in range(3))
    p = rng.uniform(-1.5, 1.5, (n, 3))
    a32, b32, c32, p32 = (x.astype(np.float32) for x in (a, b, c, p))
    want = _tri_dist64(*(x.astype(np.float64) for x in (p32, a32, b32, c32)))
    got = np.array([od.tri_dist(p32[i], a32[i], b32[i], c32[i]) for i in range(n)])
    assert np.max(np.abs(got - want)) < 2e-6
    # the vertices and points on the triangle are at distance ~0
    for i in range(50):
        for v in (a32[i], b32[i], c32[i], (a32[i] + b32[i]) / 2):
            assert od.tri_dist(v, a32[i], b32[i], c32[i]) < 1e-6


def test_compute_distance_mesh_against_float64():
    from mplicits_gb300 import synthetic
    pos, _, faces = synthetic.surface_mesh(10, 16)
    rng = np.random.default_rng(4)
    pts = rng.uniform(-0.9, 0.9, (300, 3)).astype(np.float32)
    got = od.compute_distance(pos, faces, pts)
    P = pos.astype(np.float64)
    A, B, C = P[faces[:, 0]], P[faces[:, 1]], P[faces[:, 2]]
    want = np.min(_tri_dist64(pts.astype(np.float64)[:, None], A[None], B[None], C[None]), 1)
    assert np.max(np.abs(got - want)) < 2e-6
    bad = od.compute_distance(pos, faces, np.array([[np.nan, 0, 0]], np.float32))
    assert np.isnan(bad[0])


def test_slab_converges_to_half_gap():
    from golden.make_calc_deltas import slab
    pos, nrm, faces = slab(6, 0.08)
    out, _ = od.calc_deltas(np.concatenate([pos, nrm], 1), pos, faces, 0.2, 100, cell=0.05)
    # the inscribed ball between two sheets has radius gap / 2; the bisection
    # lands within eps of it
    assert np.all(np.abs(out[:, 6] - 0.04) < 3e-4)


def test_arguments():
    pos, faces = np.zeros((3, 3), np.float32), np.array([[0, 1, 2]], np.int32)
    with pytest.raises(ValueError):
        od.calc_deltas(np.zeros((0, 6), np.float32), pos, faces)
    with pytest.raises(ValueError):
        od.calc_deltas(np.zeros((2, 5), np.float32), pos, faces)
    with pytest.raises(ValueError):
        od.calc_deltas(np.zeros((2, 6), np.float32), pos, np.array([[0, 1, 3]], np.int32))


def test_oracle_stopping_rule_edges():
    from golden.make_calc_deltas import slab
    pos, nrm, faces = slab(4, 0.08)
    V = np.concatenate([pos, nrm], 1)
    # the first step already reaches max_delta: no iteration runs
    out, it = od.calc_deltas(V, pos, faces, 0.2, 1)
    assert it == 0 and np.all(out[:, 6] == np.float32(0.2))
    out, it = od.calc_deltas(V, pos, faces, 0.0, 50)
    assert it == 0 and np.all(out[:, 6] == 0.0)
    # grid and brute force agree when the ball covers the whole mesh
    a, ia = od.calc_deltas(V, pos, faces, 5.0, 30)
    b, ib = od.calc_deltas(V, pos, faces, 5.0, 30, cell=0.05)
    assert ia == ib and np.array_equal(a, b)


def test_synthetic_mesh_is_closed_and_outward():
    """The triangulated synthetic surface: every edge shared by exactly two
    faces in opposite directions, and face normals along the analytic
    vertex normals."""
    from mplicits_gb300 import synthetic
    pos, nrm, faces = synthetic.surface_mesh(12, 18)
    assert pos.shape == ((12 - 1) * 18 + 2, 3) and faces.shape == (2 * (12 - 1) * 18, 3)
    e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
    directed = {tuple(x) for x in e}
    assert len(directed) == e.shape[0]
    assert all((b, a) in directed for a, b in directed)
    a, b, c = pos[faces[:, 0]], pos[faces[:, 1]], pos[faces[:, 2]]
    fn = np.cross(b - a, c - a)
    assert np.all(np.sum(fn * nrm[faces].mean(1), 1) > 0)
    assert np.allclose(np.linalg.norm(nrm, axis=1), 1, atol=1e-6)
    with pytest.raises(ValueError):
        synthetic.surface_mesh(1, 18)


def test_fast_decision_equals_minimum_on_a_larger_mesh():
    from mplicits_gb300 import synthetic
    pos, nrm, faces = synthetic.surface_mesh(40, 80)
    V = np.concatenate([pos, nrm], 1)
    a, ia = od.calc_deltas(V, pos, faces, 0.06, 100, cell=0.03)
    b, ib = od.calc_deltas(V, pos, faces, 0.06, 100, cell=0.02, fast=True)
    c, ic = od.calc_deltas(V, pos, faces, 0.06, 100, bvh=True)
    assert ia == ib == ic and np.array_equal(a, b) and np.array_equal(a, c)
