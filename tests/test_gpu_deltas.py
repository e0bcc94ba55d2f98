"""calc_deltas and the triangle scene on the GPU against the oracle: the
reference's golden vectors bit for bit, nearest-triangle distances bit for
bit, a larger mesh against the oracle's grid search, and a full-size mesh
through a subset checked at the run's own stopping point."""

import os

import numpy as np
import pytest
import torch

from oracle import deltas as od

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "calc_deltas.npz")


def _golden():
    g = np.load(GOLDEN)
    for name in g["cases"]:
        yield str(name), {k.split("__", 1)[1]: g[k] for k in g.files if k.startswith(f"{name}__")}


@pytest.mark.parametrize("cell", [0.0, 0.004, 0.03, 0.11, 2.0])
def test_golden_bit_exact(cell):
    from mplicits_gb300.scene import RaycastingScene, calc_deltas
    for name, c in _golden():
        scene = RaycastingScene(c["positions"], c["faces"], cell=cell)
        md = float(c["max_delta"]) if str(c["max_delta_kind"]) == "float" \
            else torch.tensor(float(c["max_delta"]), dtype=torch.float32)
        out, it = calc_deltas(torch.from_numpy(c["vertices"]), scene, max_delta=md,
                              n_iters=int(c["n_iters"]), return_iterations=True)
        assert it == int(c["iterations"]), name
        got = out.cpu().numpy()
        np.testing.assert_array_equal(got, c["out"], err_msg=f"{name} cell {cell}")


def _points(pos, n, rng):
    near = pos[rng.integers(0, pos.shape[0], n)] + rng.normal(0, 0.05, (n, 3))
    far = rng.uniform(-4, 4, (n // 4, 3))
    return np.concatenate([near, far, [[np.nan, 0, 0], [0, np.inf, 0], [1e3, -1e3, 5e2]]]) \
        .astype(np.float32)


@pytest.mark.parametrize("cell", [0.0, 0.01, 0.3])
def test_compute_distance_bit_exact(cell):
    from mplicits_gb300 import synthetic
    from mplicits_gb300.scene import RaycastingScene
    pos, _, faces = synthetic.surface_mesh(24, 40)
    rng = np.random.default_rng(8)
    pts = _points(pos, 3000, rng)
    scene = RaycastingScene(pos, faces, cell=cell)
    got = scene.compute_distance(torch.from_numpy(pts)).cpu().numpy()
    want = od.compute_distance(pos, faces, pts)
    np.testing.assert_array_equal(got, want)


def test_larger_mesh_equals_oracle_grid():
    from mplicits_gb300 import synthetic
    from mplicits_gb300.scene import RaycastingScene, calc_deltas
    pos, nrm, faces = synthetic.surface_mesh(96, 192)
    V = np.concatenate([pos, nrm], 1)
    scene = RaycastingScene(pos, faces)
    out, it = calc_deltas(V, scene, max_delta=0.05, n_iters=100, return_iterations=True)
    want, it_ref = od.calc_deltas(V, pos, faces, 0.05, 100, cell=0.02)
    assert it == it_ref
    np.testing.assert_array_equal(out.cpu().numpy(), want)


def test_full_size_subset_at_the_runs_stopping_point():
    """524k vertices: a seeded subset of 3000 vertices recomputed by the
    oracle with the GPU run's iteration count (each vertex's path depends on
    the others only through that count)."""
    from mplicits_gb300 import synthetic
    from mplicits_gb300.scene import RaycastingScene, calc_deltas
    pos, nrm, faces = synthetic.surface_mesh(512, 1024)
    V = np.concatenate([pos, nrm], 1)
    scene = RaycastingScene(pos, faces)
    out, it = calc_deltas(V, scene, max_delta=0.05, n_iters=100, return_iterations=True)
    got = out.cpu().numpy()
    d = got[:, 6]
    assert np.all(d > 0) and np.all(np.isfinite(d))
    # the loop stops once one delta reaches max_delta, or after n_iters
    assert it == 100 or d.max() >= np.float32(0.05)
    idx = np.random.default_rng(2).choice(V.shape[0], 3000, replace=False)
    want, _ = od.calc_deltas(V[idx], pos, faces, 0.05, 100, cell=0.01, force_iters=it)
    np.testing.assert_array_equal(got[idx], want)


def test_scene_rejects_bad_faces_and_inputs():
    from mplicits_gb300 import capi
    from mplicits_gb300.scene import RaycastingScene, calc_deltas
    pos = np.zeros((3, 3), np.float32)
    with pytest.raises(capi.MplError):
        RaycastingScene(pos, np.array([[0, 1, 3]], np.int32))
    with pytest.raises(capi.MplError):
        RaycastingScene(pos, np.array([[0, -1, 2]], np.int32))
    scene = RaycastingScene(np.eye(3, dtype=np.float32), np.array([[0, 1, 2]], np.int32))
    with pytest.raises(ValueError):
        calc_deltas(np.zeros((0, 6), np.float32), scene)
    with pytest.raises(ValueError):
        calc_deltas(np.zeros((4, 5), np.float32), scene)
    assert capi.device_status() == capi.MPL_OK


def _degenerate_mesh():
    from golden.make_calc_deltas import slab
    pos, nrm, faces = slab(5, 0.1)
    extra = np.array([[0.1, 0.1, 0.05], [0.3, 0.1, 0.05], [0.2, 0.1, 0.05]], np.float32)
    base = pos.shape[0]
    pos = np.concatenate([pos, extra])
    nrm = np.concatenate([nrm, np.tile([[0, 0, 1]], (3, 1)).astype(np.float32)])
    # a zero-area triangle (collinear corners) and one with a repeated corner
    faces = np.concatenate([faces, [[base, base + 1, base + 2], [base, base, base + 1]]])
    return pos, nrm, faces.astype(np.int32)


@pytest.mark.parametrize("case", ["degenerate", "huge_radius", "one_iteration", "zero_max",
                                  "offset_scene"])
def test_edge_cases_bit_exact(case):
    from mplicits_gb300.scene import RaycastingScene, calc_deltas
    from golden.make_calc_deltas import slab
    pos, nrm, faces = slab(6, 0.08)
    md, iters = 0.2, 100
    if case == "degenerate":
        pos, nrm, faces = _degenerate_mesh()
    elif case == "huge_radius":
        md = 5.0
    elif case == "one_iteration":
        iters = 1
    elif case == "zero_max":
        md = 0.0
    elif case == "offset_scene":
        pos = pos * 40.0 + np.float32([100.0, -250.0, 30.0])
        md = 8.0
    V = np.concatenate([pos, nrm], 1).astype(np.float32)
    scene = RaycastingScene(pos, faces)
    got, it = calc_deltas(V, scene, max_delta=md, n_iters=iters, return_iterations=True)
    want, it_ref = od.calc_deltas(V, pos, faces, md, iters)
    assert it == it_ref
    np.testing.assert_array_equal(got.cpu().numpy(), want)
    rng = np.random.default_rng(3)
    pts = (pos[rng.integers(0, pos.shape[0], 500)] + rng.normal(0, 0.1, (500, 3)) *
           (40.0 if case == "offset_scene" else 1.0)).astype(np.float32)
    np.testing.assert_array_equal(scene.compute_distance(pts).cpu().numpy(),
                                  od.compute_distance(pos, faces, pts))
