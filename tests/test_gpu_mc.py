"""GPU marching cubes against the CPU restatement (oracle/mc.c): vertices,
normals, values and triangle indices bit for bit on identical grids."""

import numpy as np
import pytest
import torch

from conftest import golden, tiny_levels
from oracle import mc, siren

pytestmark = pytest.mark.gpu


def _gpu_mc(S, vs, origin=(-1.0, -1.0, -1.0)):
    from mplicits_gb300.meshing import MarchingCubes
    N = S.shape[0]
    m = MarchingCubes(N, "cuda")
    v, f, n, val = m(torch.from_numpy(np.ascontiguousarray(S)).cuda().reshape(-1), 0.0, vs,
                     origin)
    return v.cpu().numpy(), f.cpu().numpy(), n.cpu().numpy(), val.cpu().numpy()


def _assert_same(S, vs=None):
    N = S.shape[0]
    vs = 2.0 / (N - 1) if vs is None else vs
    a = _gpu_mc(S, vs)
    b = mc.marching_cubes_raw(S, 0.0, np.float32(vs), (-1.0, -1.0, -1.0))
    for x, y in zip(a, b):
        assert x.shape == y.shape
        assert np.array_equal(x.view(np.uint32) if x.dtype == np.float32 else x,
                              y.view(np.uint32) if y.dtype == np.float32 else y)
    return a


def _sphere(N, r=0.6):
    x = np.linspace(-1, 1, N, dtype=np.float32)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    return (np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - r).astype(np.float32)


@pytest.mark.parametrize("N", [2, 3, 17, 64, 129])
def test_sphere_bit_exact(lib, N):
    _assert_same(_sphere(N))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_fields_bit_exact(lib, seed):
    rng = np.random.default_rng(seed)
    S = rng.standard_normal((33, 33, 33)).astype(np.float32)
    S[rng.random(S.shape) < 0.05] = 0.0  # exact iso values: ties go "outside"
    _assert_same(S)


def test_reference_volume_bit_exact(lib):
    _, _, d = tiny_levels()
    N = int(d["N"])
    _assert_same(d["S_banded"].reshape(N, N, N))


def test_empty_and_full(lib):
    v, f, n, val = _assert_same(np.ones((9, 9, 9), np.float32))
    assert v.shape[0] == 0 and f.shape[0] == 0
    _assert_same(-np.ones((9, 9, 9), np.float32))


def test_large_grid_matches_oracle(lib):
    x = np.linspace(-1, 1, 300, dtype=np.float32)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    S = (np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - 0.6 - 0.03 * np.sin(12 * X) * np.sin(12 * Y)
         ).astype(np.float32)
    _assert_same(S)


def test_largest_grid_and_densest_line(lib):
    """N = 1024 (the largest supported grid) with lines whose every edge
    along k crosses the surface: the in-line vertex prefixes reach their
    largest values there."""
    N = 1024
    S = np.ones((N, N, N), np.float32)
    alt = np.where(np.arange(N) % 2 == 0, -1.0, 1.0).astype(np.float32)
    for i, j in ((0, 0), (511, 700), (1022, 1023), (1023, 5)):
        S[i, j, :] = alt
    x = np.linspace(-1, 1, N, dtype=np.float32)
    # and a sphere, so that many rows of cells emit triangles
    S[:, :, :] = np.minimum(S, (np.sqrt(x[:, None, None] ** 2 + x[None, :, None] ** 2 +
                                        x[None, None, :] ** 2) - 0.5).astype(np.float32))
    for i, j in ((0, 0), (511, 700), (1022, 1023), (1023, 5)):
        S[i, j, :] = alt
    v, f, _, _ = _assert_same(S)
    assert v.shape[0] > 1000 and f.shape[0] > 1000


def test_grid_limit_is_reported(lib):
    import ctypes
    from mplicits_gb300 import capi
    nb = ctypes.c_int64(0)
    assert lib.mpl_mc_workspace_bytes(1025, ctypes.byref(nb)) == capi.MPL_ERR_UNSUPPORTED
    assert lib.mpl_mc_workspace_bytes(1024, ctypes.byref(nb)) == capi.MPL_OK
