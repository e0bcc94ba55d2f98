"""mpl_mc_noalloc: marching cubes for callers that cannot allocate device
memory (a frame loop that must not pay cudaMalloc's device-wide
synchronisation, or a host that can only pass buffers it registered itself).
Its workspace is a fixed array inside the library, shared by every call, so
two calls in a row must both agree with the allocating entry points."""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _field(N, seed):
    rng = np.random.default_rng(seed)
    x = np.linspace(-1, 1, N, dtype=np.float32)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    S = np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - 0.55 + 0.02 * rng.standard_normal(X.shape)
    return torch.from_numpy(S.astype(np.float32)).cuda().reshape(-1)


def test_noalloc_matches_allocating_marching_cubes_twice(lib):
    from mplicits_gb300 import capi
    from mplicits_gb300.meshing import MarchingCubes
    origin = (ctypes.c_float * 3)(-1.0, -1.0, -1.0)
    # the documented maximum N = 256 first, then a smaller grid over the
    # array the first call left behind
    for call, (N, seed) in enumerate(((256, 1), (96, 2), (200, 3))):
        S = _field(N, seed)
        vs = float(np.float32(2.0 / (N - 1)))
        rv, rf, rn, rval = MarchingCubes(N, "cuda")(S, 0.0, vs, (-1.0, -1.0, -1.0))
        V, F = rv.shape[0], rf.shape[0]
        verts = torch.empty(V, 3, device="cuda")
        normals = torch.empty(V, 3, device="cuda")
        values = torch.empty(V, device="cuda")
        faces = torch.empty(F, 3, dtype=torch.int32, device="cuda")
        counts = torch.full((2,), -1, dtype=torch.int64, device="cuda")
        st = lib.mpl_mc_noalloc(capi.ptr(S), N, ctypes.c_float(0.0), ctypes.c_float(vs), origin,
                                capi.ptr(verts), capi.ptr(normals), capi.ptr(values),
                                capi.ptr(faces), V, F, capi.ptr(counts), capi.stream_ptr())
        assert st == capi.MPL_OK, (call, st)
        torch.cuda.synchronize()
        assert counts.tolist() == [V, F], call
        # same tolerance as the other marching-cubes tests: bit for bit
        for a, b in ((verts, rv), (normals, rn), (values, rval), (faces, rf)):
            assert torch.equal(a, b), call


def test_noalloc_rejects_grids_beyond_its_workspace(lib):
    from mplicits_gb300 import capi
    S = torch.zeros(257 ** 3, device="cuda")
    counts = torch.zeros(2, dtype=torch.int64, device="cuda")
    origin = (ctypes.c_float * 3)(-1.0, -1.0, -1.0)
    st = lib.mpl_mc_noalloc(capi.ptr(S), 257, ctypes.c_float(0.0), ctypes.c_float(0.01), origin,
                            None, None, None, None, 0, 0, capi.ptr(counts), capi.stream_ptr())
    assert st == capi.MPL_ERR_CAPACITY


def test_noalloc_truncates_at_the_capacities_and_reports_full_counts(lib):
    """Capacities below the mesh size: counts still give the full [V, F],
    the buffers hold the first max_verts vertices and max_tris triangles of
    the full mesh, and nothing is written past their ends (guard regions
    keep their sentinel).  Zero capacities with null outputs only count."""
    from mplicits_gb300 import capi
    from mplicits_gb300.meshing import MarchingCubes
    N = 120
    S = _field(N, 5)
    vs = float(np.float32(2.0 / (N - 1)))
    origin = (ctypes.c_float * 3)(-1.0, -1.0, -1.0)
    rv, rf, rn, rval = MarchingCubes(N, "cuda")(S, 0.0, vs, (-1.0, -1.0, -1.0))
    V, F = rv.shape[0], rf.shape[0]
    cv, cf, guard = V // 3, F // 2, 4096
    sentinel = -12345.0
    verts = torch.full((cv + guard, 3), sentinel, device="cuda")
    normals = torch.full((cv + guard, 3), sentinel, device="cuda")
    values = torch.full((cv + guard,), sentinel, device="cuda")
    faces = torch.full((cf + guard, 3), -7, dtype=torch.int32, device="cuda")
    counts = torch.full((2,), -1, dtype=torch.int64, device="cuda")
    st = lib.mpl_mc_noalloc(capi.ptr(S), N, ctypes.c_float(0.0), ctypes.c_float(vs), origin,
                            capi.ptr(verts), capi.ptr(normals), capi.ptr(values),
                            capi.ptr(faces), cv, cf, capi.ptr(counts), capi.stream_ptr())
    assert st == capi.MPL_OK
    torch.cuda.synchronize()
    assert counts.tolist() == [V, F]
    assert torch.equal(verts[:cv], rv[:cv]) and torch.equal(normals[:cv], rn[:cv])
    assert torch.equal(values[:cv], rval[:cv]) and torch.equal(faces[:cf], rf[:cf])
    assert (verts[cv:] == sentinel).all() and (normals[cv:] == sentinel).all()
    assert (values[cv:] == sentinel).all() and (faces[cf:] == -7).all()

    counts.fill_(-1)
    st = lib.mpl_mc_noalloc(capi.ptr(S), N, ctypes.c_float(0.0), ctypes.c_float(vs), origin,
                            None, None, None, None, 0, 0, capi.ptr(counts), capi.stream_ptr())
    assert st == capi.MPL_OK
    torch.cuda.synchronize()
    assert counts.tolist() == [V, F]
