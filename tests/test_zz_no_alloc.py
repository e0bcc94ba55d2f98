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
    for call, (N, seed) in enumerate(((200, 1), (96, 2))):
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
