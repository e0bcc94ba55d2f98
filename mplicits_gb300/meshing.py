"""Band-culled multistage reconstruction on the GPU (drop-in for i3d.meshing).

``create_mesh_multistage`` keeps the signature and return tuple of
i3d/meshing.py:135-264.  Instead of a Python loop over 32^3-point chunks with
boolean gathers and host syncs, it runs one fused kernel launch per level:

    level 0  on all N^3 grid points (coordinates generated in-kernel),
             storing S and appending the points with |S| < delta_0;
    level i  on the band list of level i-1 (count read on the device),
             S[p] += f_i, appending the points with |S| < delta_i;

then marching cubes on the device, and copies only the mesh to the host.
"""

from __future__ import annotations

import ctypes
import time

import numpy as np
import torch

from . import capi


def _grid_points(N, voxel_size, voxel_origin=(-1, -1, -1)):
    # column c of the reference grid adds voxel_origin[2 - c] (i3d/meshing.py:61-63)
    return capi.MplPoints(kind=capi.MPL_POINTS_GRID, grid_n=int(N),
                          voxel_size=float(np.float32(voxel_size)),
                          offset=(ctypes.c_float * 3)(float(voxel_origin[2]),
                                                      float(voxel_origin[1]),
                                                      float(voxel_origin[0])))


def gen_mc_coordinate_grid(N, voxel_size, t=None, device="cuda", voxel_origin=[-1, -1, -1]):
    """Grid of i3d/meshing.py:11-69 as an (N^3, 4) tensor (xyz + SDF slot),
    computed on the GPU with the reference's float32 formula."""
    if t is not None:
        raise NotImplementedError("space-time (4-D) grids are not part of the GB300 path")
    dev = torch.device(device)
    if dev.type != "cuda":
        raise RuntimeError("mplicits_gb300 builds the grid on a CUDA device only")
    n = N ** 3
    samples = torch.zeros(n, 4, device=dev)
    xyz = torch.empty(n, 3, device=dev)
    pts = _grid_points(N, voxel_size, voxel_origin)
    capi.check(capi.load().mpl_grid_points(ctypes.byref(pts), None, n, capi.ptr(xyz),
                                           capi.stream_ptr()), "mpl_grid_points")
    samples[:, :3] = xyz
    return samples


class MarchingCubes:
    """GPU marching cubes with a reusable workspace (mpl_mc_count/emit)."""

    def __init__(self, N, device):
        self.N = int(N)
        self.device = torch.device(device)
        nbytes = ctypes.c_int64(0)
        capi.check(capi.load().mpl_mc_workspace_bytes(self.N, ctypes.byref(nbytes)),
                   "mpl_mc_workspace_bytes")
        self._ws_raw = torch.empty(nbytes.value + 256, dtype=torch.uint8, device=self.device)
        off = (-self._ws_raw.data_ptr()) % 256
        self.ws = self._ws_raw[off:off + nbytes.value]
        self.counts = torch.zeros(2, dtype=torch.int64, device=self.device)

    def count(self, S, iso=0.0):
        capi.check(capi.load().mpl_mc_count(capi.ptr(S), self.N, float(iso), capi.ptr(self.ws),
                                            capi.ptr(self.counts), capi.stream_ptr()),
                   "mpl_mc_count")
        return self.counts

    def emit(self, S, V, F, iso=0.0, voxel_size=1.0, origin=(0.0, 0.0, 0.0)):
        dev = self.device
        verts = torch.empty(V, 3, dtype=torch.float32, device=dev)
        normals = torch.empty(V, 3, dtype=torch.float32, device=dev)
        values = torch.empty(V, dtype=torch.float32, device=dev)
        faces = torch.empty(F, 3, dtype=torch.int32, device=dev)
        org = (ctypes.c_float * 3)(*[float(o) for o in origin])
        capi.check(capi.load().mpl_mc_emit(
            capi.ptr(S), self.N, float(iso), float(np.float32(voxel_size)), org,
            capi.ptr(self.ws), capi.ptr(verts), capi.ptr(normals), capi.ptr(values),
            capi.ptr(faces), V, F, capi.stream_ptr()), "mpl_mc_emit")
        return verts, faces, normals, values

    def __call__(self, S, iso=0.0, voxel_size=1.0, origin=(0.0, 0.0, 0.0)):
        counts = self.count(S, iso).cpu()
        V, F = int(counts[0]), int(counts[1])
        return self.emit(S, V, F, iso, voxel_size, origin)


class BandedReconstruction:
    """Reusable buffers and launches of the band-culled multistage evaluation.

    ``levels`` are SIREN modules (coarse first); ``deltas`` one per residual
    level (empty: evaluate every level everywhere, i3d/meshing.py:232-233).

    ``refine_margin`` (tensor-core precisions only): an upper bound m of the
    tensor-core error of a partial sum.  Points whose value lies within m of
    a band threshold are re-evaluated with the FP32 kernels before the band
    list is cut, and points with |S| < m after the last level get every level
    in FP32, so the band decisions and the marching-cubes signs are those of
    the plain FP32 path.

    Band widths that never grow from one level to the next (the usual case)
    make each band a subset of the previous one, so every level cuts the next
    level's list as it stores (fused band lists).  When a width grows, the
    reference's masks differ: level i runs on every point of a chunk of
    ``chunk`` consecutive grid points with ``|S| < delta_{i-1}``, and a chunk
    none of whose points was in band i stops there (i3d/meshing.py:221-231,
    ``chunk`` is its ``max_batch``).  Those bands are cut by a compaction over
    the whole grid and filtered by chunk on the device (one host read of each
    band's size).
    """

    def __init__(self, levels, deltas, N, device="cuda", precision=None, refine_margin=None,
                 chunk=64 ** 3):
        self.levels = list(levels)
        self.deltas = list(deltas or [])
        self.N = int(N)
        self.device = torch.device(device)
        self.precision = precision
        self.chunk = int(chunk)
        if self.chunk < 1:
            raise ValueError("chunk (max_batch) must be positive")
        if self.deltas and len(self.deltas) < len(self.levels) - 1:
            raise IndexError("deltas needs one entry per residual level")
        self.nested = not self.deltas or all(self.deltas[i + 1] <= self.deltas[i]
                                             for i in range(len(self.levels) - 2))
        if not self.nested and refine_margin:
            raise NotImplementedError(
                "FP32 refinement margins need band widths that do not grow")
        n = self.N ** 3
        self.n = n
        self.voxel_size = 2.0 / (self.N - 1)
        self.points = _grid_points(self.N, self.voxel_size)
        self.S = torch.empty(n, dtype=torch.float32, device=self.device)
        m = len(self.levels) - 1 if self.deltas else 0
        self.band_index = [torch.empty(n, dtype=torch.int32, device=self.device)
                           for _ in range(m)]
        self.band_count = torch.zeros(max(m, 1), dtype=torch.int32, device=self.device)
        self._bands = []
        for i in range(m):
            b = capi.MplBand(delta=float(self.deltas[i]), out_index=self.band_index[i].data_ptr(),
                             count_dev=self.band_count[i:].data_ptr(), capacity=n)
            self._bands.append(b)
        self.mc = None
        self.refine_margin = float(refine_margin) if refine_margin else 0.0
        if self.refine_margin:
            if self.deltas and self.refine_margin >= min(self.deltas[:m]):
                raise ValueError("refine_margin must be smaller than every band width")
            self.cand_index = [torch.empty(n, dtype=torch.int32, device=self.device)
                               for _ in range(m)]
            self.amb_index = torch.empty(n, dtype=torch.int32, device=self.device)
            self.aux_count = torch.zeros(m + 1, dtype=torch.int32, device=self.device)

    def _prec(self, model):
        return capi.PRECISIONS[self.precision or getattr(model, "precision", "fp32")]

    def _band(self, delta, out, count_view, lower=0.0):
        return capi.MplBand(delta=float(delta), out_index=out.data_ptr(),
                            count_dev=count_view.data_ptr(), capacity=self.n, lower=float(lower))

    def _level(self, i, precision, mode, index=None, count=None, band=None, st=None):
        net, packed = self.levels[i].packed()
        capi.check(capi.load().mpl_level_forward(
            ctypes.byref(net), capi.ptr(packed), ctypes.byref(self.points), capi.ptr(index),
            capi.ptr(count), self.n, capi.ptr(self.S), mode,
            None if band is None else ctypes.byref(band), precision, st), "mpl_level_forward")

    def _compact(self, band, index, count, st):
        capi.check(capi.load().mpl_band_compact(
            capi.ptr(self.S), capi.ptr(index), capi.ptr(count), self.n, ctypes.byref(band), st),
            "mpl_band_compact")

    def _sample_refined(self, st):
        """Tensor-core levels with FP32 re-evaluation inside the margins."""
        m = self.refine_margin
        fp32 = capi.MPL_FP32
        amb, amb_n = self.amb_index, self.aux_count[len(self.cand_index):]
        L = len(self.levels)
        keep = []  # (band structs) kept alive until the launches are queued
        idx, cnt = None, None
        for i in range(L):
            prec = self._prec(self.levels[i])
            mode = capi.MPL_STORE if i == 0 else capi.MPL_ACCUMULATE
            if i < len(self.cand_index):
                cand, cand_n = self.cand_index[i], self.aux_count[i:]
                b = self._band(self.deltas[i] + m, cand, cand_n)
                keep.append(b)
                self._level(i, prec, mode, idx, cnt, b, st)
                # the ambiguous shell of this threshold, re-evaluated in FP32
                ba = self._band(self.deltas[i] + m, amb, amb_n, lower=self.deltas[i] - m)
                keep.append(ba)
                self._compact(ba, cand, cand_n, st)
                for k in range(i + 1):
                    self._level(k, fp32, capi.MPL_STORE if k == 0 else capi.MPL_ACCUMULATE,
                                amb, amb_n, None, st)
                # the exact band list from the corrected values
                self._compact(self._bands[i], cand, cand_n, st)
                idx, cnt = self.band_index[i], self.band_count[i:]
            else:
                self._level(i, prec, mode, idx, cnt, None, st)
        # the zero level: every level in FP32 where |S| < m
        bz = self._band(m, amb, amb_n)
        keep.append(bz)
        if idx is None:
            self._compact(bz, None, None, st)
        else:
            self._compact(bz, idx, cnt, st)
        for k in range(L):
            self._level(k, fp32, capi.MPL_STORE if k == 0 else capi.MPL_ACCUMULATE, amb, amb_n,
                        None, st)
        self._keep = keep
        return self.S

    def _sample_general(self, stream):
        """Bands of growing widths: level i on the points of the still-open
        chunks with |S| < delta_{i-1}; a chunk with none closes."""
        n, chunk = self.n, self.chunk
        nchunks = (n + chunk - 1) // chunk
        st = capi.stream_ptr(stream)
        with torch.cuda.stream(stream) if stream is not None else torch.cuda.device(self.device):
            self._level(0, self._prec(self.levels[0]), capi.MPL_STORE, st=st)
            open_ = torch.ones(nchunks, dtype=torch.bool, device=self.device)
            keep = []
            for i in range(1, len(self.levels)):
                lst, cnt = self.band_index[i - 1], self.band_count[i - 1:]
                b = self._band(self.deltas[i - 1], lst, cnt)
                keep.append(b)
                self._compact(b, None, None, st)
                m = int(cnt[0])  # host read: the band's size
                idx = lst[:m].long()
                ch = idx // chunk
                sel = open_[ch]
                idx, ch = idx[sel], ch[sel]
                hit = torch.zeros(nchunks, dtype=torch.bool, device=self.device)
                hit[ch] = True
                open_ &= hit
                lst[:idx.numel()] = idx.to(torch.int32)
                cnt[0] = idx.numel()
                self._level(i, self._prec(self.levels[i]), capi.MPL_ACCUMULATE, lst, cnt, None,
                            st)
            self._keep = keep
        return self.S

    def sample(self, stream=None):
        """Evaluate S over the grid (stream-ordered; with nested band widths
        no host sync)."""
        lib = capi.load()
        st = capi.stream_ptr(stream)
        if not self.nested:
            return self._sample_general(stream)
        if self.refine_margin and any(self._prec(mo) != capi.MPL_FP32 for mo in self.levels):
            return self._sample_refined(st)
        for i, model in enumerate(self.levels):
            net, packed = model.packed()
            if i == 0:
                band = ctypes.byref(self._bands[0]) if self._bands else None
                capi.check(lib.mpl_level_forward(
                    ctypes.byref(net), capi.ptr(packed), ctypes.byref(self.points), None, None,
                    self.n, capi.ptr(self.S), capi.MPL_STORE, band, self._prec(model), st),
                    "mpl_level_forward")
            elif self.deltas:
                band = ctypes.byref(self._bands[i]) if i < len(self._bands) else None
                capi.check(lib.mpl_level_forward(
                    ctypes.byref(net), capi.ptr(packed), ctypes.byref(self.points),
                    capi.ptr(self.band_index[i - 1]), capi.ptr(self.band_count[i - 1:]),
                    self.n, capi.ptr(self.S), capi.MPL_ACCUMULATE, band, self._prec(model), st),
                    "mpl_level_forward")
            else:
                capi.check(lib.mpl_level_forward(
                    ctypes.byref(net), capi.ptr(packed), ctypes.byref(self.points), None, None,
                    self.n, capi.ptr(self.S), capi.MPL_ACCUMULATE, None, self._prec(model), st),
                    "mpl_level_forward")
        return self.S

    def band_sizes(self):
        return [int(c) for c in self.band_count[:len(self._bands)].cpu()]

    def mesh(self, iso=0.0):
        if self.mc is None:
            self.mc = MarchingCubes(self.N, self.device)
        return self.mc(self.S, iso, self.voxel_size, (-1.0, -1.0, -1.0))


def convert_sdf_samples_to_ply(sdf_volume, voxel_grid_origin, voxel_size, offset=None,
                               scale=None):
    """GPU restatement of i3d/meshing.py:267-313 on a device [N,N,N] volume;
    returns numpy arrays (verts, faces, normals, values)."""
    S = sdf_volume.reshape(-1)
    N = sdf_volume.shape[0]
    mc = MarchingCubes(N, S.device)
    verts, faces, normals, values = mc(S, 0.0, voxel_size, voxel_grid_origin)
    if verts.shape[0] == 0:
        lo, hi = float(S.min()), float(S.max())
        if 0.0 < lo or 0.0 > hi:
            print("Surface level must be within volume data range.")
            z = np.zeros((0, 3))
            return z, np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0)
    verts = verts.cpu().numpy()
    if scale is not None:
        verts = verts / scale
    if offset is not None:
        verts = verts - offset
    return verts, faces.cpu().numpy(), normals.cpu().numpy(), values.cpu().numpy()


def save_ply(verts, faces, filename, vertex_attributes=None):
    """Binary PLY with the element layout plyfile writes for
    i3d/meshing.py:316-384 (vertex x,y,z float; face vertex_indices list)."""
    verts = np.asarray(verts)
    faces = np.asarray(faces, np.int32)
    dtypes = [("x", "<f4"), ("y", "<f4"), ("z", "<f4")]
    if vertex_attributes is not None:
        dtypes[3:3] = [(n, "<" + t.lstrip("<>=")) for n, t in vertex_attributes]
    vt = np.zeros(verts.shape[0], dtype=dtypes)
    for c, (name, _) in enumerate(dtypes):
        vt[name] = verts[:, c]
    ft = np.zeros(faces.shape[0], dtype=[("n", "u1"), ("v", "<i4", (3,))])
    ft["n"] = 3
    ft["v"] = faces
    ply_types = {"f4": "float", "f8": "double", "u1": "uchar", "i1": "char", "u2": "ushort",
                 "i2": "short", "u4": "uint", "i4": "int"}
    for n, t in dtypes:
        if t[1:] not in ply_types:
            raise ValueError(f"vertex attribute {n!r}: PLY has no type for numpy dtype {t!r}")
    props = "\n".join(f"property {ply_types[t[1:]]} {n}" for n, t in dtypes)
    header = (f"ply\nformat binary_little_endian 1.0\nelement vertex {verts.shape[0]}\n"
              f"{props}\nelement face {faces.shape[0]}\n"
              "property list uchar int vertex_indices\nend_header\n")
    with open(filename, "wb") as f:
        f.write(header.encode("ascii"))
        f.write(vt.tobytes())
        f.write(ft.tobytes())


def create_mesh_multistage(decoders, deltas=[], filename="", t=None, N=256, max_batch=64 ** 3,
                           offset=None, scale=None, device="cpu", silent=False, precision=None):
    """Drop-in for i3d/meshing.py:135-264; returns (verts, faces, normals,
    values, sampling_time).  Each level runs as one launch over its whole
    point list; ``max_batch`` matters only when a band width grows from one
    level to the next, where the reference's per-chunk masks depend on it.
    ``precision`` ("fp32", "bf16" or "fp16") overrides the decoders' own
    setting."""
    if t is not None and t != -1:
        raise NotImplementedError("space-time (4-D) decoders are not part of the GB300 path")
    dev = torch.device(device)
    if dev.type != "cuda":
        raise RuntimeError("mplicits_gb300 reconstructs on a CUDA device only (no CPU fallback)")
    for d in decoders:
        d.eval()
    rec = BandedReconstruction(decoders, deltas, N, dev, precision, chunk=max_batch)
    for d in decoders:  # pack outside the timing window, as the reference's weights
        d.packed()       # are already resident when its loop starts
    torch.cuda.synchronize(dev)
    start = time.perf_counter()
    rec.sample()
    torch.cuda.synchronize(dev)
    sampling_time = time.perf_counter() - start
    if not silent:
        print(f"Sampling took: {sampling_time} s")
    verts, faces, normals, values = convert_sdf_samples_to_ply(
        rec.S.view(N, N, N), [-1, -1, -1], rec.voxel_size, offset, scale)
    if filename:
        if not silent:
            print(f"Saving mesh to {filename}")
        save_ply(verts, faces, filename)
        if not silent:
            print("Done")
    return verts, faces, normals, values, sampling_time


def create_mesh(decoder, filename="", t=None, N=256, max_batch=64 ** 3, offset=None, scale=None,
                device="cpu", silent=False, precision=None):
    """Single-level variant (i3d/meshing.py:72-132)."""
    v, f, n, val, _ = create_mesh_multistage([decoder], [], filename, t, N, max_batch, offset,
                                             scale, device, silent, precision)
    return v, f, n, val
