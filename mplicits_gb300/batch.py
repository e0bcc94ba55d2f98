"""Serving-style evaluation of many levels of many models in persistent
launches.

``BatchedLevels`` takes a list of (level, points) entries, writes the device
entry table once (``mpl_batch_prepare``, entries grouped by width), picks the
kernel configuration with the library's autotuner (one or two tiles per CTA x
epilogue unit width x weight-ring depth, timed on the plan itself and cached
per plan signature), and evaluates every entry in one persistent launch per
width group (``mpl_batch_run``), optionally replayed from a CUDA graph.  It replaces the reference's one launch chain per model and level
(renderer/cuda/gemms.cu:5-192, i3d/meshing.py:212-236).

Entries write disjoint outputs: tiles of different entries run concurrently,
so an entry in MPL_ACCUMULATE mode adds into values that exist before the
launch, never into another entry's output of the same launch.
"""

from __future__ import annotations

import ctypes

import torch

from . import capi

_TUNED = {}


class BatchEntry:
    """One level on one point list: ``x`` [P, 3] points (or a grid
    ``(N, voxel_size, offset)``), optional ``index`` (int32 [n]) and device
    count ``n_dev`` (int32 [1]), output ``S`` indexed like the points."""

    def __init__(self, model, S, x=None, grid=None, index=None, n=None, n_dev=None,
                 accumulate=False):
        self.model, self.S, self.x, self.grid = model, S, x, grid
        self.index, self.n_dev, self.accumulate = index, n_dev, accumulate
        if n is None:
            n = index.shape[0] if index is not None else (
                x.shape[0] if x is not None else grid[0] ** 3)
        self.n = int(n)


class BatchedLevels:
    def __init__(self, entries, precision="bf16", device="cuda"):
        if precision not in ("bf16", "fp16"):
            raise ValueError("the batched launch runs on the tensor cores: bf16 or fp16")
        self.entries = list(entries)
        if len(self.entries) > capi.MPL_BATCH_MAX_ENTRIES:
            raise ValueError(f"at most {capi.MPL_BATCH_MAX_ENTRIES} entries per plan")
        self.precision = precision
        self.device = torch.device(device)
        lib = capi.load()
        nbytes = ctypes.c_int64(0)
        capi.check(lib.mpl_batch_workspace_bytes(len(self.entries), ctypes.byref(nbytes)),
                   "mpl_batch_workspace_bytes")
        buf = torch.empty(nbytes.value + 256, dtype=torch.uint8, device=self.device)
        off = (-buf.data_ptr()) % 256
        self._ws_buf = buf
        self.workspace = buf[off:off + max(nbytes.value, 1)]
        self._keep = []
        arr = (capi.MplBatchEntry * max(len(self.entries), 1))()
        for i, e in enumerate(self.entries):
            net, packed = e.model.packed()
            self._keep.append(packed)
            ce = arr[i]
            ce.net = net
            ce.packed_dev = packed.data_ptr()
            if e.grid is not None:
                N, vs, offset = e.grid
                ce.points.kind = capi.MPL_POINTS_GRID
                ce.points.grid_n = int(N)
                ce.points.voxel_size = float(vs)
                for k in range(3):
                    ce.points.offset[k] = float(offset[k])
            else:
                x = e.x.detach().float().contiguous()
                self._keep.append(x)
                ce.points.kind = capi.MPL_POINTS_XYZ
                ce.points.xyz = x.data_ptr()
            ce.index_dev = e.index.data_ptr() if e.index is not None else None
            ce.n_dev = e.n_dev.data_ptr() if e.n_dev is not None else None
            ce.n = e.n
            ce.S_dev = e.S.data_ptr()
            ce.store_mode = capi.MPL_ACCUMULATE if e.accumulate else capi.MPL_STORE
        self.plan = capi.MplBatchPlan()
        capi.check(lib.mpl_batch_prepare(arr, len(self.entries), capi.PRECISIONS[precision],
                                         capi.ptr(self.workspace), nbytes.value,
                                         ctypes.byref(self.plan), capi.stream_ptr()),
                   "mpl_batch_prepare")
        self.config = None
        self._graph = None

    def signature(self):
        """Plan shape for the autotuner cache: widths, depths and point
        counts (rounded to powers of two) of the entries."""
        sig = []
        for e in self.entries:
            net = e.model.mpl_net()
            dims = tuple(net.dims[i] for i in range(net.n_layers + 1))
            sig.append((dims, max(e.n, 1).bit_length()))
        return (self.precision, tuple(sorted(sig)))

    def autotune(self, repeats=3, cache=True):
        key = self.signature()
        if cache and key in _TUNED:
            self.config = _TUNED[key][0]
            return self.config, _TUNED[key][1]
        best = capi.MplBatchConfig()
        ms = ctypes.c_float(0.0)
        capi.check(capi.load().mpl_batch_autotune(ctypes.byref(self.plan), int(repeats),
                                                  ctypes.byref(best), ctypes.byref(ms),
                                                  capi.stream_ptr()), "mpl_batch_autotune")
        self.config = best
        _TUNED[key] = (best, ms.value)
        return best, ms.value

    def run(self, config=None):
        cfg = config if config is not None else self.config
        capi.check(capi.load().mpl_batch_run(ctypes.byref(self.plan),
                                             ctypes.byref(cfg) if cfg is not None else None,
                                             capi.stream_ptr()), "mpl_batch_run")

    def capture(self):
        """Record the launch into a CUDA graph (after autotune, if wanted)."""
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.run()  # first launch outside capture: kernel attributes, module load
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run()
        self._graph = g
        return g

    def replay(self):
        if self._graph is None:
            self.capture()
        self._graph.replay()
