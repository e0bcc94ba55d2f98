"""Multiscale sphere tracing with band-gated levels and analytic normals.

Restates the reference renderer's frame (renderer/cuda/state.cu:816-1055,
kernels.cu:315-487) headless.  One step for every marching ray:

    S  = f0(p)                       (fused list of rays with |S| < delta_0)
    S += f1(p)  on that list         (fused list of rays with |S| < delta_1)
    S += f2(p)  on that list
    hit if |S| < eps, else p += d * S; leaving the bounding sphere is a miss.

The reference evaluates every level for every pixel in fixed per-level
phases; here a ray only pays for the levels whose band it is in, and a ray
stops when it hits.  The loop of ``max_steps`` steps (level launches on
device-side counts, no host sync) is captured once into a CUDA graph and
replayed per frame.  Normals of the hits are the sum of the band-gated level
gradients (forward-mode kernel), as the reference's sum_residual_normals
(kernels.cu:65-120) sums its per-level normals.

With ``tail_from=k`` (tensor-core precisions), steps k .. max_steps-1 run in
one persistent launch (mpl_trace_march) that keeps each tile of 128 rays on
one CTA for all of them: late steps touch few rays, and there the fixed
latency of the per-level launches dominates.  Every ray gets the same result
as from the launch-per-level loop.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import capi


def orbit_cameras(n=8, radius=2.5, width=1920, height=1080, fov=45.0, seed=3):
    """n viewpoints on a sphere of ``radius`` around the origin: azimuths
    spread evenly with a seeded jitter, elevations seeded in [-0.5, 0.5]."""
    rng = np.random.default_rng(seed)
    cams = []
    for k in range(n):
        az = 2.0 * math.pi * (k + rng.uniform(-0.25, 0.25)) / n
        el = rng.uniform(-0.5, 0.5)
        eye = (radius * math.cos(el) * math.cos(az), radius * math.sin(el),
               radius * math.cos(el) * math.sin(az))
        cams.append(dict(eye=eye, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), fov=fov,
                         width=width, height=height))
    return cams


def _camera(c):
    cam = capi.MplCamera()
    for i in range(3):
        cam.eye[i] = c["eye"][i]
        cam.target[i] = c["target"][i]
        cam.up[i] = c["up"][i]
    cam.fov_y_deg = c["fov"]
    cam.width = c["width"]
    cam.height = c["height"]
    return cam


class SphereTracer:
    """Reusable buffers, and the captured step loop, for one image size."""

    def __init__(self, levels, deltas, width, height, max_steps=96, eps=1e-4, radius=1.2,
                 device="cuda", precision=None, graph=True, tail_from=None):
        self.levels = list(levels)
        self.deltas = list(deltas)
        if len(self.deltas) < len(self.levels) - 1:
            raise ValueError("one band width per residual level")
        self.W, self.H = int(width), int(height)
        self.P = self.W * self.H
        self.max_steps = int(max_steps)
        self.eps = float(eps)
        self.R = float(radius)
        self.device = torch.device(device)
        self.precision = precision
        self.use_graph = graph
        self.tail_from = None if tail_from is None else int(tail_from)
        P, dev = self.P, self.device
        f32 = dict(dtype=torch.float32, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        self.org = torch.empty(P, 3, **f32)
        self.dir = torch.empty(P, 3, **f32)
        self.S = torch.empty(P, **f32)
        self.G = torch.zeros(P, 3, **f32)
        self.state = torch.empty(P, **i32)
        self.active = [torch.empty(P, **i32), torch.empty(P, **i32)]
        self.hits = torch.empty(P, **i32)
        # counts: [active A, active B, hits, band 1, band 2, ...]
        self.counts = torch.zeros(3 + len(self.levels), **i32)
        self.bands = [torch.empty(P, **i32) for _ in range(len(self.levels) - 1)]
        self.image = torch.empty(P, dtype=torch.int32, device=dev)
        self._band_structs = [
            capi.MplBand(delta=float(self.deltas[i]), out_index=self.bands[i].data_ptr(),
                         count_dev=self.counts[3 + i:].data_ptr(), capacity=P)
            for i in range(len(self.levels) - 1)]
        self._pts = capi.MplPoints(kind=capi.MPL_POINTS_XYZ, xyz=self.org.data_ptr())
        self._graph = None
        self.launches_per_frame = 0

    def _prec(self, model):
        return capi.PRECISIONS[self.precision or getattr(model, "precision", "fp32")]

    def _levels_on(self, index, count_ptr, gradient, st):
        """Band-gated level launches on the rays index[0 .. *count_ptr)."""
        lib = capi.load()
        launches = 0
        for i, model in enumerate(self.levels):
            net, packed = model.packed()
            idx = index if i == 0 else capi.ptr(self.bands[i - 1])
            cnt = count_ptr if i == 0 else capi.ptr(self.counts[3 + i - 1:])
            band = (ctypes.byref(self._band_structs[i]) if i < len(self._band_structs) else None)
            mode = capi.MPL_STORE if i == 0 else capi.MPL_ACCUMULATE
            if gradient:
                capi.check(lib.mpl_level_gradient(
                    ctypes.byref(net), capi.ptr(packed), ctypes.byref(self._pts), idx, cnt,
                    self.P, capi.ptr(self.S), capi.ptr(self.G), mode, band, self._prec(model),
                    st), "mpl_level_gradient")
            else:
                capi.check(lib.mpl_level_forward(
                    ctypes.byref(net), capi.ptr(packed), ctypes.byref(self._pts), idx, cnt,
                    self.P, capi.ptr(self.S), mode, band, self._prec(model), st),
                    "mpl_level_forward")
            launches += 1
        return launches

    def _tail_step(self):
        """First step of the persistent marching launch, or None when every
        step runs as level launches (no tail requested, or a level in FP32)."""
        if self.tail_from is None or self.tail_from >= self.max_steps:
            return None
        precs = {self._prec(m) for m in self.levels}
        if len(precs) != 1 or precs.pop() == capi.MPL_FP32 or len(self.levels) > 3:
            return None
        return max(self.tail_from, 0)

    def _march(self, st):
        lib = capi.load()
        launches = 0
        tail = self._tail_step()
        for k in range(self.max_steps if tail is None else tail):
            a, b = k & 1, (k + 1) & 1
            launches += self._levels_on(capi.ptr(self.active[a]), capi.ptr(self.counts[a:]),
                                        False, st)
            capi.check(lib.mpl_trace_step(
                capi.ptr(self.S), capi.ptr(self.active[a]), capi.ptr(self.counts[a:]), self.P,
                capi.ptr(self.org), capi.ptr(self.dir), capi.ptr(self.state), self.eps, self.R,
                int(k == self.max_steps - 1), capi.ptr(self.active[b]),
                capi.ptr(self.counts[b:]), capi.ptr(self.hits), capi.ptr(self.counts[2:]),
                self.P, st), "mpl_trace_step")
            launches += 1
        if tail is not None:
            L = len(self.levels)
            nets = (capi.MplNet * L)()
            packed = (ctypes.c_void_p * L)()
            for i, model in enumerate(self.levels):
                net, pk = model.packed()
                nets[i] = net
                packed[i] = pk.data_ptr()
            deltas = (ctypes.c_float * max(L - 1, 1))(*[float(d) for d in self.deltas[:L - 1]])
            a = tail & 1
            capi.check(lib.mpl_trace_march(
                nets, ctypes.cast(packed, ctypes.c_void_p), L, ctypes.cast(deltas, ctypes.c_void_p),
                capi.ptr(self.active[a]), capi.ptr(self.counts[a:]),
                self.P, capi.ptr(self.org), capi.ptr(self.dir), capi.ptr(self.state),
                capi.ptr(self.S), self.eps, self.R, self.max_steps - tail, 1,
                capi.ptr(self.hits), capi.ptr(self.counts[2:]), self.P,
                self._prec(self.levels[0]), st), "mpl_trace_march")
            launches += 1
        return launches

    def render(self, camera, shade_mode=1):
        """Trace one frame; returns (image [H, W] RGBA8 as int32, state [P])."""
        lib = capi.load()
        for m in self.levels:
            m.packed()
        st = capi.stream_ptr()
        cam = _camera(camera)
        if cam.width != self.W or cam.height != self.H:
            raise ValueError("camera size differs from the tracer's buffers")
        capi.check(lib.mpl_trace_init(ctypes.byref(cam), self.R, capi.ptr(self.org),
                                      capi.ptr(self.dir), capi.ptr(self.state),
                                      capi.ptr(self.active[0]), capi.ptr(self.counts[0:]), st),
                   "mpl_trace_init")
        self.counts[2:3].zero_()
        launches = 1
        if self.use_graph:
            if self._graph is None:
                s = torch.cuda.Stream(self.device)
                s.wait_stream(torch.cuda.current_stream())
                with torch.cuda.stream(s):
                    self._march(capi.stream_ptr(s))  # warm the launch path once
                torch.cuda.current_stream().wait_stream(s)
                # the warm-up advanced the rays: restart the frame, then capture
                capi.check(lib.mpl_trace_init(ctypes.byref(cam), self.R, capi.ptr(self.org),
                                              capi.ptr(self.dir), capi.ptr(self.state),
                                              capi.ptr(self.active[0]),
                                              capi.ptr(self.counts[0:]), st), "mpl_trace_init")
                self.counts[2:3].zero_()
                torch.cuda.synchronize(self.device)
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    self._steps_in_graph = self._march(capi.stream_ptr())
                self._graph = g
            self._graph.replay()
            launches += self._steps_in_graph
        else:
            launches += self._march(st)
        # normals of the hits: band-gated level gradients summed
        launches += self._levels_on(capi.ptr(self.hits), capi.ptr(self.counts[2:]), True, st)
        capi.check(lib.mpl_trace_shade(capi.ptr(self.org), capi.ptr(self.dir), capi.ptr(self.G),
                                       capi.ptr(self.state), self.P, shade_mode,
                                       capi.ptr(self.image), st), "mpl_trace_shade")
        self.launches_per_frame = launches + 1
        return self.image.view(self.H, self.W), self.state
