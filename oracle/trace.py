"""numpy restatement of the band-gated sphere tracer (test oracle).

TEST INFRASTRUCTURE ONLY (see the package docstring).  Follows
renderer/cuda/kernels.cu:400-487 (rays, entry onto the bounding sphere),
kernels.cu:315-398 with state.cu:848-880 (the marching step) and
kernels.cu:65-120 (summed level normals), with the level sum gated by the
delta-bands as in i3d/meshing.py:221-231 and hits at |S| < eps.
"""

from __future__ import annotations

import math

import numpy as np

from . import siren


def camera_rays(cam, radius=1.2):
    """(origins, dirs, state) like mpl_trace_init (state 0 marching, 2 miss)."""
    eye = np.asarray(cam["eye"], np.float64)
    tgt = np.asarray(cam["target"], np.float64)
    up = np.asarray(cam["up"], np.float64)
    W, H = cam["width"], cam["height"]
    f = tgt - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    th = math.tan(0.5 * math.radians(cam["fov"]))
    i = np.tile(np.arange(W), H)
    j = np.repeat(np.arange(H), W)
    nx = 2.0 * i / W - 1.0
    ny = 1.0 - 2.0 * j / H
    d = (s[None] * (nx * th * W / H)[:, None] + u[None] * (ny * th)[:, None] + f[None])
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.broadcast_to(eye, d.shape).copy()
    b = (o * d).sum(1)
    c = (o * o).sum(1) - radius * radius
    state = np.zeros(len(d), np.int32)
    if c[0] > 0:
        disc = b * b - c
        ok = (b < 0) & (disc > 0)
        t = -b - np.sqrt(np.where(ok, disc, 0.0))
        o[ok] += t[ok, None] * d[ok]
        state[~ok] = 2
    return o, d, state


def banded_sum(levels, deltas, x):
    """S(x) with the finer levels only inside their bands; also the masks."""
    S = siren.siren_forward(*levels[0], x, np.float64)
    masks = []
    for i in range(1, len(levels)):
        m = np.abs(S) < deltas[i - 1]
        if i > 1:
            m &= masks[-1]
        if m.any():
            S[m] += siren.siren_forward(*levels[i], x[m], np.float64)
        masks.append(m)
    return S, masks


def trace(levels, deltas, cam, max_steps=96, eps=1e-4, radius=1.2):
    """Returns origins (final positions), state (1 hit, 2 miss, 3 budget)
    and the summed level gradients at the hits."""
    o, d, state = camera_rays(cam, radius)
    for k in range(max_steps):
        act = np.nonzero(state == 0)[0]
        if act.size == 0:
            break
        S, _ = banded_sum(levels, deltas, o[act])
        hit = np.abs(S) < eps
        state[act[hit]] = 1
        mv = act[~hit]
        o[mv] += d[mv] * S[~hit][:, None]
        out = ((o[mv] ** 2).sum(1) > radius * radius) & ((o[mv] * d[mv]).sum(1) > 0)
        state[mv[out]] = 2
        if k == max_steps - 1:
            rest = mv[~out]
            state[rest] = 3
    G = np.zeros_like(o)
    hits = np.nonzero(state == 1)[0]
    if hits.size:
        x = o[hits]
        S, masks = banded_sum(levels, deltas, x)
        g = siren.siren_input_grad(*levels[0], x)
        for i in range(1, len(levels)):
            m = masks[i - 1]
            if m.any():
                g[m] += siren.siren_input_grad(*levels[i], x[m])
        G[hits] = g
    return o, state, G
