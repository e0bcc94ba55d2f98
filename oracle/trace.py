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


def camera_rays(cam, radius=1.2, pixels=None):
    """(origins, dirs, state) like mpl_trace_init (state 0 marching, 2 miss),
    for every pixel (row-major, row 0 at the top) or for the pixel indices
    ``pixels`` only (rays are independent)."""
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
    r = np.arange(W * H) if pixels is None else np.asarray(pixels, np.int64)
    i = r % W
    j = r // W
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


def trace(levels, deltas, cam, max_steps=96, eps=1e-4, radius=1.2, pixels=None):
    """Returns origins (final positions), state (1 hit, 2 miss, 3 budget)
    and the summed level gradients at the hits, for every pixel or for the
    pixel indices ``pixels``."""
    o, d, state = camera_rays(cam, radius, pixels)
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


def banded_gradient(levels, deltas, x):
    """Sum of the level gradients at x with the finer levels gated by their
    bands (the normals of kernels.cu:65-120 with band gating), float64;
    also the partial sums S_0, S_0 + S_1, ... that decided the gating."""
    S, masks = banded_sum(levels, deltas, x)
    g = siren.siren_input_grad(*levels[0], x)
    partial = [siren.siren_forward(*levels[0], x, np.float64)]
    for i in range(1, len(levels)):
        m = masks[i - 1]
        if m.any():
            g[m] += siren.siren_input_grad(*levels[i], x[m])
        nxt = partial[-1].copy()
        if m.any():
            nxt[m] += siren.siren_forward(*levels[i], x[m], np.float64)
        partial.append(nxt)
    return g, S, partial


def shade(org, dirs, G, state, mode=1):
    """RGBA8 pixels (packed little-endian into uint32) of Shade_kernel,
    renderer/cuda/kernels.cu:191-268, in float32: a hit inside the unit cube
    gets, with n = G/|G| and the light along the view direction l = -d,
    0.2 + 1 * max(n.l, 0) * 0.54 + 0.5 * max((l.r)^35, 0) on every channel,
    r = 2 (n.l) n - l (mode 1), or (|n_x|, |n_z|, |n_y|) (mode 0); every
    other pixel is white.  Channels are clamp(c, 0, 1) * 255 truncated
    (kernels.cu:29-39)."""
    f32 = np.float32
    org = np.asarray(org, f32)
    dirs = np.asarray(dirs, f32)
    G = np.asarray(G, f32)
    n = G.shape[0]

    def q(v):
        return (np.clip(v, f32(0), f32(1)) * f32(255)).astype(np.uint32)

    def pack(r, g, b):
        return (np.uint32(255) << np.uint32(24)) | (q(b) << np.uint32(16)) | \
            (q(g) << np.uint32(8)) | q(r)

    white = pack(np.ones(n, f32), np.ones(n, f32), np.ones(n, f32))
    inside = (np.abs(org) < f32(1)).all(1)
    hit = (np.asarray(state) == 1) & inside
    with np.errstate(invalid="ignore", divide="ignore"):
        ln = np.sqrt((G * G).sum(1, dtype=f32)).astype(f32)
        nrm = (G / ln[:, None]).astype(f32)
        if mode == 0:
            img = pack(np.abs(nrm[:, 0]), np.abs(nrm[:, 2]), np.abs(nrm[:, 1]))
        else:
            l = -dirs
            nl = (l * nrm).sum(1, dtype=f32).astype(f32)
            refl = (f32(2) * nl[:, None] * nrm - l).astype(f32)
            rv = (l * refl).sum(1, dtype=f32).astype(f32)
            spec = np.maximum(np.power(np.maximum(rv, f32(0)), f32(35)), f32(0)).astype(f32)
            c = (f32(0.2) + f32(1) * np.maximum(nl, f32(0)) * f32(0.54) + f32(0.5) * spec)
            c = c.astype(f32)
            img = pack(c, c, c)
    return np.where(hit, img, white).astype(np.uint32)
