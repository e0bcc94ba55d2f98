"""The synthetic surface of the three-level workload and its training batches.

Surface: r(theta, phi) = 0.6 + 0.03 sin(12 theta) sin(12 phi) in spherical
coordinates (theta polar), with analytic normals.  The reference trains on
scanned meshes read with open3d and queries their SDF with an open3d
raycasting scene (i3d/dataset.py:181-287); neither is available, so the
off-surface SDF here is the distance to a dense surface sample (scipy
cKDTree), signed by comparing |p| with r(theta(p), phi(p)).
"""

from __future__ import annotations

import numpy as np

R0, AMP, FREQ = 0.6, 0.03, 12.0


def radius(theta, phi):
    return R0 + AMP * np.sin(FREQ * theta) * np.sin(FREQ * phi)


def surface_points(n, rng, noise=0.0):
    """n points uniform in (cos theta, phi) on the surface, their unit
    normals, and optional Gaussian position noise (normals unchanged)."""
    theta = np.arccos(1.0 - 2.0 * rng.random(n))
    phi = 2.0 * np.pi * rng.random(n)
    pts, nrm = _point_normal(theta, phi)
    if noise > 0:
        pts = pts + rng.normal(0.0, noise, pts.shape)
    return pts.astype(np.float32), nrm.astype(np.float32)


def surface_mesh(n_theta, n_phi):
    """The surface as a closed triangle mesh: a pole vertex at each end and
    ``n_theta - 1`` rings of ``n_phi`` vertices, every quad split in two.
    Returns float32 positions [V, 3], unit normals [V, 3] and int32 faces
    [F, 3] (V = (n_theta - 1) n_phi + 2, F = 2 (n_theta - 1) n_phi)."""
    if n_theta < 2 or n_phi < 3:
        raise ValueError("surface_mesh needs n_theta >= 2 and n_phi >= 3")
    t = np.pi * np.arange(1, n_theta) / n_theta
    p = 2.0 * np.pi * np.arange(n_phi) / n_phi
    theta = np.concatenate([[0.0], np.repeat(t, n_phi), [np.pi]])
    phi = np.concatenate([[0.0], np.tile(p, n_theta - 1), [0.0]])
    pts, nrm = _point_normal(theta, phi)
    rings = n_theta - 1
    ring = lambda i: 1 + i * n_phi  # noqa: E731  first vertex of ring i
    j = np.arange(n_phi)
    jn = (j + 1) % n_phi
    faces = [np.stack([np.zeros(n_phi, np.int64), ring(0) + j, ring(0) + jn], 1)]
    for i in range(rings - 1):
        a, b = ring(i) + j, ring(i) + jn
        c, d = ring(i + 1) + j, ring(i + 1) + jn
        faces += [np.stack([a, c, b], 1), np.stack([b, c, d], 1)]
    south = 1 + rings * n_phi
    faces.append(np.stack([ring(rings - 1) + j, np.full(n_phi, south), ring(rings - 1) + jn], 1))
    return (pts.astype(np.float32), nrm.astype(np.float32),
            np.concatenate(faces).astype(np.int32))


def _point_normal(theta, phi):
    r = radius(theta, phi)
    st, ct, sp, cp = np.sin(theta), np.cos(theta), np.sin(phi), np.cos(phi)
    rhat = np.stack([st * cp, st * sp, ct], 1)
    that = np.stack([ct * cp, ct * sp, -st], 1)
    phat = np.stack([-sp, cp, np.zeros_like(sp)], 1)
    dr_dt = AMP * FREQ * np.cos(FREQ * theta) * np.sin(FREQ * phi)
    dr_dp = AMP * FREQ * np.sin(FREQ * theta) * np.cos(FREQ * phi)
    st_safe = np.where(np.abs(st) < 1e-9, 1e-9, st)
    g = rhat - (dr_dt / r)[:, None] * that - (dr_dp / (r * st_safe))[:, None] * phat
    nrm = g / np.linalg.norm(g, axis=1, keepdims=True)
    return r[:, None] * rhat, nrm


def inside_sign(p):
    """-1 inside the surface, +1 outside."""
    rho = np.linalg.norm(p, axis=1)
    theta = np.arccos(np.clip(p[:, 2] / np.maximum(rho, 1e-12), -1.0, 1.0))
    phi = np.arctan2(p[:, 1], p[:, 0])
    return np.where(rho < radius(theta, phi), -1.0, 1.0)


def radial_distance(p):
    """| |p| - r(theta(p), phi(p)) |: an upper bound of the distance to the
    surface along the ray from the origin."""
    rho = np.linalg.norm(p, axis=1)
    theta = np.arccos(np.clip(p[:, 2] / np.maximum(rho, 1e-12), -1.0, 1.0))
    phi = np.arctan2(p[:, 1], p[:, 0])
    return np.abs(rho - radius(theta, phi))


class SignedDistance:
    """Signed distance: nearest dense surface sample within ``bound``, the
    radial distance beyond it (nearest-neighbour queries far from a closed
    surface visit most of the tree), and the sign from ``inside_sign``."""

    def __init__(self, n_dense=1 << 21, seed=123, bound=0.1):
        from scipy.spatial import cKDTree
        pts, _ = surface_points(n_dense, np.random.default_rng(seed))
        self.tree = cKDTree(pts)
        self.bound = bound

    def __call__(self, p):
        d, _ = self.tree.query(p, distance_upper_bound=self.bound, workers=-1)
        far = ~np.isfinite(d)
        if far.any():
            d[far] = np.maximum(radial_distance(p[far]), self.bound)
        return (d * inside_sign(p)).astype(np.float32)
