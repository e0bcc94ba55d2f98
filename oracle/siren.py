"""numpy restatement of the reference SIREN evaluation path (test oracle).

Every function names the reference lines it follows.  Parameters are passed
as a list of ``(W, b)`` pairs in ``nn.Linear`` layout (``W`` is
``[out, in]``), with one omega per sine layer, exactly as
``i3d/model.py:88-103`` builds them.
"""

from __future__ import annotations

import numpy as np


def siren_forward(params, omegas, x, dtype=np.float32):
    """SIREN forward, i3d/model.py:107-129 (and SineLayer, :32-33).

    ``y = W x + b`` per layer; every layer but the last is followed by
    ``sin(omega * y)``.  Returns ``[P]`` (the squeezed ``model_out``).
    """
    h = np.asarray(x, dtype=dtype)
    n = len(params)
    for l, (W, b) in enumerate(params):
        W = np.asarray(W, dtype=dtype)
        b = np.asarray(b, dtype=dtype)
        h = h @ W.T + b
        if l < n - 1:
            h = np.sin(dtype(omegas[l]) * h)
    return h[:, 0]


def siren_input_grad(params, omegas, x):
    """d f / d x in FP64 by reverse mode (what i3d/diff_operators.py:259-265
    obtains from autograd on the same network)."""
    h = np.asarray(x, np.float64)
    zs = []
    n = len(params)
    for l, (W, b) in enumerate(params[:-1]):
        z = omegas[l] * (h @ np.asarray(W, np.float64).T + np.asarray(b, np.float64))
        zs.append(z)
        h = np.sin(z)
    g = np.broadcast_to(np.asarray(params[-1][0], np.float64)[0], h.shape).copy()
    for l in range(n - 2, -1, -1):
        g = g * np.cos(zs[l]) * omegas[l]
        g = g @ np.asarray(params[l][0], np.float64)
    return g


def grid_coords(N, voxel_size, index=None, voxel_origin=(-1, -1, -1)):
    """Grid coordinates of i3d/meshing.py:42-63, reproduced bit for bit.

    The reference writes ``(idx.long() / N) % N`` which, under PyTorch's true
    division, is ``fmod(float32(idx) / float32(N), N)`` in float32, so x and y
    carry fractional offsets.  The coordinate is then
    ``float32(s * float32(voxel_size)) + origin`` with two separate roundings.
    """
    if index is None:
        index = np.arange(N ** 3, dtype=np.int64)
    index = np.asarray(index, np.int64)
    fN = np.float32(N)
    idx_f = index.astype(np.float32)
    s2 = (index % N).astype(np.float32)
    q1 = idx_f / fN
    s1 = np.fmod(q1, fN)
    s0 = np.fmod(q1 / fN, fN)
    vs = np.float32(voxel_size)
    out = np.empty((index.shape[0], 3), np.float32)
    out[:, 0] = (s0 * vs) + np.float32(voxel_origin[2])
    out[:, 1] = (s1 * vs) + np.float32(voxel_origin[1])
    out[:, 2] = (s2 * vs) + np.float32(voxel_origin[0])
    return out


def band_mask(S, delta):
    """``torch.abs(sdf_base) < deltas[i - 1]`` of i3d/meshing.py:223: a
    float32 tensor against a Python float compares in float32."""
    return np.abs(np.asarray(S, np.float32)) < np.float32(delta)


def multistage_sdf(levels, deltas, N, chunk=32 ** 3, index=None):
    """Band-culled evaluation of i3d/meshing.py:203-236 on the grid.

    ``levels`` is a list of ``(params, omegas)``, coarse first.  With
    ``deltas == []`` every level runs on every point (:232-233).  Returns the
    SDF array over ``index`` (default: all N^3 points) and the band index
    lists (positions into ``index``) of every residual level.
    """
    if index is None:
        index = np.arange(N ** 3, dtype=np.int64)
    vs = 2.0 / (N - 1)
    out = np.empty(index.shape[0], np.float32)
    bands = [[] for _ in range(len(levels) - 1)]
    for head in range(0, index.shape[0], chunk):
        sel = index[head:head + chunk]
        pts = grid_coords(N, vs, sel)
        S = siren_forward(*levels[0], pts)
        for i in range(1, len(levels)):
            if deltas:
                m = band_mask(S, deltas[i - 1])
                if not m.any():
                    break
                S[m] += siren_forward(*levels[i], pts[m])
                bands[i - 1].append(np.nonzero(m)[0] + head)
            else:
                S += siren_forward(*levels[i], pts)
        out[head:head + chunk] = S
    bands = [np.concatenate(b) if b else np.zeros(0, np.int64) for b in bands]
    return out, bands


def adaptive_deltas(levels, pts, eps=0.3, batch=2 ** 18):
    """reconstruct.py:18-33: delta_i = (1 + eps) * max_j |sum_{k<i} f_k(x_j)|."""
    deltas = []
    for level in range(1, len(levels)):
        worst = 0.0
        for i in range(0, pts.shape[0], batch):
            chunk = pts[i:i + batch]
            s = sum(siren_forward(*levels[k], chunk) for k in range(level))
            worst = max(worst, float(np.abs(s).max()))
        deltas.append((1.0 + eps) * worst)
    return deltas


def params_from_state_dict(sd):
    """Layer list from an ``i3d.model.SIREN`` state_dict (keys
    ``net.{i}.0.weight|bias``), i3d/model.py:349-367."""
    keys = list(sd.keys())
    params = []
    for i in range(0, len(keys), 2):
        W = np.asarray(sd[keys[i]], np.float32)
        b = np.asarray(sd[keys[i + 1]], np.float32)
        params.append((W, b))
    return params


def multistage_sdf_threaded(levels, deltas, N, index, threads, chunk=32 ** 3):
    """``multistage_sdf`` over ``index`` with the chunks spread over a thread
    pool (numpy releases the GIL in matmul and sin).  Used to time the CPU
    baseline on the host's cores; with OPENBLAS_NUM_THREADS=1 each chunk is
    single-threaded and the pool provides the parallelism."""
    from concurrent.futures import ThreadPoolExecutor

    index = np.asarray(index, np.int64)
    heads = list(range(0, index.shape[0], chunk))
    out = np.empty(index.shape[0], np.float32)
    band_sizes = np.zeros((len(heads), max(len(levels) - 1, 1)), np.int64)

    def work(t):
        head = heads[t]
        S, bands = multistage_sdf(levels, deltas, N, chunk=chunk, index=index[head:head + chunk])
        out[head:head + chunk] = S
        for i, b in enumerate(bands):
            band_sizes[t, i] = b.shape[0]

    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(work, range(len(heads))))
    return out, band_sizes.sum(0)
