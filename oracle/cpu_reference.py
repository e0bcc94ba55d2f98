"""The reference's band-culled reconstruction as it runs on the CPU, timed on
a bounded sample: the CPU baseline of the 512^3 reconstruction workload.

TEST INFRASTRUCTURE ONLY (see the package docstring): bench.py runs this
module, in a subprocess with a fixed thread environment, for both its CPU
legs (the GPU line's ``cpu_baseline`` and ``--impl reference``), so the two
numbers measure the same thing.

``multistage_sdf`` restates the sampling loop of create_mesh_multistage
(i3d/meshing.py:203-236) with the ops the reference issues on
``device="cpu"``: ``torch.nn.Linear`` layers with ``sin(w0 x)`` between them
(i3d/model.py:107-129, through oracle.torch_ref.PlainSiren), chunks of
``max_batch`` consecutive grid points (32^3 as reconstruct.py passes), the
band masks ``|S| < delta`` with boolean gathers and the per-chunk early exit.
Grid coordinates are made before the timed window, as the reference makes
them before its ``start_sampling`` (meshing.py:205-208).  Marching cubes is
oracle/mc.c, the project's C restatement (scikit-image, the reference's
marching cubes, is not installed), with OpenMP over i-planes.

Sample: ``pairs`` pairs of adjacent i-planes of the N^3 grid, one at the
centre of each of ``pairs`` equal intervals of the i axis.
Both planes of a pair are sampled (2 N^2 points), and marching cubes runs on
the pair (one layer of cells).  Per-point sampling time and per-layer
marching-cubes time are extrapolated to the N^3 grid and its N - 1 layers.

    python -m oracle.cpu_reference --weights W.npz --N 512 --pairs 8 --threads 16
"""

from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np


def load_levels(path):
    """(params, omegas) of each level of a three-level ``L{i}.net.{j}.0.*``
    weight file (the layout of tests/golden/three_level_sphere.npz)."""
    d = np.load(path)
    levels = []
    for i in range(3):
        sd = {k[3:]: d[k] for k in d.files if k.startswith(f"L{i}.")}
        n = len(sd) // 2
        params = [(sd[f"net.{j}.0.weight"], sd[f"net.{j}.0.bias"]) for j in range(n)]
        levels.append((params, [30.0] * (n - 1)))
    return levels


def multistage_sdf(models, deltas, coords, max_batch=32 ** 3):
    """S over ``coords`` [P, 3] (a run of consecutive grid points): the chunk
    loop of i3d/meshing.py:212-236 on the CPU.  Returns S and the number of
    points each residual level evaluated."""
    import torch

    def run(m, x):
        # SIREN.forward clones its input as a leaf that requires grad
        # (i3d/model.py:120-123) before the layers run
        return m(x.clone().detach().requires_grad_(True)).squeeze(-1)

    out = torch.empty(coords.shape[0])
    evaluated = [0] * (len(models) - 1)
    with torch.no_grad():
        head = 0
        while head < coords.shape[0]:
            sub = coords[head:head + max_batch]
            S = run(models[0], sub)
            for i in range(1, len(models)):
                if deltas:
                    idx = torch.abs(S) < deltas[i - 1]
                    if not idx.any():
                        break
                    S[idx] += run(models[i], sub[idx, ...])
                    evaluated[i - 1] += int(idx.sum())
                else:
                    S += run(models[i], sub)
                    evaluated[i - 1] += sub.shape[0]
            out[head:head + max_batch] = S
            head += max_batch
    return out, evaluated


def sample(levels, deltas, N, pairs, threads):
    """Times the sample; returns (pts/s of the whole N^3 step, detail)."""
    import torch
    from . import mc, siren
    from .torch_ref import PlainSiren
    torch.set_num_threads(threads)
    models = [PlainSiren(p, om).eval() for p, om in levels]
    # the first plane of each pair: the centres of `pairs` equal intervals
    planes = np.unique(((np.arange(pairs) + 0.5) * (N - 1) / pairs).astype(np.int64))
    vs = 2.0 / (N - 1)
    coords = [torch.from_numpy(siren.grid_coords(N, vs, np.arange(2 * N * N) + i * N * N))
              for i in planes]
    # one untimed chunk: thread pool and allocator warm-up
    multistage_sdf(models, deltas, coords[0][:32 ** 3])
    t_sdf = t_mc = 0.0
    evaluated = np.zeros(len(levels) - 1, np.int64)
    tris = 0
    for c in coords:
        t0 = time.perf_counter()
        S, ev = multistage_sdf(models, deltas, c)
        t1 = time.perf_counter()
        _, f, _, _ = mc.marching_cubes_raw(S.numpy().reshape(2, N, N), 0.0, np.float32(vs),
                                           (-1.0, -1.0, -1.0))
        t2 = time.perf_counter()
        t_sdf += t1 - t0
        t_mc += t2 - t1
        evaluated += ev
        tris += f.shape[0]
    pts = len(planes) * 2 * N * N
    full = t_sdf * N ** 3 / pts + t_mc * (N - 1) / len(planes)
    detail = {"sample": f"{len(planes)} pairs of adjacent {N}x{N} planes (one per equal "
                        f"interval of the i axis) of the "
                        f"{N}^3 grid ({pts} points; residual levels on {evaluated.tolist()} of "
                        f"them; {tris} triangles): the reference's chunked torch loop "
                        f"(32^3-point chunks, {threads} threads) and the C marching cubes of "
                        "each pair, extrapolated to the full grid and its cell layers",
              "points_sampled": pts, "sdf_seconds_sample": round(t_sdf, 4),
              "mc_seconds_sample": round(t_mc, 4), "seconds_full_estimate": round(full, 3),
              "threads": threads}
    return N ** 3 / full, detail


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--weights", required=True)
    ap.add_argument("--N", type=int, default=512)
    ap.add_argument("--pairs", type=int, default=8)
    ap.add_argument("--repeats", type=int, default=1)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--deltas", type=float, nargs="*", default=[0.05, 0.01])
    a = ap.parse_args(argv)
    levels = load_levels(a.weights)
    vals, details = [], []
    for _ in range(a.repeats):
        v, d = sample(levels, a.deltas, a.N, a.pairs, a.threads)
        vals.append(v)
        details.append(d)
    print(json.dumps({"values": vals, "detail": details[-1]}), flush=True)


if __name__ == "__main__":
    main()
