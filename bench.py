#!/usr/bin/env python
"""Benchmark of the band-culled three-level reconstruction on one GB300.

Workload: three 3->256x3->1 SIREN levels (omega0 = 30) trained on the
synthetic surface r = 0.6 + 0.03 sin(12 theta) sin(12 phi)
(tests/golden/three_level_sphere.npz); the 512^3 grid of
gen_mc_coordinate_grid; bands delta0 = 0.05, delta1 = 0.01; marching cubes at
0.  One step = level 0 on all 134,217,728 grid points (fused band list),
level 1 on band 1, level 2 on band 2, marching cubes (count + emit) on the
device.  ``value`` is grid points per second of that step with the 16-bit
tcgen05 kernels (FP16 operands, the form that meets the SDF error target;
BF16 beside it); the same step with the plain FP32 kernels, the error of each
against the FP64 oracle, the end-to-end number through the public API with
host buffers, the CPU baseline and the roofline of the dominant kernel are in
the same JSON line, next to the training step, sphere tracing, the batched
64-model launch and calc_deltas sub-benchmarks.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun (N > 1) every rank runs the same workload as an independent
replica (the path has no exchange step); rank 0 prints the line.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("fused BF16 vs plain FP32 SDF pts/s & 512³ banded-MC ms on 1 GB300 "
          "at equal error")
WEIGHTS = os.path.join(ROOT, "tests", "golden", "three_level_sphere.npz")
DELTAS = [0.05, 0.01]
# FP32 re-evaluation margins: about four times the largest tensor-core error
# of a partial sum measured near the surface (BF16 ~5e-4, FP16 ~2.5e-4)
REFINE = {"bf16": 2e-3, "fp16": 1e-3}
# The headline's tensor-core operand type.  The metric asks for the fused
# 16-bit evaluator at equal error (SDF max <= 5e-4 and Chamfer <= 1e-6 against
# float64): FP16 operands meet both (2.3e-4); BF16 operands, whose 8-bit
# mantissa rounds the hidden activations, reach 1.5e-3 and are reported
# beside it under variants.bf16 and errors_vs_fp64.bf16.
HEADLINE = "fp16"
FLOP_PER_POINT = 2 * (3 * 256 + 256 * 256 * 2 + 256)  # 264,192 per level evaluation
KERNEL_LAUNCHES_PER_STEP = 3 + 5  # 3 level launches; MC count, 3 scan passes, emit


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--N", type=int, default=512)
    ap.add_argument("--fp32-steps", type=int, default=2)
    ap.add_argument("--cpu-repeats", type=int, default=3,
                    help="CPU samples of the GPU line's cpu_baseline leg")
    ap.add_argument("--skip-errors", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--bf16-unit", type=int, default=None, choices=[16, 32],
                    help="epilogue unit width of the tensor-core kernels (default: the "
                         "library's)")
    ap.add_argument("--headline", choices=["fp16", "bf16"], default=HEADLINE,
                    help="operand type of the headline step (profiling runs)")
    ap.add_argument("--skip-train", action="store_true")
    ap.add_argument("--skip-trace", action="store_true")
    ap.add_argument("--skip-batch", action="store_true")
    ap.add_argument("--skip-deltas", action="store_true")
    ap.add_argument("--only", choices=["train", "trace", "batch", "deltas"], default=None,
                    help="run one sub-benchmark alone and print its JSON (profiling runs)")
    ap.add_argument("--profile-only", action="store_true",
                    help="time only the BF16 steps (for profiler runs) and print a short line")
    return ap.parse_args()


def load_levels_np():
    d = np.load(WEIGHTS)
    levels = []
    for i in range(3):
        sd = {k[3:]: d[k] for k in d.files if k.startswith(f"L{i}.")}
        keys = sorted(sd, key=lambda k: (int(k.split(".")[1]), k.endswith("bias")))
        params = [(sd[keys[j]], sd[keys[j + 1]]) for j in range(0, len(keys), 2)]
        levels.append((sd, params))
    return levels


def rank_info():
    from mplicits_gb300.replicas import rank_info as _ri
    return _ri()


def peaks(sustained=False):
    """(bf16 TFLOP/s, HBM GB/s, source).  The burst bf16 figure is the
    comparator of a kernel that runs at full clock with no power cap (the
    level-0 launch of a 40 ms step); the sustained one is for kernels timed
    inside long power-capped loops."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        tf = (p.get("bf16_tflops_sustained") if sustained else None) or p["bf16_tflops"]
        return tf, p["hbm_gbs"], "measured"
    return (1700.0 if sustained else 1900.0), 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        rows = [r.split(",") for r in (self.out or "").strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows]
        mx = float(rows[0][2])
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if r[5 + i].strip().lower() == "active"})
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


def make_models(levels_np, precision, device):
    import torch
    from mplicits_gb300.model import SIREN
    models = []
    for sd, _ in levels_np:
        m = SIREN(3, 1, [256, 256, 256], w0=30, delay_init=True, precision=precision)
        m.load_state_dict({k: torch.from_numpy(v) for k, v in sd.items()})
        models.append(m.to(device).eval())
    return models


class Step:
    """One band-culled reconstruction on resident weights, no host sync."""

    def __init__(self, models, N, device, precision, refine_margin=None):
        import torch
        from mplicits_gb300.meshing import BandedReconstruction, MarchingCubes
        self.rec = BandedReconstruction(models, DELTAS, N, device, precision, refine_margin)
        self.mc = MarchingCubes(N, device)
        for m in models:
            m.packed()
        self.rec.sample()
        counts = self.mc.count(self.rec.S).cpu()
        self.V, self.F = int(counts[0]), int(counts[1])
        cap_v, cap_f = int(self.V * 1.05) + 1024, int(self.F * 1.05) + 1024
        self.verts = torch.empty(cap_v, 3, device=device)
        self.normals = torch.empty(cap_v, 3, device=device)
        self.values = torch.empty(cap_v, device=device)
        self.faces = torch.empty(cap_f, 3, dtype=torch.int32, device=device)
        self.cap = (cap_v, cap_f)
        self.ev = []

    def __call__(self, l0_events=None):
        import ctypes
        from mplicits_gb300 import capi
        rec = self.rec
        if l0_events is not None and not rec.refine_margin:
            l0_events[0].record()
            self._level(0)
            l0_events[1].record()
            for i in range(1, len(rec.levels)):
                self._level(i)
        else:
            rec.sample()
        self.mc.count(rec.S)
        org = (ctypes.c_float * 3)(-1.0, -1.0, -1.0)
        capi.check(capi.load().mpl_mc_emit(
            capi.ptr(rec.S), rec.N, 0.0, float(np.float32(rec.voxel_size)), org,
            capi.ptr(self.mc.ws), capi.ptr(self.verts), capi.ptr(self.normals),
            capi.ptr(self.values), capi.ptr(self.faces), self.cap[0], self.cap[1],
            capi.stream_ptr()), "mpl_mc_emit")

    def _level(self, i):
        # the launches of BandedReconstruction.sample(), one level at a time
        import ctypes
        from mplicits_gb300 import capi
        rec = self.rec
        model = rec.levels[i]
        net, packed = model.packed()
        lib = capi.load()
        st = capi.stream_ptr()
        if i == 0:
            capi.check(lib.mpl_level_forward(
                ctypes.byref(net), capi.ptr(packed), ctypes.byref(rec.points), None, None, rec.n,
                capi.ptr(rec.S), capi.MPL_STORE, ctypes.byref(rec._bands[0]), rec._prec(model),
                st), "mpl_level_forward")
        else:
            band = ctypes.byref(rec._bands[i]) if i < len(rec._bands) else None
            capi.check(lib.mpl_level_forward(
                ctypes.byref(net), capi.ptr(packed), ctypes.byref(rec.points),
                capi.ptr(rec.band_index[i - 1]), capi.ptr(rec.band_count[i - 1:]), rec.n,
                capi.ptr(rec.S), capi.MPL_ACCUMULATE, band, rec._prec(model), st),
                "mpl_level_forward")


def time_steps(step, K, W, with_l0=True):
    """W untimed steps, then exactly K steps between CUDA events, bracketed
    by a barrier over the replicas and a device synchronisation on both
    sides."""
    import torch
    from mplicits_gb300.replicas import barrier
    for _ in range(W):
        step()
    l0 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(K)] if with_l0 else None
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    e0.record()
    for k in range(K):
        step(l0[k] if with_l0 else None)
    e1.record()
    torch.cuda.synchronize()
    barrier()
    total_ms = e0.elapsed_time(e1)
    l0_ms = (float(np.mean([a.elapsed_time(b) for a, b in l0]))
             if with_l0 and not step.rec.refine_margin else None)
    return total_ms / K, l0_ms


def error_stats(step, models, N, seed=0):
    """Max/RMS |S - S_fp64| over 2^20 random grid points plus every point with
    |S| < 0.02 (which holds every crossing-edge end), using the run's own band
    membership; Chamfer of the mesh against the mesh of the FP64 values."""
    import torch
    from oracle import fp64
    from mplicits_gb300.meshing import MarchingCubes
    rec = step.rec
    dev = rec.S.device
    S = rec.S
    n = rec.n
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    rand = torch.randint(0, n, (1 << 20,), device=dev, generator=g)
    near = torch.nonzero(S.abs() < 0.02).squeeze(1)
    idx = torch.unique(torch.cat([rand, near]))
    sizes = rec.band_sizes()
    member = []
    for i in range(2):
        b = rec.band_index[i][:sizes[i]].long()
        m = torch.zeros(n, dtype=torch.bool, device=dev)
        m[b] = True
        member.append(m[idx])
    xyz = fp64.grid_xyz(N, idx, dev)
    S64 = torch.zeros(idx.numel(), dtype=torch.float64, device=dev)
    for lv, model in enumerate(models):
        params, om = fp64.level_params64(model, dev)
        sel = torch.ones_like(member[0]) if lv == 0 else member[lv - 1]
        S64[sel] += fp64.forward64(params, om, xyz[sel])
    err = (S[idx].double() - S64).abs()
    # every crossing-edge end must be inside the re-evaluated set
    Sv = S.view(N, N, N)
    worst_end = 0.0
    for ax in range(3):
        a = Sv.narrow(ax, 0, N - 1)
        b = Sv.narrow(ax, 1, N - 1)
        cross = (a < 0) != (b < 0)
        if cross.any():
            worst_end = max(worst_end, float(torch.maximum(a.abs(), b.abs())[cross].max()))
    S_ref = S.clone()
    nm = torch.isin(idx, near)
    S_ref[idx[nm]] = S64[nm].float()
    mc = MarchingCubes(N, dev)
    va = mc(S, 0.0, rec.voxel_size, (-1.0, -1.0, -1.0))[0]
    vb = mc(S_ref, 0.0, rec.voxel_size, (-1.0, -1.0, -1.0))[0]
    fa = mc(S, 0.0, rec.voxel_size, (-1.0, -1.0, -1.0))[1]
    fb = mc(S_ref, 0.0, rec.voxel_size, (-1.0, -1.0, -1.0))[1]
    if va.shape == vb.shape and torch.equal(fa, fb):
        # same topology: vertex i of one mesh is vertex i of the other
        chamfer = fp64.chamfer_matched_upper(va, vb)
        how = "matched-vertex upper bound"
    else:
        chamfer = fp64.chamfer_kdtree(va.cpu().numpy(), vb.cpu().numpy())
        how = "k-d tree"
    return {"sdf_max": float(err.max()), "sdf_rms": float(torch.sqrt((err ** 2).mean())),
            "points": int(idx.numel()), "chamfer": chamfer, "chamfer_method": how,
            "crossing_edge_end_max_abs_S": worst_end}


def mc_ambiguity(S, N):
    """Case histogram of the volume's cells (on the device) and the number of
    surface cells whose topology a face or interior test (Lewiner et al.
    2003, scikit-image's method) could resolve differently from this
    project's fixed face rule (mplicits_gb300.mc_tables.ambiguity_classes)."""
    import torch
    from mplicits_gb300.mc_tables import ambiguity_classes
    V = (S.view(N, N, N) < 0).to(torch.uint8)
    case = torch.zeros(N - 1, N - 1, N - 1, dtype=torch.uint8, device=S.device)
    for c in range(8):
        di, dj, dk = c & 1, (c >> 1) & 1, (c >> 2) & 1
        case |= V[di:N - 1 + di, dj:N - 1 + dj, dk:N - 1 + dk] << c
    hist = torch.bincount(case.reshape(-1), minlength=256).cpu().numpy()
    cls = ambiguity_classes()
    surface = int(hist.sum() - hist[0] - hist[255])
    face = int(sum(hist[c] for c in range(256) if cls[c][0]))
    interior = int(sum(hist[c] for c in range(256) if cls[c][1]))
    return {"surface_cells": surface, "cells_with_ambiguous_face": face,
            "cells_with_interior_ambiguity": interior,
            "fraction_ambiguous": (face + interior) / max(1, surface)}


def e2e_run(levels_np, N, device, K, W, precision):
    """The public API end to end: weights from pinned host memory, the
    band-culled reconstruction, marching cubes, mesh back to pinned host
    memory, every step."""
    import torch
    from mplicits_gb300.meshing import BandedReconstruction
    models = make_models(levels_np, precision, device)
    host = [[p.detach().cpu().pin_memory() for p in m.parameters()] for m in models]
    h2d = sum(t.numel() * t.element_size() for hs in host for t in hs)
    rec = BandedReconstruction(models, DELTAS, N, device, precision)
    out_host = {}
    d2h = [0]

    def step():
        with torch.no_grad():
            for m, hs in zip(models, host):
                for p, h in zip(m.parameters(), hs):
                    p.copy_(h, non_blocking=True)
        rec.sample()
        verts, faces, normals, values = rec.mesh()
        nb = 0
        for name, t in (("v", verts), ("f", faces), ("n", normals), ("s", values)):
            buf = out_host.get(name)
            if buf is None or buf.numel() < t.numel():
                buf = torch.empty(int(t.numel() * 1.2) + 1024, dtype=t.dtype, pin_memory=True)
                out_host[name] = buf
            buf[:t.numel()].copy_(t.reshape(-1), non_blocking=True)
            nb += t.numel() * t.element_size()
        d2h[0] = nb
        torch.cuda.current_stream().synchronize()

    for _ in range(W):
        step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(K):
        step()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / K
    launches = 3 + 5 + 3 * 4  # levels, MC, re-packing each level's weights
    return dt, h2d, d2h[0], launches


CPU_PAIRS = 4  # plane pairs per CPU sample step (2 * 4 * 512^2 = 2,097,152 points at 512^3)


def config_of(N, world):
    """The workload's description, the same in both arms' JSON lines."""
    return {"workload": f"3-level band-culled reconstruction, {N}^3 grid ({N ** 3} points), "
                        "3->256x3->1 SIREN levels (omega0 30, trained on the synthetic sphere), "
                        "deltas 0.05/0.01, marching cubes",
            "grid": N, "deltas": DELTAS,
            "l2": f"working set larger than L2 (129 MB) at 512^3: the {4 * N ** 3 / 1e6:.0f} MB "
                  "SDF volume is written and read every step",
            "parallelism": f"replicas x{world}",
            "arithmetic": "fused 16-bit tensor-core evaluator with FP16 operands (kind::f16, FP32 "
                          "accumulation, FP32 first layer and sines): the operand type that "
                          "meets the metric's SDF-max clause; BF16 operands reported beside"}


def cpu_reference_samples(N, repeats, pairs=CPU_PAIRS, threads=None):
    """The reference's reconstruction loop on the host cores (oracle/
    cpu_reference.py: its chunked torch sampling plus the C marching cubes),
    ``repeats`` timed samples of ``pairs`` plane pairs each, run in a child
    process whose thread environment is fixed here, so every CPU leg of the
    benchmark measures the same thing.  Returns (pts/s per sample, detail,
    wall seconds per sample)."""
    threads = threads or os.cpu_count() or 1
    env = dict(os.environ)
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        env[var] = str(threads)
    env.pop("CUDA_VISIBLE_DEVICES", None)
    cmd = [sys.executable, "-m", "oracle.cpu_reference", "--weights", WEIGHTS, "--N", str(N),
           "--pairs", str(pairs), "--repeats", str(repeats), "--threads", str(threads),
           "--deltas", *map(str, DELTAS)]
    t0 = time.perf_counter()
    out = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, check=True)
    wall = (time.perf_counter() - t0) / max(1, repeats)
    res = json.loads(out.stdout.strip().splitlines()[-1])
    return res["values"], res["detail"], wall


TRAIN_SURFACE = 1 << 16  # surface samples per batch; rows = 3x (surface, offset, dithered)
# per row: two frozen levels and the trainable level in forward mode (value
# row 2*(3*256 + 2*256*256 + 256), three tangent rows 2*(2*256*256 + 256)),
# then the backward GEMM d_a W and the weight-gradient GEMM of the two hidden
# layers over the four rows
_FWD_TANGENT = 2 * (3 * 256 + 2 * 256 * 256 + 256) + 3 * 2 * (2 * 256 * 256 + 256)
TRAIN_FLOP_PER_ROW = 3 * _FWD_TANGENT + 2 * (2 * 4 * 2 * 256 * 256)
TRAIN_LAUNCHES_PER_STEP = 7  # batch, 2 frozen gradients, fused step, weight GEMM, ends, Adam


def train_surface(n=1 << 18, seed=1):
    from mplicits_gb300.synthetic import surface_points
    pts, nrm = surface_points(n, np.random.default_rng(seed), noise=0.002)
    return np.concatenate([pts, nrm], 1).astype(np.float32)


def train_bench(levels_np, device, K, W, precision="bf16"):
    """The fine-level training step: batch construction on the device, the
    frozen coarse and medium levels' f and df/dx, the trainable level's
    forward, loss, hand-written backward and Adam (FP32 master weights)."""
    import torch
    from mplicits_gb300.train import ResidualTrainer, create_training_data_on_neighborhood
    V = torch.from_numpy(train_surface()).to(device)
    models = make_models(levels_np, precision, device)
    tr = ResidualTrainer(models[2], models[:2], lr=1e-4, precision=precision)
    it = [0]

    def step():
        it[0] += 1
        b = create_training_data_on_neighborhood(V, TRAIN_SURFACE, device=device, delta=0.01,
                                                 seed=it[0])["on_surf"]
        return tr.step(*b)

    for _ in range(W):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(K):
        losses = step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / K
    rows = 3 * TRAIN_SURFACE
    return {"workload": f"fine-level residual training step: {TRAIN_SURFACE} surface samples "
                        f"-> {rows} rows (surface, normal offset, delta1-dithered), level "
                        "3->256x3->1 trainable, coarse and medium frozen, losses of "
                        "loss_add_detail_fine, Adam lr 1e-4, FP32 master weights",
            "value": rows / (ms * 1e-3), "unit": "rows/s", "ms_per_step": ms, "steps": K,
            "warmup": W, "dtype": "bf16" if precision == "bf16" else "f32",
            "flop_per_row": TRAIN_FLOP_PER_ROW,
            "achieved_tflops": TRAIN_FLOP_PER_ROW * rows / (ms * 1e-3) / 1e12,
            "last_losses": [float(x) for x in losses.cpu()],
            "gpu_launches": K * (TRAIN_LAUNCHES_PER_STEP if precision == "bf16" else 10)}


def train_cpu_baseline(levels_np, rows=3072, steps=3):
    """The reference's training step as it runs on the CPU (torch autograd,
    all host threads) on a bounded batch of the same kind of rows."""
    import torch
    from oracle.torch_ref import PlainSiren, train_step
    from oracle import train as otrain
    torch.set_num_threads(os.cpu_count() or 1)
    om = [30.0, 30.0, 30.0]
    fine = PlainSiren(levels_np[2][1], om)
    frozen = [PlainSiren(levels_np[i][1], om) for i in range(2)]
    for m in frozen:
        m.requires_grad_(False)
    opt = torch.optim.Adam(fine.parameters(), lr=1e-4)
    verts = train_surface()
    rng = np.random.default_rng(3)
    n = rows // 3
    idx = rng.choice(verts.shape[0], n, replace=False)
    u = rng.random((n, 3)).astype(np.float32)
    p, nr, s = [torch.from_numpy(a) for a in otrain.training_batch(verts, idx, u, 0.01)]
    train_step(fine, frozen, opt, p, nr, s)
    t0 = time.perf_counter()
    for _ in range(steps):
        train_step(fine, frozen, opt, p, nr, s)
    dt = (time.perf_counter() - t0) / steps
    return {"value": rows / dt, "unit": "rows/s", "cores": torch.get_num_threads(),
            "kind": "port", "sample": f"{steps} steps of {rows} rows with torch autograd on "
                                      "the CPU (the reference's step restated)"}


DELTAS_MESH = (512, 1024)  # theta x phi rings of the triangulated synthetic surface
DELTAS_MAX, DELTAS_ITERS = 0.05, 100


def deltas_mesh():
    from mplicits_gb300.synthetic import surface_mesh
    pos, nrm, faces = surface_mesh(*DELTAS_MESH)
    return np.concatenate([pos, nrm], 1).astype(np.float32), pos, faces


def deltas_bench(device, K, W):
    """calc_deltas over the vertices of a 1,048,576-triangle mesh of the
    synthetic surface (max_delta 0.05, 100 iterations, eps 2e-4): device
    resident, and end to end from pinned host rows to host output rows.  The
    scene (grid) is built once, as the reference builds its raycasting scene
    once; its build time is reported beside."""
    import torch
    from mplicits_gb300.scene import RaycastingScene, calc_deltas
    V, pos, faces = deltas_mesh()
    M = V.shape[0]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pos_d, faces_d = torch.from_numpy(pos).to(device), torch.from_numpy(faces).to(device)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    scene = RaycastingScene(pos_d, faces_d, device=device)
    build_ms = (time.perf_counter() - t0) * 1e3
    Vd = torch.from_numpy(V).to(device)
    out, iters = calc_deltas(Vd, scene, DELTAS_MAX, DELTAS_ITERS, return_iterations=True)
    for _ in range(W - 1):
        calc_deltas(Vd, scene, DELTAS_MAX, DELTAS_ITERS)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(K):
        calc_deltas(Vd, scene, DELTAS_MAX, DELTAS_ITERS)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / K
    # end to end: pinned host rows in, host rows out, every step
    host_in = torch.from_numpy(V).pin_memory()
    host_out = torch.empty(M, 7, dtype=torch.float32).pin_memory()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(K):
        d_in = host_in.to(device, non_blocking=True)
        host_out.copy_(calc_deltas(d_in, scene, DELTAS_MAX, DELTAS_ITERS), non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / K
    info = scene.info()
    d = out[:, 6]
    return {"workload": f"calc_deltas of {M} vertices of a {faces.shape[0]}-triangle mesh of the "
                        f"synthetic surface, max_delta {DELTAS_MAX}, {DELTAS_ITERS} iterations, "
                        "eps 2e-4, uniform-grid scene",
            "value": M / (ms * 1e-3), "unit": "vertices/s", "ms_per_call": ms,
            "iterations_run": iters, "ms_per_iteration": ms / max(1, iters),
            "steps": K, "warmup": W, "dtype": "f32",
            "scene_build_ms": build_ms, "scene": info,
            "delta_percentiles": [float(x) for x in
                                  torch.quantile(d[:1 << 20], torch.tensor(
                                      [0.0, 0.1, 0.5, 0.9, 1.0], device=device)).cpu()],
            "e2e": {"value": M / (e2e_ms * 1e-3), "unit": "vertices/s", "ms_per_call": e2e_ms,
                    "h2d_bytes_per_step": V.nbytes, "d2h_bytes_per_step": M * 7 * 4},
            "gpu_launches": K * (DELTAS_ITERS + 2)}


def deltas_cpu_baseline(iters, n=16384):
    """The oracle's grid search (C, all host threads; each step decided with
    early exits and bounding-sphere skips, as the GPU kernel does) on a
    seeded subset of the same vertices run for the GPU run's iteration
    count."""
    from oracle import deltas as od
    V, pos, faces = deltas_mesh()
    idx = np.random.default_rng(2).choice(V.shape[0], n, replace=False)
    od.calc_deltas(V[idx[:64]], pos, faces, DELTAS_MAX, DELTAS_ITERS, cell=0.02,
                   force_iters=1, fast=True)  # compile and warm
    t0 = time.perf_counter()
    od.calc_deltas(V[idx], pos, faces, DELTAS_MAX, DELTAS_ITERS, cell=0.02, force_iters=iters,
                   fast=True)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "vertices/s", "cores": os.cpu_count() or 1, "kind": "port",
            "sample": f"{n} of the {V.shape[0]} vertices, {iters} iterations, grid cell 0.02, "
                      "close/touch decision with bounding-sphere skips, grid build included "
                      "(C, OpenMP over vertices)"}


# first step of the persistent marching launch (tensor-core precisions): from
# here on few enough rays are left for one tile per SM; a sweep over 8..40 on
# the 1920x1080 orbit frames put the fastest frames at 32
TRACE_TAIL_FROM = 32


def trace_bench(levels_np, device, K, W, precision="bf16", tail_from=TRACE_TAIL_FROM):
    """Sphere tracing of 1920x1080 frames from 8 orbit viewpoints; with
    ``tail_from`` the steps from that one on run in one persistent launch."""
    import torch
    from mplicits_gb300.trace import SphereTracer, orbit_cameras
    cams = orbit_cameras()
    models = make_models(levels_np, precision, device)
    tr = SphereTracer(models, DELTAS, 1920, 1080, max_steps=96, eps=1e-4, precision=precision,
                      tail_from=tail_from)
    for k in range(max(W, 1)):
        tr.render(cams[k % len(cams)])
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    hits = []
    e0.record()
    for k in range(K):
        _, state = tr.render(cams[k % len(cams)])
        hits.append(tr.counts[2:3].clone())
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / K
    P = 1920 * 1080
    return {"value": P / (ms * 1e-3), "unit": "rays/s", "ms_per_frame": ms, "frames": K,
            "hits_per_frame": [int(h) for h in torch.cat(hits).cpu()],
            "launches_per_frame": tr.launches_per_frame, "dtype": precision}, tr


def trace_cpu_baseline(levels_np, W=192, H=108):
    from oracle import trace as otrace
    from mplicits_gb300.trace import orbit_cameras
    cam = dict(orbit_cameras()[0])
    cam["width"], cam["height"] = W, H
    params = [(p, [30.0, 30.0, 30.0]) for _, p in levels_np]
    t0 = time.perf_counter()
    otrace.trace(params, DELTAS, cam, max_steps=96, eps=1e-4)
    dt = time.perf_counter() - t0
    return {"value": W * H / dt, "unit": "rays/s", "cores": os.cpu_count() or 1, "kind": "port",
            "sample": f"one {W}x{H} frame of the first orbit camera, float64 numpy oracle"}


def level_flop(width, hidden=3):
    return 2 * (3 * width + (hidden - 1) * width * width + width)


def batch_workload(device, n_models=64, lo=1e4, hi=2e6, seed=11):
    """64 independent three-level models, widths 128 or 256 drawn uniformly,
    3 hidden layers, each level from its own seed (the reference's init);
    per model three nested point lists with sizes log-uniform in [lo, hi]
    (sorted: level 0 on the largest, levels 1 and 2 on index sublists)."""
    import torch
    from mplicits_gb300.batch import BatchEntry
    from mplicits_gb300.model import SIREN
    rng = np.random.default_rng(seed)
    entries = []
    for mi in range(n_models):
        width = int(rng.choice([128, 256]))
        sizes = sorted(np.exp(rng.uniform(np.log(lo), np.log(hi), 3)).astype(np.int64),
                       reverse=True)
        n0 = int(sizes[0])
        g = torch.Generator(device).manual_seed(seed * 1000 + mi)
        x = torch.rand(n0, 3, device=device, generator=g) * 2 - 1
        perm = torch.randperm(n0, device=device, generator=g).to(torch.int32)
        for lv in range(3):
            torch.manual_seed(seed * 100000 + mi * 3 + lv)
            m = SIREN(3, 1, [width] * 3, w0=30, precision="bf16").to(device).eval()
            n = int(sizes[lv])
            S = torch.empty(n0, device=device)
            idx = None if lv == 0 else perm[:n].contiguous()
            entries.append(BatchEntry(m, S, x=x, index=idx, n=n))
    return entries


def batch_bench(device, K, W):
    """One persistent graph-captured launch over all 192 levels against
    per-level launches of the single-level kernels (BF16, and plain FP32)."""
    import ctypes
    import torch
    from mplicits_gb300 import capi
    from mplicits_gb300.batch import BatchedLevels
    entries = batch_workload(device)
    pts = sum(e.n for e in entries)
    flop = sum(e.n * level_flop(e.model.linears()[0].out_features) for e in entries)
    bl = BatchedLevels(entries, "bf16")
    t0 = time.perf_counter()
    cfg, tuned_ms = bl.autotune(repeats=3, cache=False)
    tune_s = time.perf_counter() - t0
    bl.capture()
    lib = capi.load()

    def per_level(precision):
        st = capi.stream_ptr()
        for e in entries:
            net, packed = e.model.packed()
            p = capi.MplPoints(kind=capi.MPL_POINTS_XYZ, xyz=e.x.data_ptr())
            capi.check(lib.mpl_level_forward(
                ctypes.byref(net), capi.ptr(packed), ctypes.byref(p), capi.ptr(e.index), None,
                e.n, capi.ptr(e.S), capi.MPL_STORE, None, capi.PRECISIONS[precision], st),
                "mpl_level_forward")

    def timed(fn, k, w):
        for _ in range(w):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(k):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / k

    ms_batch = timed(bl.replay, K, W)
    old = capi.get_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT)
    capi.set_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT, cfg.epilogue_unit)
    try:
        ms_bf16 = timed(lambda: per_level("bf16"), K, W)
    finally:
        capi.set_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT, old)
    ms_fp32 = timed(lambda: per_level("fp32"), 1, 1)
    peak_tf, _, src = peaks()
    widths = [e.model.linears()[0].out_features for e in entries[::3]]
    return {"workload": "64 three-level models (192 levels), widths 128/256 uniform, 3 hidden "
                        "layers, distinct seeds, nested point lists log-uniform in [1e4, 2e6]",
            "points_per_step": pts, "flop_per_step": flop,
            "models_width_256": int(sum(w == 256 for w in widths)),
            "value": pts / (ms_batch * 1e-3), "unit": "pts/s", "ms_per_step": ms_batch,
            "achieved_tflops": flop / (ms_batch * 1e-3) / 1e12,
            "frac_of_peak": flop / (ms_batch * 1e-3) / 1e12 / peak_tf,
            "peak_source": f"{src} bf16 burst",
            "autotuned": {"tiles_in_flight": cfg.tiles_in_flight,
                          "epilogue_unit": cfg.epilogue_unit, "stages": cfg.stages,
                          "ctas": cfg.ctas, "best_ms": tuned_ms, "tuning_s": round(tune_s, 3)},
            "per_level_bf16_ms": ms_bf16, "per_level_fp32_ms": ms_fp32,
            "speedup_vs_fp32_per_model": ms_fp32 / ms_batch,
            "speedup_vs_bf16_per_level": ms_bf16 / ms_batch,
            # two tiles in flight: a tile-prefix kernel and the batched kernel
            # per width group present; one tile: one launch
            "gpu_launches_per_step": (2 * sum(1 for c in bl.plan.width_count if c > 0)
                                      if cfg.tiles_in_flight == 2 else 1)}


def run_reference(args):
    """The reference arm: the reference's reconstruction loop on the host
    cores (the oracle restatement of its torch code, which cannot travel),
    W untimed and K timed samples of the same size as the GPU line's
    cpu_baseline samples; rank 0 alone works and prints."""
    rank, world, _ = rank_info()
    if rank != 0:
        return
    K, W = max(1, args.steps), max(0, args.warmup)
    vals, detail, wall = cpu_reference_samples(args.N, K + W)
    timed = vals[W:]
    value = float(np.mean(timed))
    threads = detail["threads"]
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "pts/s",
            "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": wall * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config_of(args.N, world),
            "cpu_baseline": {"value": value, "unit": "pts/s", "cores": threads, "kind": "port",
                             "sample": f"mean of {len(timed)} samples: " + detail["sample"]},
            "e2e": {"value": value, "unit": "pts/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import __graft_entry__
    __graft_entry__.build()
    N, K, W = args.N, args.steps, max(3, args.warmup)
    levels_np = load_levels_np()
    if args.only:
        if args.only == "train":
            out = train_bench(levels_np, device, K, W, "bf16")
        elif args.only == "trace":
            out, _ = trace_bench(levels_np, device, K, W, "bf16")
        elif args.only == "deltas":
            out = deltas_bench(device, K, W)
            if rank == 0 and not args.skip_cpu:
                out["cpu_baseline"] = deltas_cpu_baseline(out["iterations_run"])
        else:
            out = batch_bench(device, K, W)
        if rank == 0:
            print(json.dumps({"only": args.only, **out}), flush=True)
        return
    from mplicits_gb300 import capi
    if args.bf16_unit:
        capi.set_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT, args.bf16_unit)

    # ---- the headline: the fused 16-bit tensor-core evaluator (FP16 operands)
    hp = args.headline
    head = Step(make_models(levels_np, hp, device), N, device, hp)
    from mplicits_gb300.replicas import barrier, max_over_ranks, replica_value
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms, l0_ms = time_steps(head, K, W)
    ms = max_over_ranks(ms, device)
    value = replica_value(N ** 3, ms * 1e-3, world)
    bands = head.rec.band_sizes()
    if args.profile_only:
        if rank == 0:
            print(json.dumps({"profile_only": True, "ms_per_step": ms, "level0_ms": l0_ms,
                              "value": value, "grid": N, "band_points": bands}), flush=True)
        return

    # ---- the other arithmetic: the other 16-bit operand type, FP32
    # refinement margins, plain FP32
    other = "bf16" if hp == "fp16" else "fp16"
    variants = {hp: {"ms_per_step": ms, "level0_ms": l0_ms, "value": value}}
    steps = {hp: head}
    for name, prec, margin in ((other, other, None), ("bf16_refined", "bf16", REFINE["bf16"]),
                               ("fp16_refined", "fp16", REFINE["fp16"])):
        st = Step(make_models(levels_np, prec, device), N, device, prec, margin)
        vms, vl0 = time_steps(st, K, W)
        variants[name] = {"ms_per_step": vms, "level0_ms": vl0, "value": N ** 3 / (vms * 1e-3),
                          "refine_margin": margin}
        steps[name] = st
    fp32 = Step(make_models(levels_np, "fp32", device), N, device, "fp32")
    ms32, l0_32 = time_steps(fp32, max(1, args.fp32_steps), 1)
    steps["fp32"] = fp32

    errors = None
    if not args.skip_errors and rank == 0:
        errors = {k: error_stats(v, v.rec.levels, N) for k, v in steps.items()}
        ref_faces = fp32.faces[:fp32.F]
        for k, v in steps.items():
            errors[k]["mesh_topology_equals_fp32"] = bool(
                v.F == fp32.F and torch.equal(v.faces[:v.F], ref_faces))
        errors["mc_ambiguity_fp32"] = mc_ambiguity(fp32.rec.S, N)
        for k in ("bf16_refined", "fp16_refined"):
            a, b = fp32.rec, steps[k].rec
            errors[k]["band_lists_equal_fp32"] = all(
                torch.equal(torch.sort(a.band_index[i][:a.band_sizes()[i]])[0],
                            torch.sort(b.band_index[i][:b.band_sizes()[i]])[0]) for i in range(2))

    # ---- end to end through the public API with host buffers
    e2e_s, h2d, d2h, e2e_launch = e2e_run(levels_np, N, device, max(1, K // 2), 1, hp)

    # ---- the training step and the sphere tracer
    training = tracing = None
    if not args.skip_train:
        training = train_bench(levels_np, device, K, W, "bf16")
        training["fp32"] = train_bench(levels_np, device, K, W, "fp32")
        training["speedup_bf16_vs_fp32"] = training["fp32"]["ms_per_step"] / training["ms_per_step"]
        if rank == 0 and not args.skip_cpu:
            training["cpu_baseline"] = train_cpu_baseline(levels_np)
    if not args.skip_trace:
        tracing = {}
        for prec in ("bf16", "fp32"):
            tracing[prec], tr = trace_bench(levels_np, device, K if prec == "bf16" else 1, 1,
                                            prec)
            del tr
        tracing["workload"] = ("1920x1080 pinhole rays, 45 deg, 8 orbit viewpoints at radius "
                               "2.5, <= 96 steps, eps 1e-4, band-gated levels, gradient normals "
                               "and shading of the hits")
        if rank == 0 and not args.skip_cpu:
            tracing["cpu_baseline"] = trace_cpu_baseline(levels_np)

    batched = None
    if not args.skip_batch:
        batched = batch_bench(device, K, W)

    neigh = None
    if not args.skip_deltas:
        neigh = deltas_bench(device, K, W)
        if rank == 0 and not args.skip_cpu:
            neigh["cpu_baseline"] = deltas_cpu_baseline(neigh["iterations_run"])

    # ---- roofline of the dominant kernel (level 0 over the full grid)
    peak_tf, hbm, src = peaks()
    achieved_tf = FLOP_PER_POINT * N ** 3 / (l0_ms * 1e-3) / 1e12
    traffic = None
    kernel_name = "level 0 tensor-core launch"
    prof = os.path.join(ROOT, "profiles", "level_l0w_f16_512_traffic.json")
    if os.path.exists(prof):
        with open(prof) as f:
            pj = json.load(f)
        traffic = pj.get("dram_bytes_per_launch")
        kernel_name = pj.get("kernel", kernel_name)

    cpu = None
    if rank == 0 and not args.skip_cpu:
        vals, detail, _ = cpu_reference_samples(N, args.cpu_repeats)
        cpu = {"value": float(np.mean(vals)), "unit": "pts/s", "cores": detail["threads"],
               "kind": "port", "sample": f"mean of {len(vals)} samples: " + detail["sample"],
               "samples": vals, "detail": detail}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "pts/s", "n_gpus": world, "steps": K,
            "warmup": W, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f16" if hp == "fp16" else "bf16",
            "data": "synthetic",
            "config": config_of(N, world),
            "workload_stats": {"band_points": bands, "mesh": {"verts": head.V, "faces": head.F}},
            "banded_mc_ms": {f"{hp}_fused": ms, "fp32_plain": ms32,
                             f"{other}_fused": variants[other]["ms_per_step"]},
            "variants": variants,
            "fp32_plain": {"value": N ** 3 / (ms32 * 1e-3), "unit": "pts/s", "ms_per_step": ms32,
                           "level0_ms": l0_32},
            "speedup_vs_fp32": ms32 / ms,
            "speedup_bf16_vs_fp32": ms32 / variants["bf16"]["ms_per_step"],
            "speedup_fp16_vs_fp32": ms32 / variants["fp16"]["ms_per_step"],
            "errors_vs_fp64": errors,
            "e2e": {"value": N ** 3 / e2e_s, "unit": "pts/s", "ms_per_step": e2e_s * 1e3,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "path": "mplicits_gb300.meshing.BandedReconstruction.sample()+mesh() with "
                            "weights copied from pinned host memory and the mesh copied back"},
            "roofline": {"bound": "tensor", "kernel": kernel_name + " (level 0, full grid)",
                         "achieved": achieved_tf, "peak": peak_tf, "unit": "TFLOP/s",
                         "frac": achieved_tf / peak_tf,
                         "peak_source": f"{src} bf16 burst (the launch runs at full clock; FP16 and BF16 "
                                        "share the dense tensor rate)",
                         "flop_per_point": FLOP_PER_POINT, "points_per_launch": N ** 3,
                         "launch_ms": l0_ms, "traffic": traffic},
            "cpu_baseline": cpu,
            "training": training,
            "sphere_tracing": tracing,
            "batched_models": batched,
            "neighbourhood_deltas": neigh,
            "gpu_launches": K * KERNEL_LAUNCHES_PER_STEP,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
