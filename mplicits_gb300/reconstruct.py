#!/usr/bin/env python
"""Drop-in for the reference's reconstruct.py (reconstruct.py:37-133).

Same positional arguments and flags, same printed lines and the same
``SAMPLING_TIME_S:<seconds>`` line that reproduce.py parses; the band-culled
evaluation and marching cubes run on the GPU through libmplicits.  New flag:
``--precision {fp32,bf16,fp16}`` (fp32, the plain form, is the default).
``--input`` reads the training point cloud from a PLY file (ASCII or binary
vertex x/y/z), which the reference reads with open3d.
"""

from __future__ import annotations

import argparse
import ctypes
import os
import os.path as osp

import numpy as np
import torch

from . import capi
from .meshing import create_mesh_multistage
from .model import from_pth


def read_ply_points(path):
    """x, y, z of the vertex element of a PLY file (ascii or binary)."""
    with open(path, "rb") as f:
        header = []
        while True:
            line = f.readline()
            if not line:
                raise ValueError(f"{path}: truncated PLY header")
            header.append(line.decode("ascii", "replace").strip())
            if header[-1] == "end_header":
                break
        fmt = next(h.split()[1] for h in header if h.startswith("format"))
        nv, props, in_vertex = 0, [], False
        for h in header:
            tok = h.split()
            if tok[:1] == ["element"]:
                in_vertex = tok[1] == "vertex"
                if in_vertex:
                    nv = int(tok[2])
            elif tok[:1] == ["property"] and in_vertex:
                if tok[1] == "list":
                    raise ValueError("list properties on vertices are not supported")
                props.append((tok[2], tok[1]))
        types = {"float": "f4", "float32": "f4", "double": "f8", "float64": "f8",
                 "uchar": "u1", "uint8": "u1", "char": "i1", "int8": "i1", "short": "i2",
                 "int16": "i2", "ushort": "u2", "uint16": "u2", "int": "i4", "int32": "i4",
                 "uint": "u4", "uint32": "u4"}
        if fmt == "ascii":
            rows = [f.readline().split() for _ in range(nv)]
            names = [p[0] for p in props]
            arr = np.array(rows, dtype=np.float64)
            return np.stack([arr[:, names.index(c)] for c in "xyz"], 1).astype(np.float32)
        endian = "<" if fmt == "binary_little_endian" else ">"
        dt = np.dtype([(n, endian + types[t]) for n, t in props])
        data = np.frombuffer(f.read(nv * dt.itemsize), dtype=dt, count=nv)
        return np.stack([data["x"], data["y"], data["z"]], 1).astype(np.float32)


def adaptive_deltas(models, input_ply, device, eps=0.3, batch=2 ** 18):
    """reconstruct.py:18-33: delta_i = (1 + eps) * max_j |sum_{k<i} f_k(x_j)|.

    ``input_ply`` is a PLY path or an [M, 3] point array.  The partial sums
    are accumulated on the device by the level kernel (f0 stored, then each
    f_k added, the float32 order of the reference's ``sum``), and each chunk's
    ``max |S|`` is reduced on the device into its own slot (mpl_abs_max), so
    the whole computation reads the host once.  The slots are then combined
    as the reference's ``worst = max(worst, float(...))`` does, chunk by
    chunk in order (a chunk whose maximum is NaN leaves ``worst`` unchanged).
    """
    from .model import level_forward
    src = read_ply_points(input_ply) if isinstance(input_ply, (str, os.PathLike)) else input_ply
    pts = torch.as_tensor(np.asarray(src, np.float32)).to(device).contiguous()
    M = pts.shape[0]
    heads = list(range(0, M, batch))
    lib = capi.load()
    maxima = torch.zeros(max(len(models) - 1, 1), max(len(heads), 1), dtype=torch.float32,
                         device=device)
    S = torch.empty(min(batch, max(M, 1)), dtype=torch.float32, device=device)
    with torch.no_grad():
        for level in range(1, len(models)):
            for c, i in enumerate(heads):
                chunk = pts[i:i + batch]
                s = S[:chunk.shape[0]]
                level_forward(models[0], chunk, S=s)
                for k in range(1, level):
                    level_forward(models[k], chunk, S=s, accumulate=True)
                capi.check(lib.mpl_abs_max(capi.ptr(s), s.shape[0], capi.ptr(maxima[level - 1, c:]),
                                           capi.stream_ptr()), "mpl_abs_max")
    host = maxima.cpu().tolist()
    deltas = []
    for level in range(1, len(models)):
        worst = 0.0
        for m in host[level - 1][:len(heads)]:
            worst = max(worst, m)
        deltas.append((1.0 + eps) * worst)
    return deltas


def main(argv=None):
    parser = argparse.ArgumentParser(description="Run marching cubes using a trained model.")
    parser.add_argument("model_path", help="Path to the PyTorch weights file")
    parser.add_argument("--coarse_path", default=None,
                        help="Path to the PyTorch weights file for the coarse network")
    parser.add_argument("--medium_path", default=None,
                        help="Path to the medium resolution model. Only use this when "
                             "reconstructing a fine-level model.")
    parser.add_argument("output_path", help="Path to the output mesh file")
    parser.add_argument("--w0", type=int, default=1, help="Value for \\omega_0. Default is 1.")
    parser.add_argument("--resolution", "-r", default=128, type=int,
                        help="Resolution to use on marching cubes. Default is 128.")
    parser.add_argument("--device", default="cpu",
                        help="Device to run the inference. By default is \"cpu\".")
    parser.add_argument("--multistage", action="store_true",
                        help="Use the multiscale optimization (finer levels only evaluated "
                             "near the surface).")
    parser.add_argument("--input", default=None,
                        help="Training point cloud (.ply) for the adaptive band widths.")
    parser.add_argument("--deltas", type=float, nargs="+", default=None,
                        help="Explicit band widths (one per residual level).")
    parser.add_argument("--precision", choices=["fp32", "bf16", "fp16"], default="fp32",
                        help="Arithmetic of the hidden layers: fp32 (plain form), or bf16 / "
                             "fp16 operands on the tcgen05 tensor cores.")
    args = parser.parse_args(argv)
    out_dir = osp.split(args.output_path)[0]
    if out_dir and not osp.exists(out_dir):
        os.makedirs(out_dir)

    device = args.device
    if "cuda" not in device:
        # the GB300 path has no CPU fallback: evaluate on the current GPU
        print(f"[WARNING] mplicits_gb300 runs on the GPU; using \"cuda\" instead of \"{device}\".")
        device = "cuda"
    if not torch.cuda.is_available():
        raise RuntimeError("mplicits_gb300 needs a CUDA device")
    capi.load()
    device = torch.device(device)
    model = from_pth(args.model_path, w0=args.w0, precision=args.precision).eval().to(device)
    print(model)
    model_list = [model]
    print(f"Running marching cubes running with resolution {args.resolution}")
    if args.medium_path is not None:
        print("Using residual approach for fine level")
        model_medium = from_pth(args.medium_path, w0=1, precision=args.precision).eval().to(device)
        model_list.append(model_medium)
        print("========== Medium model ==========")
        print(model_medium)
    if args.coarse_path is not None:
        print("Using the residual approach")
        model_coarse = from_pth(args.coarse_path, w0=1, precision=args.precision).eval().to(device)
        model_list.append(model_coarse)
        print("========== Coarse model ==========")
        print(model_coarse)

    if args.multistage:
        if args.deltas is not None:
            deltas = list(args.deltas)
        elif args.input is not None:
            deltas = adaptive_deltas(model_list[::-1], args.input, device)
            print("adaptive band widths (Eq. 5):", ", ".join(f"{d:.3e}" for d in deltas))
        else:
            deltas = [0.1, 0.06][:len(model_list) - 1]
            print("[WARNING] --multistage without --input: using fixed band widths"
                  f" {deltas}; pass the training point cloud for the paper's adaptive bands.")
    else:
        deltas = []

    _, _, _, _, sampling_time = create_mesh_multistage(
        model_list[::-1], deltas=deltas, filename=args.output_path, N=args.resolution,
        max_batch=32 ** 3, device=device)
    print(f"SAMPLING_TIME_S:{sampling_time}")
    print("Done")


if __name__ == "__main__":
    main()
