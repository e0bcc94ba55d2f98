"""Drop-in SIREN whose forward runs the fused GB300 level kernels.

Mirrors ``i3d.model`` (i3d/model.py:10-180, 322-424) and ``i3d.util.from_pth``
(i3d/util.py:79-142): the same constructor, module tree and state_dict keys
(``net.{i}.0.weight|bias``), the same initialisation (so a seed gives the same
weights), the same ``forward(x, preserve_grad=False) -> {"model_in",
"model_out"}`` and the same omega baking.  ``forward`` evaluates the whole
level in one ``mpl_level_forward`` launch on the current CUDA stream; CPU
tensors raise (there is no CPU fallback).
"""

from __future__ import annotations

import ctypes
import math
import os.path as osp
from collections import OrderedDict

import torch
from torch import nn

from . import capi


@torch.no_grad()
def sine_init(m, w0):
    """Hidden/output layers: U(-sqrt(6/n_in)/w0, +sqrt(6/n_in)/w0) (i3d/model.py:10-15)."""
    if hasattr(m, "weight"):
        n_in = m.weight.size(-1)
        bound = math.sqrt(6 / n_in) / w0
        m.weight.uniform_(-bound, bound)


@torch.no_grad()
def first_layer_sine_init(m):
    """First layer: U(-1/n_in, 1/n_in) (i3d/model.py:18-22)."""
    if hasattr(m, "weight"):
        n_in = m.weight.size(-1)
        m.weight.uniform_(-1 / n_in, 1 / n_in)


class SineLayer(nn.Module):
    """``sin(w0 * x)`` (i3d/model.py:25-36); kept for the module tree."""

    def __init__(self, w0=30):
        super().__init__()
        self.w0 = w0

    def forward(self, x):
        return torch.sin(self.w0 * x)

    def __repr__(self):
        return f"SineLayer(w0={self.w0})"


class PackedLevel:
    """Device image of one level's weights, repacked when a parameter changes."""

    def __init__(self):
        self.key = None
        self.buf = None
        self.net = None

    def get(self, model):
        params = [p for p in model.parameters()]
        key = tuple((p.data_ptr(), p._version) for p in params) + \
            (model.w0, model.ww, params[0].device)
        if key == self.key:
            return self.net, self.buf
        net = model.mpl_net()
        lib = capi.load()
        nbytes = ctypes.c_int64(0)
        capi.check(lib.mpl_net_packed_bytes(ctypes.byref(net), ctypes.byref(nbytes)),
                   "mpl_net_packed_bytes")
        dev = params[0].device
        buf = torch.empty(nbytes.value + 256, dtype=torch.uint8, device=dev)
        off = (-buf.data_ptr()) % 256
        view = buf[off:off + nbytes.value]
        ws = [l.weight.detach().contiguous().float() for l in model.linears()]
        bs = [l.bias.detach().contiguous().float() for l in model.linears()]
        wp = (ctypes.c_void_p * len(ws))(*[w.data_ptr() for w in ws])
        bp = (ctypes.c_void_p * len(bs))(*[b.data_ptr() for b in bs])
        capi.check(lib.mpl_net_pack(ctypes.byref(net), wp, bp, capi.ptr(view),
                                    capi.stream_ptr()), "mpl_net_pack")
        self._keep = (buf, ws, bs)
        self.key, self.buf, self.net = key, view, net
        return net, view


def _require_cuda(x):
    if not x.is_cuda:
        raise RuntimeError("mplicits_gb300 evaluates levels on a CUDA device only "
                           "(no CPU fallback); move the model and inputs to 'cuda'")


class _LevelForward(torch.autograd.Function):
    """model_out = f(x) through mpl_level_forward; backward via the
    input-gradient and weight-gradient kernels (see mplicits_gb300.grad)."""

    @staticmethod
    def forward(ctx, x, model, *params):
        out = level_forward(model, x.reshape(-1, x.shape[-1]))
        ctx.model = model
        ctx.save_for_backward(x, *params)
        return out.reshape(x.shape[:-1] + (1,))

    @staticmethod
    def backward(ctx, gy):
        from . import grad as _grad
        x, *params = ctx.saved_tensors
        return _grad.level_backward(ctx.model, x, gy, params, ctx.needs_input_grad)


def level_forward(model, x, S=None, accumulate=False, precision=None):
    """One launch of the fused level kernel on points ``x`` [P, 3]; returns
    (or accumulates into) ``S`` [P]."""
    _require_cuda(x)
    x = x.detach()
    if x.dtype != torch.float32:
        x = x.float()
    x = x.contiguous()
    P = x.shape[0]
    if S is None:
        S = torch.empty(P, dtype=torch.float32, device=x.device)
    net, packed = model.packed()
    pts = capi.MplPoints(kind=capi.MPL_POINTS_XYZ, xyz=x.data_ptr())
    prec = capi.PRECISIONS[precision or model.precision]
    capi.check(capi.load().mpl_level_forward(
        ctypes.byref(net), capi.ptr(packed), ctypes.byref(pts), None, None, P, capi.ptr(S),
        capi.MPL_ACCUMULATE if accumulate else capi.MPL_STORE, None, prec,
        capi.stream_ptr()), "mpl_level_forward")
    return S


class SIREN(nn.Module):
    """SIREN level with the signature of i3d.model.SIREN (i3d/model.py:76-105).

    Extra attribute ``precision`` ("fp32" plain form, default; or "bf16" for
    the tcgen05 hidden GEMMs) selects the kernel of ``forward``.
    """

    def __init__(self, n_in_features, n_out_features, hidden_layer_config=[], w0=30, ww=None,
                 delay_init=False, precision="fp32"):
        super().__init__()
        self.in_features = n_in_features
        self.out_features = n_out_features
        self.w0 = w0
        self.ww = w0 if ww is None else ww
        self.precision = precision
        widths = [n_in_features] + list(hidden_layer_config)
        blocks = [nn.Sequential(nn.Linear(widths[0], widths[1]), SineLayer(self.w0))]
        for i in range(1, len(hidden_layer_config)):
            blocks.append(nn.Sequential(nn.Linear(widths[i], widths[i + 1]), SineLayer(self.ww)))
        blocks.append(nn.Sequential(nn.Linear(widths[-1], n_out_features)))
        self.net = nn.Sequential(*blocks)
        self._packed = PackedLevel()
        if not delay_init:
            self.reset_weights()

    # -- topology --------------------------------------------------------
    def linears(self):
        return [blk[0] for blk in self.net]

    def omegas(self):
        out = []
        for blk in self.net[:-1]:
            out.append(float(blk[1].w0))
        return out

    def mpl_net(self):
        lins = self.linears()
        if self.out_features != 1 or self.in_features != 3:
            raise ValueError("the GB300 kernels evaluate 3 -> ... -> 1 SDF levels")
        if len(lins) > capi.MPL_MAX_LAYERS:
            raise ValueError(f"at most {capi.MPL_MAX_LAYERS} layers are supported")
        net = capi.MplNet()
        net.n_layers = len(lins)
        dims = [lins[0].in_features] + [l.out_features for l in lins]
        for i, d in enumerate(dims):
            net.dims[i] = d
        for i, w in enumerate(self.omegas()):
            net.omega[i] = w
        return net

    def packed(self):
        return self._packed.get(self)

    # -- reference API ---------------------------------------------------
    def forward(self, x, preserve_grad=False):
        """Same contract as i3d/model.py:107-129."""
        coords_org = x if preserve_grad else x.clone().detach().requires_grad_(True)
        params = tuple(self.parameters())
        if torch.is_grad_enabled() and (coords_org.requires_grad or
                                        any(p.requires_grad for p in params)):
            y = _LevelForward.apply(coords_org, self, *params)
        else:
            y = level_forward(self, coords_org.reshape(-1, coords_org.shape[-1]))
            y = y.reshape(coords_org.shape[:-1] + (1,))
        return {"model_in": coords_org, "model_out": y}

    def reset_weights(self):
        """i3d/model.py:131-141."""
        self.net[0].apply(first_layer_sine_init)
        self.net[1:].apply(lambda module: sine_init(module, self.ww))
        return self

    def update_omegas(self, w0=1, ww=None):
        """Bake omega into the weights (i3d/model.py:143-180): every tensor
        but the last two is scaled by old_w0 / w0."""
        if ww is None:
            ww = w0
        sd = self.state_dict()
        keys = list(sd.keys())
        for k in keys[:-2]:
            sd[k] = sd[k] * (self.w0 / w0)
        self.load_state_dict(sd)
        self.w0 = w0
        self.ww = ww
        self.net[0][1].w0 = w0
        for i in range(1, len(self.net) - 1):
            self.net[i][1].w0 = ww
        return self


def _siren_v1_to_v2(weights):
    out = OrderedDict()
    for k, v in weights.items():
        out[k[4:]] = v
    return out


def from_state_dict(weights, device="cpu", w0=1, ww=None, precision="fp32"):
    """Topology from the bias shapes, then load (i3d/model.py:322-380)."""
    keys = list(weights.keys())
    n_layers = len(weights) // 2
    bias_keys = [k for k in keys if "bias" in k]
    hidden = [weights[bias_keys[i]].shape[0] for i in range(n_layers - 1)]
    model = SIREN(weights[keys[0]].shape[1], weights[keys[-1]].shape[0], hidden, w0=w0, ww=ww,
                  delay_init=True, precision=precision)
    upgraded = False
    try:
        model.load_state_dict(weights)
    except RuntimeError:
        print("Found weights from old version of SIREN. Converting to v2.")
        model.load_state_dict(_siren_v1_to_v2(weights))
        upgraded = True
    return model, upgraded


def from_pth(path, device="cpu", w0=1, ww=None, precision="fp32"):
    """i3d/util.py:79-142 (and i3d/model.py:383-424)."""
    if not osp.exists(path):
        raise FileNotFoundError(f"Weights file not found at \"{path}\"")
    weights = torch.load(path, map_location=torch.device(device))
    model, upgraded = from_state_dict(weights, device=device, w0=w0, ww=ww, precision=precision)
    if upgraded:
        torch.save(model.state_dict(), path.split(".")[0] + "_v2.pth")
    return model.to(device=device)
