"""Analytic input gradients of a level (normals, eikonal term).

``level_gradient`` returns f(x) and df/dx in one launch of the fused
forward-mode kernel (``mpl_level_gradient``).  It is what
``torch.autograd.grad(model_out, model_in)`` on a ``mplicits_gb300.SIREN``
evaluates (the reference obtains it from autograd, i3d/diff_operators.py:
259-265), and what the sphere tracer and marching cubes use for normals.
"""

from __future__ import annotations

import ctypes

import torch

from . import capi


def level_gradient(model, x, S=None, G=None, accumulate=False, precision=None, index=None,
                   n_dev=None, n=None):
    """(S, G): f(x) [P] and df/dx [P, 3] of one level.  With ``index`` the
    points are x[index[q]] and the results land at S[index[q]], G[index[q]]."""
    if not x.is_cuda:
        raise RuntimeError("mplicits_gb300 evaluates levels on a CUDA device only")
    x = x.detach().float().contiguous()
    P = x.shape[0]
    n = P if n is None else n
    if S is None:
        S = torch.empty(P, dtype=torch.float32, device=x.device)
    if G is None:
        G = torch.empty(P, 3, dtype=torch.float32, device=x.device)
    net, packed = model.packed()
    pts = capi.MplPoints(kind=capi.MPL_POINTS_XYZ, xyz=x.data_ptr())
    prec = capi.PRECISIONS[precision or model.precision]
    capi.check(capi.load().mpl_level_gradient(
        ctypes.byref(net), capi.ptr(packed), ctypes.byref(pts), capi.ptr(index),
        capi.ptr(n_dev), n, capi.ptr(S), capi.ptr(G),
        capi.MPL_ACCUMULATE if accumulate else capi.MPL_STORE, None, prec, capi.stream_ptr()),
        "mpl_level_gradient")
    return S, G


def level_backward(model, x, gy, params, needs_input_grad):
    """Backward of model_out = f(x) for ``_LevelForward``.

    d(model_in) = gy * df/dx comes from the fused gradient kernel; under
    ``create_graph=True`` (i3d/diff_operators.py:259-265) it is the
    differentiable op of ``mplicits_gb300.train.level_input_grad``, whose own
    backward is the double backward of the eikonal and normal losses.
    Weight gradients come from the hand-written backward kernels
    (``mplicits_gb300.train.param_grads``) with seed gy.
    """
    from . import train as _train
    shape = x.shape
    x2 = x.detach().reshape(-1, shape[-1])
    g2 = gy.reshape(-1)
    dx = None
    if needs_input_grad[0]:
        if torch.is_grad_enabled():
            G = _train.level_input_grad(model, x.reshape(-1, shape[-1]))
            dx = (gy.reshape(-1, 1) * G).reshape(shape)
        else:
            _, G = level_gradient(model, x2, precision="fp32")
            dx = (g2.reshape(-1, 1).to(G.dtype) * G).reshape(shape)
    pgrads = (None,) * len(params)
    if any(needs_input_grad[2:]):
        pgrads = tuple(_train.param_grads(model, x2, df=g2.detach()))
    return (dx, None) + pgrads
