"""Training of a residual level with the hand-written backward kernels.

``ResidualTrainer.step`` is the step of the reference's fine-level trainer
(experiment_scripts/train_sdf_on_neighborhood_fine.py:220-262) with its loss
``loss_add_detail_fine`` (i3d/loss_functions.py:347-394) on the GPU kernels:
the frozen levels' f and df/dx come from the forward-mode gradient kernel, the
trainable level runs a plain FP32 forward that keeps its pre-activations, the
loss kernel produces per-point seeds dL/df and dL/d(df/dx), one backward pass
through the level's forward-mode graph gives every weight gradient (the
double backward included), and an Adam kernel updates the FP32 weights.

``param_grads`` exposes the same backward to autograd: ``SIREN.forward`` and
the input-gradient op use it, so ``torch.autograd.grad(..., create_graph=True)``
followed by ``loss.backward()`` (the reference trainers' own code) trains a
``mplicits_gb300.SIREN`` through these kernels.
"""

from __future__ import annotations

import ctypes

import torch

from . import capi
from .grad import level_gradient

DEFAULT_WEIGHTS = {"sdf_constraint": 3e3, "normal_constraint": 1e2, "grad_constraint": 5e1}
TRUE_SDF_WEIGHTS = {"sdf_on_surf": 3e3, "sdf_off_surf": 2e2, "normal_constraint": 1e2,
                    "grad_constraint": 5e1}
LOSSES = {"residual": (capi.MPL_LOSS_RESIDUAL, DEFAULT_WEIGHTS),
          "true_sdf": (capi.MPL_LOSS_TRUE_SDF, TRUE_SDF_WEIGHTS)}


class _Scratch:
    """Per-model buffers of the backward, grown on demand."""

    def __init__(self, model):
        self.model = model
        self.n = -1

    def ensure(self, n, device):
        if n <= self.n:
            return
        net = self.model.mpl_net()
        fl = ctypes.c_int64(0)
        capi.check(capi.load().mpl_train_scratch_floats(ctypes.byref(net), n, ctypes.byref(fl)),
                   "mpl_train_scratch_floats")
        self.pre = torch.empty(fl.value, dtype=torch.float32, device=device)
        self.da = torch.empty(fl.value, dtype=torch.float32, device=device)
        self.f = torch.empty(n, dtype=torch.float32, device=device)
        self.g = torch.empty(n, 3, dtype=torch.float32, device=device)
        self.seeds = torch.empty(n, 4, dtype=torch.float32, device=device)
        self.n = n
        # padded gradient buffers, one per nn.Linear weight and bias
        wp = _padded_width(self.model)
        L = len(self.model.linears())
        self.dW, self.db = [], []
        for l in range(L):
            rows = wp if l < L - 1 else 1
            cols = 3 if l == 0 else wp
            if l == L - 1:
                self.dW.append(torch.zeros(wp, dtype=torch.float32, device=device))
                self.db.append(torch.zeros(1, dtype=torch.float32, device=device))
            else:
                self.dW.append(torch.zeros(rows, cols, dtype=torch.float32, device=device))
                self.db.append(torch.zeros(wp, dtype=torch.float32, device=device))


def _padded_width(model):
    w = max(l.out_features for l in model.linears()[:-1])
    return 64 if w <= 64 else (128 if w <= 128 else 256)


def _scratch(model, n, device):
    sc = getattr(model, "_train_scratch", None)
    if sc is None:
        sc = _Scratch(model)
        model._train_scratch = sc
    sc.ensure(n, device)
    return sc


def _forward_with_scratch(model, x, sc):
    net, packed = model.packed()
    n = x.shape[0]
    capi.check(capi.load().mpl_train_forward(
        ctypes.byref(net), capi.ptr(packed), capi.ptr(x), n, capi.ptr(sc.f), capi.ptr(sc.g),
        capi.ptr(sc.pre), capi.stream_ptr()), "mpl_train_forward")


def _backward(model, x, sc):
    """Weight gradients into the padded buffers (zeroed first)."""
    net, packed = model.packed()
    for t in sc.dW + sc.db:
        t.zero_()
    n = x.shape[0]
    dW = (ctypes.c_void_p * len(sc.dW))(*[t.data_ptr() for t in sc.dW])
    db = (ctypes.c_void_p * len(sc.db))(*[t.data_ptr() for t in sc.db])
    capi.check(capi.load().mpl_train_backward(
        ctypes.byref(net), capi.ptr(packed), capi.ptr(x), n, capi.ptr(sc.pre),
        capi.ptr(sc.seeds[:n]), capi.ptr(sc.da), dW, db, capi.stream_ptr()), "mpl_train_backward")


def _unpad(model, sc):
    """Gradients in the shapes of the nn.Linear parameters (weight, bias, ...)."""
    out = []
    L = len(model.linears())
    for l, lin in enumerate(model.linears()):
        if l == L - 1:
            out.append(sc.dW[l][:lin.in_features].reshape(1, -1).clone())
            out.append(sc.db[l][:1].clone())
        else:
            out.append(sc.dW[l][:lin.out_features, :lin.in_features].clone())
            out.append(sc.db[l][:lin.out_features].clone())
    return out


def param_grads(model, x, df=None, dg=None, want_dx=False):
    """d/dtheta of sum_p df_p f(x_p) + dg_p . (df/dx)(x_p) for one level: the
    weight gradients of any loss with seeds df [n] and dg [n, 3].  With
    ``want_dx`` also d/dx of the same sum, [n, 3] (W0^T times the layer-0
    value-row adjoint, which holds the Hessian term of the dg seeds)."""
    x = x.detach().float().contiguous()
    n = x.shape[0]
    sc = _scratch(model, n, x.device)
    _forward_with_scratch(model, x, sc)
    seeds = sc.seeds[:n]
    seeds.zero_()
    if df is not None:
        seeds[:, 0] = df.reshape(-1).float()
    if dg is not None:
        seeds[:, 1:] = dg.reshape(-1, 3).float()
    _backward(model, x, sc)
    grads = _unpad(model, sc)
    if not want_dx:
        return grads
    lin0 = model.linears()[0]
    wp = _padded_width(model)
    da0 = sc.da[:n * 4 * wp].view(n, 4, wp)[:, 0, :lin0.out_features]
    return grads, da0 @ lin0.weight.detach().float()


class _LevelInputGrad(torch.autograd.Function):
    """df/dx of a level, differentiable w.r.t. the level's parameters (the
    double backward of the eikonal and normal losses)."""

    @staticmethod
    def forward(ctx, x, model, *params):
        _, G = level_gradient(model, x.detach(), precision="fp32")
        ctx.model = model
        ctx.save_for_backward(x)
        return G

    @staticmethod
    def backward(ctx, gG):
        (x,) = ctx.saved_tensors
        grads, dx = param_grads(ctx.model, x, dg=gG, want_dx=True)
        if not ctx.needs_input_grad[0]:
            dx = None
        return (dx, None) + tuple(grads)


def level_input_grad(model, x):
    return _LevelInputGrad.apply(x, model, *model.parameters())


def create_training_data_on_neighborhood(vertices, n_on_surf, device="cuda", delta=0.02,
                                         use_neigh_delta=False, dithering_sampling=True,
                                         delta_eps=0.0005, seed=None):
    """Drop-in for experiment_scripts/utils.py:92-169, built by one kernel.

    ``vertices`` [M, 6 or 7] (xyz, normal, [neighbourhood delta]).  With
    ``seed=None`` the sample indices and uniforms are drawn from torch's
    generators exactly as the reference draws them (``torch.randperm`` on
    ``device``, ``torch.rand`` on the CPU), so the batch equals the
    reference's for the same generator state.  With an integer ``seed`` they
    come from the kernel's counter-based generator (no host work; indices
    drawn with replacement).  Returns {"on_surf": [pts, normals, sdfs]}.
    """
    V = vertices.detach().to(device=device, dtype=torch.float32).contiguous()
    if not V.is_cuda:
        raise RuntimeError("mplicits_gb300 builds training batches on a CUDA device only")
    M, C = V.shape
    n = min(int(n_on_surf), M)
    idx = u = None
    if seed is None:
        if int(n_on_surf) == M:
            idx = torch.arange(M, device=V.device)
        else:
            idx = torch.randperm(M, device=V.device)[:n_on_surf]
        u = torch.rand((n, 3)).to(V.device)
        idx = idx.to(torch.int64).contiguous()
    rows = 3 * n if dithering_sampling else 2 * n
    pts = torch.empty(rows, 3, dtype=torch.float32, device=V.device)
    nrm = torch.empty(rows, 3, dtype=torch.float32, device=V.device)
    sdf = torch.empty(rows, dtype=torch.float32, device=V.device)
    flags = (capi.MPL_BATCH_NEIGH_DELTA if use_neigh_delta else 0) | \
        (capi.MPL_BATCH_DITHER if dithering_sampling else 0)
    capi.check(capi.load().mpl_train_batch(
        capi.ptr(V), M, C, capi.ptr(idx), capi.ptr(u), n, float(delta), float(delta_eps), flags,
        0 if seed is None else int(seed) & ((1 << 64) - 1), capi.ptr(pts), capi.ptr(nrm),
        capi.ptr(sdf), capi.stream_ptr()), "mpl_train_batch")
    return {"on_surf": [pts, nrm, sdf]}


class ResidualTrainer:
    """Adam training of one level against frozen coarser levels.

    ``loss="residual"`` is the medium and fine trainers' loss_add_detail(_fine)
    (i3d/loss_functions.py:263-394): ``step(x, normals, sdf)`` takes a batch
    built like create_training_data_on_neighborhood (sdf == -1 marks points
    without SDF or normal supervision) and returns the weighted terms
    (sdf, normal, eikonal) as a device tensor [3].  ``loss="true_sdf"`` is the
    coarse trainer's loss (i3d/loss_functions.py:123-163; no frozen levels;
    sdf == 0 marks surface points) with terms (sdf on surface, sdf off
    surface, normal, eikonal) [4].  No host sync either way.
    """

    def __init__(self, model, frozen=(), lr=1e-4, betas=(0.9, 0.999), eps=1e-8,
                 constraint_weights=None, precision="fp32", loss="residual"):
        if precision not in ("fp32", "bf16"):
            raise ValueError("precision is 'fp32' (plain kernels) or 'bf16' (tensor cores)")
        if loss not in LOSSES:
            raise ValueError(f"loss is one of {sorted(LOSSES)}")
        if loss == "true_sdf" and frozen:
            raise ValueError("the true_sdf loss trains a first level: no frozen levels")
        self.precision = precision
        self.model = model
        self.frozen = list(frozen)
        self.lr, self.betas, self.eps = lr, betas, eps
        kind, defaults = LOSSES[loss]
        w = dict(defaults)
        if constraint_weights:
            w.update({k: float(v) for k, v in constraint_weights.items()})
        self.weights = w
        self.names = list(defaults)
        self.loss = capi.MplLoss(kind=kind)
        for i, k in enumerate(self.names):
            self.loss.weight[i] = w[k]
        self.params = list(model.parameters())
        self.exp_avg = [torch.zeros_like(p) for p in self.params]
        self.exp_avg_sq = [torch.zeros_like(p) for p in self.params]
        self.t = 0
        self.loss_sums = torch.zeros(4, dtype=torch.float32, device=self.params[0].device)
        self._scale = torch.tensor([w[k] for k in self.names], dtype=torch.float32,
                                   device=self.params[0].device)

    @torch.no_grad()
    def loss_and_grads(self, x, normals, sdf):
        """The weighted loss terms (``self.names``) and the gradients of their
        sum, in ``model.parameters()`` order."""
        x = x.detach().float().reshape(-1, 3).contiguous()
        normals = normals.detach().float().reshape(-1, 3).contiguous()
        sdf = sdf.detach().float().reshape(-1).contiguous()
        n = x.shape[0]
        Ff = Gf = None
        if self.frozen:
            Ff = torch.empty(n, dtype=torch.float32, device=x.device)
            Gf = torch.empty(n, 3, dtype=torch.float32, device=x.device)
            for i, m in enumerate(self.frozen):
                level_gradient(m, x, S=Ff, G=Gf, accumulate=i > 0, precision=self.precision)
        if self.precision == "bf16":
            return self._tc_loss_and_grads(x, normals, sdf, Ff, Gf)
        sc = _scratch(self.model, n, x.device)
        _forward_with_scratch(self.model, x, sc)
        capi.check(capi.load().mpl_train_loss(
            n, capi.ptr(sc.f), capi.ptr(sc.g), capi.ptr(Ff), capi.ptr(Gf), capi.ptr(sdf),
            capi.ptr(normals), ctypes.byref(self.loss), capi.ptr(sc.seeds[:n]),
            capi.ptr(self.loss_sums), capi.stream_ptr()), "mpl_train_loss")
        _backward(self.model, x, sc)
        grads = _unpad(self.model, sc)
        return self.loss_sums[:len(self.names)] * (self._scale / n), grads

    def _tc_loss_and_grads(self, x, normals, sdf, Ff, Gf):
        """One mpl_train_tc_step: forward, loss, backward and weight gradients
        on the tensor cores."""
        n = x.shape[0]
        lib = capi.load()
        net, packed = self.model.packed()
        nb = ctypes.c_int64(0)
        capi.check(lib.mpl_train_tc_scratch_bytes(ctypes.byref(net), n, ctypes.byref(nb)),
                   "mpl_train_tc_scratch_bytes")
        buf = getattr(self, "_tc_buf", None)
        if buf is None or buf.numel() < nb.value + 256:
            buf = torch.empty(nb.value + 256, dtype=torch.uint8, device=x.device)
            self._tc_buf = buf
        off = (-buf.data_ptr()) % 256
        sc = _scratch(self.model, 1, x.device)  # the padded gradient buffers
        seeds = getattr(self, "_tc_seeds", None)
        if seeds is None or seeds.shape[0] < n:
            seeds = torch.empty(n, 4, dtype=torch.float32, device=x.device)
            self._tc_seeds = seeds
        for t in sc.dW + sc.db:
            t.zero_()
        P = ctypes.c_void_p
        dW = (P * len(sc.dW))(*[t.data_ptr() for t in sc.dW])
        db = (P * len(sc.db))(*[t.data_ptr() for t in sc.db])
        capi.check(lib.mpl_train_tc_step(
            ctypes.byref(net), capi.ptr(packed), capi.ptr(x), n, capi.ptr(Ff), capi.ptr(Gf),
            capi.ptr(sdf), capi.ptr(normals), ctypes.byref(self.loss),
            ctypes.c_void_p(buf.data_ptr() + off), nb.value, capi.ptr(seeds),
            capi.ptr(self.loss_sums), dW, db, capi.stream_ptr()), "mpl_train_tc_step")
        grads = _unpad(self.model, sc)
        return self.loss_sums[:len(self.names)] * (self._scale / n), grads

    @torch.no_grad()
    def step(self, x, normals, sdf):
        losses, grads = self.loss_and_grads(x, normals, sdf)
        self.t += 1
        cnt = len(self.params)
        P = ctypes.c_void_p
        capi.check(capi.load().mpl_adam_step(
            cnt, (P * cnt)(*[p.data_ptr() for p in self.params]),
            (P * cnt)(*[g.data_ptr() for g in grads]),
            (P * cnt)(*[m.data_ptr() for m in self.exp_avg]),
            (P * cnt)(*[v.data_ptr() for v in self.exp_avg_sq]),
            (ctypes.c_int64 * cnt)(*[p.numel() for p in self.params]),
            self.lr, self.betas[0], self.betas[1], self.eps, self.t, capi.stream_ptr()),
            "mpl_adam_step")
        # the update is in place and bypasses autograd's version counter
        self.model._packed.key = None
        return losses
