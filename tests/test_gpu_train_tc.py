"""The tensor-core (BF16) training step against the plain FP32 kernels (whose
gradients match the reference's autograd and the FP64 oracle) and the FP64
oracle itself, on 128- and 256-wide levels with ragged point counts."""

import numpy as np
import pytest
import torch

from oracle import train as ot

pytestmark = pytest.mark.gpu


def _level(widths, seed, scale=2.0):
    rng = np.random.default_rng(seed)
    dims = [3] + widths + [1]
    params = []
    for i in range(len(dims) - 1):
        fan = dims[i]
        lim = (1.0 / fan) if i == 0 else (np.sqrt(6.0 / fan) / 30.0)
        W = rng.uniform(-lim, lim, (dims[i + 1], fan)).astype(np.float32) * (scale if i else 1)
        b = rng.uniform(-0.05, 0.05, dims[i + 1]).astype(np.float32)
        params.append((W, b))
    return params


def _siren(params, precision):
    from mplicits_gb300.model import SIREN
    widths = [W.shape[0] for W, _ in params[:-1]]
    m = SIREN(3, 1, widths, w0=30, delay_init=True, precision=precision)
    m.load_state_dict({f"net.{j}.0.{k}": torch.from_numpy(v)
                       for j, (W, b) in enumerate(params) for k, v in (("weight", W), ("bias", b))})
    return m.cuda()


def _batch(n, seed):
    rng = np.random.default_rng(seed)
    xs = rng.uniform(-0.9, 0.9, (n, 3)).astype(np.float32)
    nrm = (xs / np.linalg.norm(xs, axis=1, keepdims=True)).astype(np.float32)
    sdf = rng.uniform(-0.02, 0.02, (n, 1)).astype(np.float32)
    sdf[rng.random(n) < 0.4] = -1.0
    return xs, nrm, sdf


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("widths,n", [([256] * 3, 3000), ([128] * 3, 4099), ([256] * 2, 777),
                                      ([128] * 2, 1)])
def test_tensor_core_step_matches_fp32_and_oracle(lib, widths, n):
    from mplicits_gb300.train import ResidualTrainer
    params = _level(widths, 40 + n)
    fparams = _level([128] * 3, 5)
    xs, nrm, sdf = _batch(n, n)
    X, N, D = (torch.from_numpy(a).cuda() for a in (xs, nrm, sdf))
    res = {}
    for prec in ("fp32", "bf16"):
        fine = _siren(params, prec)
        frozen = [_siren(fparams, prec).eval()]
        tr = ResidualTrainer(fine, frozen, precision=prec)
        losses, grads = tr.loss_and_grads(X, N, D)
        torch.cuda.synchronize()
        res[prec] = (losses.cpu().numpy(), [g.cpu().numpy().astype(np.float64) for g in grads])
    from mplicits_gb300 import capi
    assert capi.device_status() == capi.MPL_OK
    ref_l, ref_g = ot.residual_step_grads(params, [30.0] * (len(widths)),
                                          [(fparams, [30.0] * 3)], xs, sdf, nrm)
    keys = ["sdf_constraint", "normal_constraint", "grad_constraint"]
    # BF16 roundings: a few 1e-3 relative on each gradient; a loss over a
    # handful of points (squared) sees the tail of that spread
    ltol = 3e-2 if n >= 100 else 6e-2
    for i, k in enumerate(keys):
        assert abs(res["fp32"][0][i] - ref_l[k]) <= 1e-4 * abs(ref_l[k]) + 1e-6, k
        assert abs(res["bf16"][0][i] - ref_l[k]) <= ltol * abs(ref_l[k]) + 1e-4, k
    for j in range(len(params)):
        for t in range(2):
            ref = ref_g[j][t].reshape(res["bf16"][1][2 * j + t].shape)
            assert _rel(res["fp32"][1][2 * j + t], ref) <= 1e-4, (j, t)
            # BF16 operands: a few 1e-3 of each tensor's norm
            assert _rel(res["bf16"][1][2 * j + t], ref) <= 3e-2, (j, t, _rel(res["bf16"][1][2 * j + t], ref))


def test_tensor_core_training_descends_like_fp32(lib):
    """Twenty Adam steps on the same batches from the same start: the BF16
    step's losses track the FP32 step's."""
    from mplicits_gb300.train import ResidualTrainer
    params = _level([256] * 3, 7)
    fparams = _level([256] * 3, 8)
    curves = {}
    for prec in ("fp32", "bf16"):
        fine = _siren(params, prec)
        tr = ResidualTrainer(fine, [_siren(fparams, prec).eval()], lr=1e-4, precision=prec)
        out = []
        for k in range(20):
            xs, nrm, sdf = _batch(8192, 100 + k)
            L = tr.step(*(torch.from_numpy(a).cuda() for a in (xs, nrm, sdf)))
            out.append(float(L.sum()))
        curves[prec] = np.array(out)
    a, b = curves["fp32"], curves["bf16"]
    assert a[-1] < a[0] and b[-1] < b[0]
    assert np.all(np.abs(a - b) <= 0.05 * np.abs(a) + 1e-3), (a, b)


@pytest.mark.parametrize("widths,n", [([256] * 3, 2500), ([128] * 3, 999)])
def test_tensor_core_true_sdf_step_matches_oracle(lib, widths, n):
    """The coarse trainer's loss on the tensor-core step against the FP64
    oracle (itself pinned to the reference's true_sdf and finite differences)."""
    from mplicits_gb300.train import ResidualTrainer
    params = _level(widths, 77 + n)
    rng = np.random.default_rng(n)
    xs = rng.uniform(-0.9, 0.9, (n, 3)).astype(np.float32)
    nrm = (xs / np.linalg.norm(xs, axis=1, keepdims=True)).astype(np.float32)
    sdf = rng.uniform(-0.3, 0.3, (n, 1)).astype(np.float32)
    sdf[: n // 2] = 0.0
    nrm[n // 2:] = 0.0  # off-surface rows carry no normal, as the reference's batches
    X, N, D = (torch.from_numpy(a).cuda() for a in (xs, nrm, sdf))
    ref_l, ref_g = ot.true_sdf_step_grads(params, [30.0] * len(widths), xs, sdf, nrm)
    for prec, tol_l, tol_g in (("fp32", 1e-4, 1e-4), ("bf16", 3e-2, 3e-2)):
        tr = ResidualTrainer(_siren(params, prec), precision=prec, loss="true_sdf")
        losses, grads = tr.loss_and_grads(X, N, D)
        lo = losses.cpu().numpy()
        for i, k in enumerate(tr.names):
            assert abs(lo[i] - ref_l[k]) <= tol_l * abs(ref_l[k]) + 1e-4, (prec, k)
        for j in range(len(params)):
            for t in range(2):
                got = grads[2 * j + t].cpu().numpy().astype(np.float64)
                ref = ref_g[j][t].reshape(got.shape)
                assert _rel(got, ref) <= tol_g, (prec, j, t, _rel(got, ref))
