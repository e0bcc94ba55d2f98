"""The device-timeout contract: a bounded device-side wait that cannot
complete gives up, the status word reports MPL_ERR_DEVICE_TIMEOUT, the
CTA's other waits leave through its abort flag, the launch returns, and the
next normal call succeeds.  No fault is made: the waits are on mbarriers
that nothing arrives at, with no copy or MMA in flight."""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_the_context_stays_usable(lib):
    from mplicits_gb300 import capi
    from mplicits_gb300.model import SIREN, level_forward
    assert capi.device_status() == capi.MPL_OK
    limit = 50_000_000  # 50 ms
    res = torch.full((4,), -1, dtype=torch.int64, device="cuda")
    capi.check(lib.mpl_wait_selftest(limit, capi.ptr(res), capi.stream_ptr()),
               "mpl_wait_selftest")
    assert capi.device_status() == capi.MPL_ERR_DEVICE_TIMEOUT
    ok0, ok1, dt0, dt1 = res.tolist()
    assert ok0 == 0 and ok1 == 0
    assert dt0 >= limit
    # warp 1 waited with the kernels' 2 s limit but left through the abort
    # flag shortly after warp 0 gave up
    assert dt1 < 1_000_000_000
    # the status word was cleared by the read; a normal launch succeeds
    assert capi.device_status() == capi.MPL_OK
    torch.manual_seed(0)
    m = SIREN(3, 1, [256, 256, 256], w0=30, precision="bf16").cuda().eval()
    x = torch.rand(4096, 3, device="cuda") * 2 - 1
    S = level_forward(m, x)
    ref = level_forward(m, x, precision="fp32")
    torch.cuda.synchronize()
    assert capi.device_status() == capi.MPL_OK
    assert (S - ref).abs().max().item() < 5e-3


def test_wait_selftest_rejects_limits_outside_its_range(lib):
    from mplicits_gb300 import capi
    res = torch.zeros(4, dtype=torch.int64, device="cuda")
    for bad in (0, 999_999, 2_000_000_001):
        assert lib.mpl_wait_selftest(bad, capi.ptr(res), capi.stream_ptr()) == \
            capi.MPL_ERR_INVALID_ARG
    assert lib.mpl_wait_selftest(10_000_000, None, capi.stream_ptr()) == capi.MPL_ERR_INVALID_ARG
