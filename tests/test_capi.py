"""The C-ABI library loads and exports exactly what include/mplicits.h
declares (no compute calls: runs without a GPU)."""

import ctypes
import os
import re
import subprocess

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "mplicits.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return set(re.findall(r"\b(mpl_\w+)\s*\(", src))


def test_header_and_binding_agree():
    from mplicits_gb300 import capi
    assert _declared() == set(capi.SIGNATURES)


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib._name], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (mpl_\w+)", out))
    assert _declared() <= exported
    for name in _declared():
        assert isinstance(getattr(lib, name), ctypes._CFuncPtr)


def test_host_side_queries_without_gpu(lib):
    from mplicits_gb300 import capi
    assert lib.mpl_abi_version() == 1
    assert lib.mpl_status_string(capi.MPL_ERR_CAPACITY) == b"output capacity exceeded"
    net = capi.MplNet()
    net.n_layers = 4
    for i, d in enumerate([3, 256, 256, 256, 1]):
        net.dims[i] = d
    nb = ctypes.c_int64(0)
    assert lib.mpl_net_packed_bytes(ctypes.byref(net), ctypes.byref(nb)) == 0
    assert nb.value > 2 * 256 * 256 * 4
    net.dims[0] = 4  # space-time models are not on the path
    assert lib.mpl_net_packed_bytes(ctypes.byref(net), ctypes.byref(nb)) == capi.MPL_ERR_UNSUPPORTED
    net.dims[0] = 3
    net.dims[2] = 300
    assert lib.mpl_net_packed_bytes(ctypes.byref(net), ctypes.byref(nb)) == capi.MPL_ERR_UNSUPPORTED
    ws = ctypes.c_int64(0)
    assert lib.mpl_mc_workspace_bytes(512, ctypes.byref(ws)) == 0 and ws.value > 512 * 512 * 16
    assert lib.mpl_mc_workspace_bytes(1, ctypes.byref(ws)) == capi.MPL_ERR_INVALID_ARG
    # invalid arguments are rejected before any device work
    assert lib.mpl_level_forward(None, None, None, None, None, 0, None, 0, None, 0, None) == \
        capi.MPL_ERR_INVALID_ARG


def test_trace_march_rejects_before_device_work(lib):
    """The persistent marching entry point validates its arguments and the
    levels' shapes on the host: missing buffers, FP32 precision, unequal
    widths and widths without a tensor-core tiling are refused."""
    from mplicits_gb300 import capi
    P = ctypes.c_void_p

    def net(widths):
        n = capi.MplNet()
        dims = [3] + list(widths) + [1]
        n.n_layers = len(dims) - 1
        for i, d in enumerate(dims):
            n.dims[i] = d
        for i in range(n.n_layers):
            n.omega[i] = 30.0
        return n

    fake = P(1 << 20)  # 256-byte aligned, never dereferenced on these paths
    deltas = (ctypes.c_float * 2)(0.05, 0.01)

    def call(nets, packed, levels, precision, active=fake):
        arr = (capi.MplNet * len(nets))(*nets)
        pk = (ctypes.c_void_p * len(packed))(*packed)
        return lib.mpl_trace_march(arr, ctypes.cast(pk, P), levels, ctypes.cast(deltas, P), active,
                                   fake, 16, fake, fake, fake, fake, 1e-4, 1.2, 8, 1, fake, fake,
                                   16, precision, None)

    w256 = [256, 256, 256]
    assert call([net(w256)] * 3, [fake] * 3, 3, capi.MPL_BF16, active=None) == \
        capi.MPL_ERR_INVALID_ARG
    assert call([net(w256)] * 3, [fake] * 3, 0, capi.MPL_BF16) == capi.MPL_ERR_INVALID_ARG
    assert call([net(w256)] * 4, [fake] * 4, 4, capi.MPL_BF16) == capi.MPL_ERR_INVALID_ARG
    assert call([net(w256)] * 3, [fake] * 3, 3, capi.MPL_FP32) == capi.MPL_ERR_UNSUPPORTED
    assert call([net(w256), net([128, 128, 128]), net(w256)], [fake] * 3, 3, capi.MPL_BF16) == \
        capi.MPL_ERR_UNSUPPORTED
    assert call([net([64, 64])] * 2, [fake] * 2, 2, capi.MPL_F16) == capi.MPL_ERR_UNSUPPORTED
    assert call([net(w256)] * 3, [fake, P(1 << 20 | 8), fake], 3, capi.MPL_BF16) == \
        capi.MPL_ERR_INVALID_ARG
