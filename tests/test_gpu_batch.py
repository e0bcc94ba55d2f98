"""One persistent launch over many levels of many models: bit-exact against
the single-level tensor-core kernel on each entry, within the BF16 error of
the plain FP32 form, under every configuration the autotuner chooses from,
and replayed from a CUDA graph."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _model(width, depth, seed, precision):
    from mplicits_gb300.model import SIREN
    torch.manual_seed(seed)
    return SIREN(3, 1, [width] * depth, w0=30, precision=precision).cuda().eval()


def _entries(precision, seed=0):
    from mplicits_gb300.batch import BatchEntry
    g = torch.Generator("cuda").manual_seed(seed)
    rng = np.random.default_rng(seed)
    specs = [(256, 3, 5000), (128, 3, 777), (64, 3, 130), (256, 2, 129), (128, 2, 4096),
             (256, 3, 1), (128, 3, 20000), (64, 2, 3000), (256, 3, 0), (128, 3, 2500)]
    entries, models = [], []
    for i, (w, d, n) in enumerate(specs):
        m = _model(w, d, 100 + i, precision)
        models.append(m)
        P = max(n, 1) + 17
        x = torch.rand(P, 3, device="cuda", generator=g) * 2 - 1
        S = torch.full((P,), 7.0, device="cuda")
        kw = {}
        if i % 3 == 1:  # index list
            kw["index"] = torch.from_numpy(rng.permutation(P)[:n].astype(np.int32)).cuda()
        if i % 4 == 2:  # device count below n
            kw["n_dev"] = torch.tensor([max(n - 5, 0)], dtype=torch.int32, device="cuda")
        entries.append(BatchEntry(m, S, x=x, n=n, accumulate=(i % 5 == 4), **kw))
    # a grid entry
    m = _model(256, 3, 99, precision)
    models.append(m)
    Sg = torch.zeros(24 ** 3, device="cuda")
    entries.append(BatchEntry(m, Sg, grid=(24, 2.0 / 23, (-1.0, -1.0, -1.0))))
    return entries, models


def _single(entries, precision):
    """Each entry through mpl_level_forward (its own launch)."""
    import ctypes
    from mplicits_gb300 import capi
    outs = []
    for e in entries:
        S = e.S.clone()
        net, packed = e.model.packed()
        if e.grid is not None:
            N, vs, off = e.grid
            pts = capi.MplPoints(kind=capi.MPL_POINTS_GRID, grid_n=N, voxel_size=vs)
            for k in range(3):
                pts.offset[k] = off[k]
        else:
            pts = capi.MplPoints(kind=capi.MPL_POINTS_XYZ, xyz=e.x.data_ptr())
        capi.check(capi.load().mpl_level_forward(
            ctypes.byref(net), capi.ptr(packed), ctypes.byref(pts), capi.ptr(e.index),
            capi.ptr(e.n_dev), e.n, capi.ptr(S),
            capi.MPL_ACCUMULATE if e.accumulate else capi.MPL_STORE, None,
            capi.PRECISIONS[precision], capi.stream_ptr()), "mpl_level_forward")
        outs.append(S)
    return outs


CONFIGS = [(1, 16, 3), (1, 16, 2), (1, 32, 3), (1, 32, 2), (2, 32, 0)]


def _check_against_single(entries, precision, tiles, unit, stages, ctas=0):
    from mplicits_gb300 import capi
    from mplicits_gb300.batch import BatchedLevels
    init = [e.S.clone() for e in entries]
    old = capi.get_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT)
    capi.set_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT, unit)
    try:
        ref = _single(entries, precision)
        bl = BatchedLevels(entries, precision)
        bl.run(capi.MplBatchConfig(epilogue_unit=unit, stages=stages, ctas=ctas,
                                   tiles_in_flight=tiles))
        torch.cuda.synchronize()
    finally:
        capi.set_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT, old)
    assert capi.device_status() == capi.MPL_OK
    for i, (e, r) in enumerate(zip(entries, ref)):
        assert torch.equal(e.S, r), i
        if e.n > 50:
            assert not torch.equal(e.S, init[i]), i


@pytest.mark.parametrize("precision", ["bf16", "fp16"])
@pytest.mark.parametrize("tiles,unit,stages", CONFIGS)
def test_batched_launch_equals_single_level_launches(lib, precision, tiles, unit, stages):
    entries, _ = _entries(precision)
    _check_against_single(entries, precision, tiles, unit, stages)


@pytest.mark.parametrize("tiles,unit,stages,ctas,precision",
                         [(2, 32, 0, 0, "bf16"), (2, 32, 0, 7, "bf16"), (2, 32, 0, 0, "fp16"),
                          (1, 32, 3, 5, "bf16"), (1, 16, 2, 0, "bf16")])
def test_many_small_entries_of_mixed_shapes(lib, tiles, unit, stages, ctas, precision):
    """Hundreds of entries of one to a few tiles each, widths and depths
    mixed, so that nearly every tile of a CTA changes entry (the slots'
    constants are refilled over and over) and rounds end with one slot
    empty; also a grid smaller than the two slots of one round."""
    from mplicits_gb300.batch import BatchEntry
    rng = np.random.default_rng(11)
    g = torch.Generator("cuda").manual_seed(11)
    models = {}
    for w in (64, 128, 256):
        for d in (2, 3):
            models[(w, d)] = _model(w, d, 7 * w + d, precision)
    entries = []
    for i in range(300):
        w = int(rng.choice([64, 128, 256]))
        d = int(rng.choice([2, 3]))
        n = int(rng.integers(0, 400))
        P = n + 3
        x = torch.rand(P, 3, device="cuda", generator=g) * 2 - 1
        kw = {}
        if i % 7 == 3:
            kw["index"] = torch.from_numpy(rng.permutation(P)[:n].astype(np.int32)).cuda()
        entries.append(BatchEntry(models[(w, d)], torch.full((P,), 5.0, device="cuda"), x=x,
                                  n=n, accumulate=(i % 11 == 5), **kw))
    _check_against_single(entries, precision, tiles, unit, stages, ctas)


def test_two_tile_pipeline_rejects_a_ring_depth_and_16_wide_units(lib):
    import ctypes
    from mplicits_gb300 import capi
    from mplicits_gb300.batch import BatchedLevels
    entries, _ = _entries("bf16")
    bl = BatchedLevels(entries[:2], "bf16")
    assert list(bl.plan.width_count) == [0, 1, 1]  # widths 256 and 128, grouped
    cfg = capi.MplBatchConfig(epilogue_unit=32, stages=2, tiles_in_flight=2)
    assert capi.load().mpl_batch_run(ctypes.byref(bl.plan), ctypes.byref(cfg),
                                     capi.stream_ptr()) == capi.MPL_ERR_UNSUPPORTED
    cfg = capi.MplBatchConfig(epilogue_unit=16, tiles_in_flight=2)
    assert capi.load().mpl_batch_run(ctypes.byref(bl.plan), ctypes.byref(cfg),
                                     capi.stream_ptr()) == capi.MPL_ERR_UNSUPPORTED
    cfg = capi.MplBatchConfig(tiles_in_flight=3)
    assert capi.load().mpl_batch_run(ctypes.byref(bl.plan), ctypes.byref(cfg),
                                     capi.stream_ptr()) == capi.MPL_ERR_INVALID_ARG


def test_batched_launch_within_bf16_error_of_fp32(lib):
    from mplicits_gb300.batch import BatchedLevels
    entries, models = _entries("bf16", seed=3)
    ref = []
    for e, m in zip(entries, models):
        m32 = type(m)(3, 1, [l.out_features for l in m.linears()[:-1]], w0=30,
                      delay_init=True, precision="fp32").cuda()
        m32.load_state_dict(m.state_dict())
        ref.append(m32)
    base = _single([type(e)(r, e.S.clone(), x=e.x, grid=e.grid, index=e.index, n=e.n,
                            n_dev=e.n_dev, accumulate=e.accumulate)
                    for e, r in zip(entries, ref)], "fp32")
    BatchedLevels(entries, "bf16").run()
    torch.cuda.synchronize()
    for e, b in zip(entries, base):
        assert (e.S - b).abs().max().item() <= 2e-3


def test_autotune_and_graph_replay(lib):
    from mplicits_gb300 import capi
    from mplicits_gb300.batch import BatchedLevels
    entries, _ = _entries("bf16", seed=5)
    for e in entries:
        e.accumulate = False
    bl = BatchedLevels(entries, "bf16")
    cfg, ms = bl.autotune(repeats=2)
    assert cfg.epilogue_unit in (16, 32) and cfg.stages in (0, 2, 3) and ms > 0
    assert cfg.tiles_in_flight in (1, 2)
    for e in entries:
        e.S.fill_(-3.0)
    old = capi.get_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT)
    capi.set_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT, cfg.epilogue_unit)
    try:
        ref = _single(entries, "bf16")
    finally:
        capi.set_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT, old)
    bl.capture()
    bl.replay()
    torch.cuda.synchronize()
    for e, r in zip(entries, ref):
        assert torch.equal(e.S, r)
    # the cache answers the same signature without timing again
    cfg2, ms2 = BatchedLevels(entries, "bf16").autotune()
    assert (cfg2.tiles_in_flight, cfg2.epilogue_unit, cfg2.stages, ms2) == \
        (cfg.tiles_in_flight, cfg.epilogue_unit, cfg.stages, ms)


def test_graph_replay_follows_device_counts(lib):
    """Device counts changed between replays of one captured graph: the
    tile prefix is rebuilt on the device by every replay."""
    from mplicits_gb300 import capi
    from mplicits_gb300.batch import BatchEntry, BatchedLevels
    g = torch.Generator("cuda").manual_seed(21)
    entries, counts = [], []
    for i, (w, d, P) in enumerate([(256, 3, 3000), (128, 3, 5000), (256, 2, 700), (128, 2, 900)]):
        m = _model(w, d, 300 + i, "bf16")
        x = torch.rand(P, 3, device="cuda", generator=g) * 2 - 1
        c = torch.tensor([P], dtype=torch.int32, device="cuda")
        counts.append(c)
        entries.append(BatchEntry(m, torch.zeros(P, device="cuda"), x=x, n=P, n_dev=c))
    bl = BatchedLevels(entries, "bf16")
    bl.config = capi.MplBatchConfig(epilogue_unit=32, tiles_in_flight=2)
    bl.capture()
    old = capi.get_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT)
    capi.set_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT, 32)
    try:
        for frac in (1.0, 0.37, 0.0, 0.81):
            for e, c in zip(entries, counts):
                c.fill_(int(e.n * frac))
                e.S.fill_(9.0)
            ref = _single(entries, "bf16")
            bl.replay()
            torch.cuda.synchronize()
            for i, (e, r) in enumerate(zip(entries, ref)):
                assert torch.equal(e.S, r), (frac, i)
    finally:
        capi.set_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT, old)
    assert capi.device_status() == capi.MPL_OK


def test_batch_rejects_unsupported_entries(lib):
    import ctypes
    from mplicits_gb300 import capi
    from mplicits_gb300.batch import BatchEntry, BatchedLevels
    m = _model(256, 5, 1, "bf16")  # four hidden GEMMs
    x = torch.rand(10, 3, device="cuda")
    with pytest.raises(capi.MplError):
        BatchedLevels([BatchEntry(m, torch.empty(10, device="cuda"), x=x)], "bf16")
    with pytest.raises(ValueError):
        BatchedLevels([], "fp32")
    plan = capi.MplBatchPlan()
    assert capi.load().mpl_batch_prepare(None, 1, capi.MPL_BF16, None, 0, ctypes.byref(plan),
                                         None) == capi.MPL_ERR_INVALID_ARG
