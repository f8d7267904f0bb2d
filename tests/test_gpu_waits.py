"""Bounded device-side waits that run out, on the GPU, without a fault or a hang.

The compaction's decoupled look-back waits (bounded) for the tile before it to publish its
prefix.  tqpk_debug_compact_wait makes one tile's CTA publish nothing and shortens the poll
limit, so the next tile's wait runs out: the kernel still finishes, the count it leaves is the
status TQPK_ETIMEOUT, the Python layer raises TimeoutError, and the context stays usable."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEFAULT_SPIN_LIMIT = 1 << 21


@pytest.fixture(scope="module")
def lib():
    from tqpk import build, _lib
    build.build()
    return _lib.load()


@pytest.fixture
def stalled_tile(lib):
    from tqpk import _lib as L
    assert lib.tqpk_debug_compact_wait(4096, 1) == L.OK       # tile 1 stays silent; 4096 polls
    yield
    assert lib.tqpk_debug_compact_wait(DEFAULT_SPIN_LIMIT, -1) == L.OK


def _arrays(ptrs):
    a = (C.c_void_p * len(ptrs))()
    for i, p in enumerate(ptrs):
        a[i] = p
    return a


def _compact_count(lib, mask, col, noalloc):
    from tqpk import _lib as L
    from tqpk.dtypes import code_of
    n = mask.numel()
    out = torch.empty_like(col)
    cnt = torch.full((1,), 12345, dtype=torch.int64, device="cuda")
    dts = (C.c_int32 * 1)(code_of(col.dtype))
    s = torch.cuda.current_stream().cuda_stream
    if noalloc:
        st = lib.tqpk_compact_noalloc(None, mask.data_ptr(), n, 1, _arrays([col.data_ptr()]), dts,
                                      _arrays([out.data_ptr()]), cnt.data_ptr(), s)
    else:
        ws = torch.empty(lib.tqpk_compact_workspace_bytes(n), dtype=torch.uint8, device="cuda")
        st = lib.tqpk_compact(None, mask.data_ptr(), n, 1, _arrays([col.data_ptr()]), dts,
                              _arrays([out.data_ptr()]), cnt.data_ptr(), ws.data_ptr(), ws.numel(), s)
        torch.cuda.synchronize()
    assert st == L.OK, st
    torch.cuda.synchronize()
    return int(cnt.item()), out


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    mask = torch.from_numpy(rng.random(n) < 0.4).cuda()
    col = torch.from_numpy(rng.integers(-2**40, 2**40, n)).cuda()
    return mask, col


@pytest.mark.parametrize("noalloc", [False, True])
def test_compaction_lookback_timeout_is_reported(lib, stalled_tile, noalloc):
    from tqpk import _lib as L
    mask, col = _inputs(64 * 4096 + 5, 7)
    got, _ = _compact_count(lib, mask, col, noalloc)
    assert got == L.ETIMEOUT


def test_compaction_timeout_raises_in_python(lib, stalled_tile):
    from tqpk.ops import compact
    mask, col = _inputs(20 * 4096, 8)
    with pytest.raises(TimeoutError):
        compact([col], mask)


def test_compaction_correct_after_a_timeout(lib):
    from tqpk import _lib as L
    mask, col = _inputs(64 * 4096 + 5, 9)
    assert lib.tqpk_debug_compact_wait(4096, 1) == L.OK
    try:
        assert _compact_count(lib, mask, col, False)[0] == L.ETIMEOUT
    finally:
        assert lib.tqpk_debug_compact_wait(DEFAULT_SPIN_LIMIT, -1) == L.OK
    for noalloc in (False, True):
        m, out = _compact_count(lib, mask, col, noalloc)
        keep = mask.cpu().numpy()
        assert m == int(keep.sum())
        np.testing.assert_array_equal(out[:m].cpu().numpy(), col.cpu().numpy()[keep])


def test_topk_grid_barrier_timeout_is_reported(lib):
    """The single-launch top-k's grid barrier (fused join pipeline, k <= 32) made to wait for an
    arrival that never comes: every CTA's bounded wait runs out, the pipeline's error word holds
    TQPK_ETIMEOUT and result_device raises TimeoutError; the next run, with the defaults back, is
    the same as the one before."""
    from tqpk import _lib as L, datagen
    from tqpk.pipeline import JoinAggTopK
    t = {k: torch.from_numpy(v).cuda() for k, v in datagen.join_tables(100_000, 400_003, 71).items()}
    pipe = JoinAggTopK(t["b_key"], 1, 100_000, t["p_fk"], {12: t["b_date"]}, [["bd#12", "<", "1170"]],
                       {22: t["p_date"], 23: t["p_price"], 24: t["p_discount"]}, [["pd#22", ">", "1170"]],
                       [["p#23", "*", ["1.0", "-", "d#24"]]], k=10)
    pipe.run()
    keys0, vals0, m0 = pipe.result_device()
    keys0, vals0 = keys0.cpu().numpy(), vals0.cpu().numpy()
    assert lib.tqpk_debug_topk_barrier(4096, 1) == L.OK
    try:
        pipe.run()
        with pytest.raises(TimeoutError):
            pipe.result_device()
    finally:
        assert lib.tqpk_debug_topk_barrier(DEFAULT_SPIN_LIMIT, 0) == L.OK
    pipe.run()
    keys1, vals1, m1 = pipe.result_device()
    assert m1 == m0 == 10
    np.testing.assert_array_equal(keys1.cpu().numpy(), keys0)
    np.testing.assert_allclose(vals1.cpu().numpy(), vals0, rtol=1e-12)

