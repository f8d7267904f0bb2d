"""The allocation-free compaction entry point against the regular one.

tqpk_compact_noalloc is for callers that cannot allocate device memory when
they call; it keeps its scratch in a static array inside the library.  This
file is named so pytest collects it last; it passes on its own in a fresh
process as well as after the other tests.  Both entry points are called
through the C ABI; compaction is exact, so the outputs must be identical."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from tqpk import build, _lib
    build.build()
    return _lib.load()


def _arrays(ptrs):
    a = (C.c_void_p * len(ptrs))()
    for i, p in enumerate(ptrs):
        a[i] = p
    return a


def _run(lib, fn, n, mask, cols, with_ws):
    from tqpk import _lib as L
    from tqpk.dtypes import code_of
    outs = [torch.empty(n, dtype=c.dtype, device="cuda") for c in cols] + [torch.empty(n, dtype=torch.int64,
                                                                                        device="cuda")]
    dts = (C.c_int32 * (len(cols) + 1))(*([code_of(c.dtype) for c in cols] + [L.ROWID]))
    ins = _arrays([c.data_ptr() for c in cols] + [None])
    optr = _arrays([o.data_ptr() for o in outs])
    cnt = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    if with_ws:
        ws = torch.empty(lib.tqpk_compact_workspace_bytes(n), dtype=torch.uint8, device="cuda")
        st = fn(None, mask.data_ptr(), n, len(cols) + 1, ins, dts, optr, cnt.data_ptr(), ws.data_ptr(), ws.numel(), s)
    else:
        st = fn(None, mask.data_ptr(), n, len(cols) + 1, ins, dts, optr, cnt.data_ptr(), s)
    assert st == 0, st
    torch.cuda.synchronize()
    m = int(cnt.item())
    return m, [o[:m].cpu().numpy() for o in outs]


def test_noalloc_matches_compact_on_two_calls_in_a_row(lib):
    for n, density, seed in ((1_000_003, 0.6, 1), (70_001, 0.05, 2)):
        rng = np.random.default_rng(seed)
        mask = torch.from_numpy(rng.random(n) < density).cuda()
        cols = [torch.from_numpy(rng.integers(-2**40, 2**40, n)).cuda(),
                torch.from_numpy(rng.random(n)).cuda(),
                torch.from_numpy(rng.integers(0, 255, n).astype(np.uint8)).cuda()]
        m_ref, ref = _run(lib, lib.tqpk_compact, n, mask, cols, True)
        m_na, got = _run(lib, lib.tqpk_compact_noalloc, n, mask, cols, False)
        assert m_na == m_ref == int(mask.sum().item())
        for a, b in zip(got, ref):
            np.testing.assert_array_equal(a, b)


def test_noalloc_rejects_inputs_beyond_its_scratch(lib):
    from tqpk import _lib as L
    too_many = lib.tqpk_compact_noalloc_max_rows() + 1
    cnt = torch.full((1,), 7, dtype=torch.int64, device="cuda")
    mask = torch.ones(16, dtype=torch.bool, device="cuda")      # the call must not touch these
    out = torch.zeros(16, dtype=torch.int64, device="cuda")
    dts = (C.c_int32 * 1)(L.ROWID)
    st = lib.tqpk_compact_noalloc(None, mask.data_ptr(), too_many, 1, _arrays([None]), dts, _arrays([out.data_ptr()]),
                                  cnt.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert st == L.ENOMEM
    assert int(cnt.item()) == 7 and int(out.abs().sum().item()) == 0
