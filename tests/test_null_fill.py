"""Null-filled gathers of a right-outer join's build-side columns (conversion.py:52-57).

The reference fills the rows of unmatched probe rows with masked_fill_ of a [K] mask, which torch
broadcasts from the right.  A 1-D column gets per-row nulls.  A 2-D [K, w] result is filled per row
when K == 1, per column when K == w, and otherwise the call raises RuntimeError.  The oracle's
restatement and the drop-in's host logic are checked here against the reference's own function,
run on CPU tensors.  The drop-in's two gather kernels are replaced by torch indexing with their
documented semantics; the kernels themselves are checked on the GPU against the oracle.
"""
import sys
from pathlib import Path

import numpy as np
import pytest
import torch

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from oracle import reference  # noqa: E402
from oracle import tqp_oracle as O  # noqa: E402

NULL = -64

# (rows N, width w or 0 for a 1-D column, output indices with NULL for unmatched probe rows)
CASES = [
    (6, 0, [0, 2, NULL, 1]),            # 1-D: per-row nulls
    (6, 5, [3]),                        # K == 1 (one matched pair, nothing to fill)
    (6, 4, [0, NULL, 2, 5]),            # K == w: column 1 of every row
    (6, 3, [4, NULL, NULL]),            # K == w: columns 1 and 2
    (6, 5, [0, 2, NULL]),               # K != 1, K != w: refused
    (6, 1, [1]),                        # [N, 1], K == 1
    (6, 1, [0, 2, NULL, 1]),            # [N, 1], K > 1: refused
]


def _data(n, w, dtype=torch.int8):
    shape = (n,) if w == 0 else (n, w)
    return torch.arange(1, 1 + int(np.prod(shape)), dtype=torch.int64).reshape(shape).to(dtype)


def _reference(ref, data, idx):
    try:
        return ref.hashjoin.index_with_null(data.clone(), idx)
    except RuntimeError:
        return RuntimeError


@pytest.fixture(scope="module")
def ref():
    ok, why = reference.available()
    if not ok:
        pytest.skip(why)
    return reference.load()


@pytest.mark.parametrize("n,w,idx", CASES)
def test_oracle_index_with_null_follows_the_reference(ref, n, w, idx):
    data = _data(n, w)
    t = torch.tensor(idx, dtype=torch.int64)
    expect = _reference(ref, data, t)
    if expect is RuntimeError:
        with pytest.raises(RuntimeError):
            O.index_with_null(data.numpy(), t.numpy())
        return
    got = O.index_with_null(data.numpy(), t.numpy())
    assert got.shape == tuple(expect.shape)
    np.testing.assert_array_equal(got, expect.numpy())


@pytest.fixture()
def cpu_gathers(monkeypatch):
    """The drop-in's gather with its two kernels replaced by torch indexing on CPU tensors."""
    from tqpk import ops

    def gather_1d(cols, idx, null_aware):
        outs = []
        for c in cols:
            c = c.reshape(-1)
            if null_aware:
                m = idx == NULL
                o = c[idx.masked_fill(m, 0)].clone()
                o[m] = NULL
            else:
                o = c[idx]
            outs.append(o)
        return outs

    def gather_rows(col, idx):
        assert col.dim() == 2 and col.shape[1] > 1      # [N, 1] takes the 1-D kernel
        return col[idx]

    monkeypatch.setattr(ops, "_gather_1d", gather_1d)
    monkeypatch.setattr(ops, "gather_rows", gather_rows)
    return ops


@pytest.mark.parametrize("n,w,idx", CASES)
@pytest.mark.parametrize("dtype", [torch.int8, torch.float64])
def test_drop_in_null_fill_follows_the_reference(ref, cpu_gathers, n, w, idx, dtype):
    data = _data(n, w, dtype)
    t = torch.tensor(idx, dtype=torch.int64)
    expect = _reference(ref, data, t)
    if expect is RuntimeError:
        with pytest.raises(RuntimeError):
            cpu_gathers.gather([data], t, null_aware=True)
        return
    (got,) = cpu_gathers.gather([data], t, null_aware=True)
    assert got.shape == expect.shape and got.dtype == expect.dtype
    torch.testing.assert_close(got, expect, rtol=0, atol=0)


def test_drop_in_gather_keeps_torch_shapes(cpu_gathers):
    """A join's payload columns keep their shapes: [N] -> [K], [N, 1] -> [K, 1], [N, w] -> [K, w]
    (hashjoin.py:153-175 indexes them with x[idx])."""
    cols = [_data(7, 0, torch.int32), _data(7, 1, torch.int64), _data(7, 4), _data(7, 1, torch.float64)]
    idx = torch.tensor([6, 0, 3, 3, 1], dtype=torch.int64)
    outs = cpu_gathers.gather(cols, idx)
    for c, o in zip(cols, outs):
        torch.testing.assert_close(o, c[idx], rtol=0, atol=0)
        assert o.shape == c[idx].shape


def test_right_outer_outputs_follow_the_reference(cpu_gathers):
    """hashjoin._outputs for a right-outer join: build-side columns null-filled by the rule above
    (a 1-D and an [N, 1] column here, K == 1 and K > 1), probe-side columns plain."""
    from tqpk.operators.hashjoin import _outputs
    from tqpk.variable import Variable
    left = {11: Variable(_data(5, 0, torch.int32), "int"), 12: Variable(_data(5, 1, torch.int64), "int")}
    right = {21: Variable(_data(4, 0, torch.int32), "int")}
    bi = torch.tensor([2, NULL, NULL], dtype=torch.int64)
    pi = torch.tensor([1, 0, 3], dtype=torch.int64)
    with pytest.raises(RuntimeError):              # [5, 1] build column, K = 3
        _outputs(left, right, [11, 12, 21], "right-outer", bi, pi)
    o11, o21 = _outputs({11: left[11]}, right, [11, 21], "right-outer", bi, pi)
    assert o11.tolist() == [3, NULL, NULL] and o21.tolist() == [2, 1, 4]
    o11, o12, o21 = _outputs(left, right, [11, 12, 21], "right-outer", bi[:1], pi[:1])
    assert o11.tolist() == [3] and o12.tolist() == [[3]] and o21.tolist() == [2]
    # no matched pair: the build side's columns come out empty (hashjoin.py:154)
    o11, o21 = _outputs({11: left[11]}, right, [11, 21], "right-outer", bi[1:], pi[1:])
    assert o11.numel() == 0 and o21.tolist() == [1, 4]
