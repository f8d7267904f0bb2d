"""compile_aggregate memoises by query shape: a repeated query gets the same program bound to
its own columns, and a change of shape (dtype, results) compiles afresh."""
import copy

import torch

from tqpk.expr import _AGG_MEMO, compile_aggregate

ARGS = {"is partial": False, "keys": ["k#11"], "input ids": [11, 23, 24],
        "results": ["k#11", [[["sum", [["p#23", "*", ["1.0", "-", "d#24"]]]], "#", "301"], "AS", "rev#302"],
                    [[["avg", ["d#24"]], "#", "303"], "AS", "a#304"]],
        "out agg ids": [302, 304]}


def _cols(n, key_dtype=torch.int32):
    return {11: torch.arange(n, dtype=key_dtype).reshape(-1, 1), 23: torch.rand(n, dtype=torch.float64),
            24: torch.rand(n, dtype=torch.float64)}


def _prog_bytes(p):
    s = type(p.spec).from_buffer_copy(p.spec)
    for k in range(s.n_keys):
        s.keys[k] = 0
    for c in range(s.n_cols):
        s.cols[c] = 0
    return bytes(s)


def test_repeated_query_rebinds_its_columns():
    _AGG_MEMO.clear()
    a, b = _cols(100), _cols(50)
    pa = compile_aggregate(copy.deepcopy(ARGS), a, derived=True)
    pb = compile_aggregate(copy.deepcopy(ARGS), b, derived=True)
    assert len(_AGG_MEMO) == 1
    assert _prog_bytes(pa) == _prog_bytes(pb)                  # same program
    assert pb.spec.keys[0] == b[11].data_ptr()                 # [N, 1] key viewed as 1-D, same storage
    assert {pb.spec.cols[i] for i in range(pb.spec.n_cols)} == {b[23].data_ptr(), b[24].data_ptr()}
    assert pa.spec.keys[0] == a[11].data_ptr()                 # the first program keeps its columns
    assert pb.outputs == pa.outputs and pb.key_outputs == pa.key_outputs
    _AGG_MEMO.clear()
    fresh = compile_aggregate(copy.deepcopy(ARGS), b, derived=True)    # compiled, not cached
    assert _prog_bytes(fresh) == _prog_bytes(pb)


def test_changed_shape_compiles_afresh():
    _AGG_MEMO.clear()
    compile_aggregate(copy.deepcopy(ARGS), _cols(10), derived=True)
    p64 = compile_aggregate(copy.deepcopy(ARGS), _cols(10, torch.int64), derived=True)
    assert len(_AGG_MEMO) == 2
    assert p64.spec.key_dtypes[0] != compile_aggregate(copy.deepcopy(ARGS), _cols(10), derived=True).spec.key_dtypes[0]
    other = copy.deepcopy(ARGS)
    other["results"] = other["results"][:2]
    other["out agg ids"] = [302]
    assert len(compile_aggregate(other, _cols(10), derived=True).outputs) == 1
    assert len(_AGG_MEMO) == 3
