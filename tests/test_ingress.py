"""tqp_scan (operators/scan.py:8-54): column files, type mapping, dtype conversion, primary-key
marking; on the CPU path (gpu_enable=False), which needs no GPU."""
import numpy as np
import pytest
import torch


class _Holder(torch.nn.Module):
    def __init__(self, t):
        super().__init__()
        self.p = torch.nn.Parameter(t, requires_grad=False)

    def forward(self):
        return self.p


def _write(path, t):
    torch.jit.script(_Holder(t)).save(str(path))


def _tables(tmp_path, sf=1):
    rng = np.random.default_rng(4)
    n = 1000
    cols = {
        "L_ORDERKEY": torch.from_numpy(np.arange(n, dtype=np.int32)),
        "L_QUANTITY": torch.from_numpy(rng.integers(1, 51, n).astype(np.float32)),
        "L_SHIPDATE": torch.from_numpy(rng.integers(0, 2557, n).astype(np.int64)),
        "L_SHIPMODE": torch.from_numpy(rng.integers(65, 90, (n, 10)).astype(np.uint8)),
        "L_LINENUMBER": torch.from_numpy(rng.integers(1, 8, n).astype(np.int8)),
    }
    for name, t in cols.items():
        _write(tmp_path / f"SF{sf}-tensor-{name}.pth", t)
    schema = {"L_ORDERKEY": "identifier", "L_QUANTITY": "decimal,15,2", "L_SHIPDATE": "date",
              "L_SHIPMODE": "fixed text,10", "L_LINENUMBER": "integer", "PRIMARY_KEY": "L_ORDERKEY"}
    return cols, schema


def test_scan_types_and_conversions(tmp_path):
    from tqpk.operators import tqp_scan
    cols, schema = _tables(tmp_path)
    tg = {}
    args = {"output names": ["l_orderkey", "l_quantity", "l_shipdate", "l_shipmode", "l_linenumber"],
            "output ids": [1, 2, 3, 4, 5]}
    rows = tqp_scan(False, tg, args, {"tensors path": str(tmp_path)}, schema, 1, None)
    assert rows == 1000
    exp = {1: ("int", torch.int64), 2: ("float", torch.float64), 3: ("date", torch.int32),
           4: ("string", torch.int8), 5: ("int", torch.int64)}
    for cid, (tt, dt) in exp.items():
        assert tg[cid].tensor_type == tt and tg[cid].tensor.dtype == dt, cid
    assert tg[1].is_sorted and not tg[2].is_sorted
    np.testing.assert_array_equal(tg[2].tensor.numpy(), cols["L_QUANTITY"].numpy().astype(np.float64))
    np.testing.assert_array_equal(tg[4].tensor.numpy(), cols["L_SHIPMODE"].numpy().astype(np.int8))
    assert tg[4].tensor.shape == (1000, 10)


def test_scan_missing_column_file_raises(tmp_path):
    from tqpk.operators import tqp_scan
    _, schema = _tables(tmp_path)
    with pytest.raises(Exception):
        tqp_scan(False, {}, {"output names": ["l_comment"], "output ids": [9]}, {"tensors path": str(tmp_path)},
                 dict(schema, L_COMMENT="variable text"), 1, None)


def test_scan_matches_the_reference(tmp_path):
    """The drop-in tqp_scan against the reference's own (operators/scan.py, compiled into
    oracle/_ref) on the same column files, both on their CPU path: values, dtypes, type names,
    the primary-key flag and the row count."""
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    if str(root) not in sys.path:
        sys.path.insert(0, str(root))
    from oracle import reference
    ok, why = reference.available()
    if not ok:
        pytest.skip(why)
    R = reference.load()
    from tqpk.operators import tqp_scan
    _, schema = _tables(tmp_path)
    args = {"output names": ["l_orderkey", "l_quantity", "l_shipdate", "l_shipmode", "l_linenumber"],
            "output ids": [1, 2, 3, 4, 5]}
    ref_tg, tg = {}, {}
    with reference.cpu_mode():
        ref_rows = R.scan.tqp_scan(False, ref_tg, dict(args), {"tensors path": str(tmp_path)}, schema, 1, None)
    rows = tqp_scan(False, tg, dict(args), {"tensors path": str(tmp_path)}, schema, 1, None)
    assert rows == ref_rows
    for cid in args["output ids"]:
        e, g = ref_tg[cid], tg[cid]
        assert (g.tensor_type, g.tensor.dtype, tuple(g.tensor.shape)) == (e.tensor_type, e.tensor.dtype,
                                                                          tuple(e.tensor.shape)), cid
        assert bool(g.is_sorted) == bool(e.is_sorted), cid
        assert torch.equal(g.tensor, e.tensor), cid
