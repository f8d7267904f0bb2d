"""Loading helpers for tests/golden/*.npz (written by tests/golden/make_golden.py)."""
import json
from pathlib import Path

import numpy as np

GOLD = Path(__file__).resolve().parent / "golden"


def load(name):
    z = np.load(GOLD / f"{name}.npz", allow_pickle=False)
    ins = {int(k[3:]) if k[3:].isdigit() else k[3:]: z[k] for k in z.files if k.startswith("in_")}
    outs = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    return ins, outs, json.loads(str(z["args"]))


def assert_f64_close(a, b, rel=1e-12, magnitude=None):
    """|a - b| <= rel * max(|a|, |b|), or rel * magnitude where given: for sums with
    cancellation the error bound of any summation order scales with sum(|x|), so
    tests pass that per element (the sum of absolute values of the summed terms)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    same_nan = np.isnan(a) & np.isnan(b)
    scale = np.maximum(np.abs(a), np.abs(b))
    if magnitude is not None:
        scale = np.maximum(scale, np.asarray(magnitude, np.float64))
    ok = (np.abs(a - b) <= rel * scale) | same_nan | (a == b)
    assert np.all(ok), (a[~ok][:5], b[~ok][:5])


def rows_sorted(*cols):
    m = np.stack([np.asarray(c).reshape(-1).astype(np.float64) for c in cols], 1)
    return m[np.lexsort(m.T[::-1])] if m.size else m


def key_tuple_order(keys):
    """Row order of groups by key tuple ascending: each key compared by value, a 2-D
    (string) key byte column by byte column, the first key most significant."""
    cols = []
    for k in keys:
        k = np.asarray(k)
        k2 = k.reshape(k.shape[0], -1)
        cols.extend(k2[:, j] for j in range(k2.shape[1]))
    return np.lexsort(cols[::-1])
