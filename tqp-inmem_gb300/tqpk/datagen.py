"""Seeded synthetic tables with the shapes of the benchmark workloads.

TPC-H data is not available here; these generators stand in for it with the
cardinalities and value distributions of the lineitem/orders-style columns
the workloads use (numpy PCG64, so x86 and Arm produce identical bytes).

* lineitem(n):   ship_date int32 U[0,2557) days, quantity f64 integers 1-50,
                 price f64 900.00-104,950.00 (2 decimals), discount f64
                 0.00-0.10, tax f64 0.00-0.08, flag uint8 {0,1,2}, status uint8 {0,1}.
* join_tables(b, p): build key = permutation of 1..b (int32) + date;
                 probe fk uniform over 1..b (int32) + date + price + discount.
* star_tables(f, a, b, c): fact fkA/fkB + price/discount; dim A (key, uint8
                 category 1-5), dim B (key, fkC), dim C (key).
"""
from __future__ import annotations

from typing import Dict

import numpy as np

DAYS = 2557


def lineitem(n: int, seed: int = 42) -> Dict[str, np.ndarray]:
    rng = np.random.default_rng(seed)
    return {
        "quantity": rng.integers(1, 51, n).astype(np.float64),
        "price": rng.integers(90000, 10495001, n).astype(np.float64) / 100.0,
        "discount": rng.integers(0, 11, n).astype(np.float64) / 100.0,
        "tax": rng.integers(0, 9, n).astype(np.float64) / 100.0,
        "flag": rng.integers(0, 3, n).astype(np.uint8),
        "status": rng.integers(0, 2, n).astype(np.uint8),
        "ship_date": rng.integers(0, DAYS, n).astype(np.int32),
    }


def join_tables(nb: int, np_: int, seed: int = 7) -> Dict[str, np.ndarray]:
    rng = np.random.default_rng(seed)
    return {
        "b_key": (rng.permutation(nb) + 1).astype(np.int32),
        "b_date": rng.integers(0, DAYS, nb).astype(np.int32),
        "p_fk": rng.integers(1, nb + 1, np_).astype(np.int32),
        "p_date": rng.integers(0, DAYS, np_).astype(np.int32),
        "p_price": rng.integers(90000, 10495001, np_).astype(np.float64) / 100.0,
        "p_discount": rng.integers(0, 11, np_).astype(np.float64) / 100.0,
    }


def star_tables(nf: int, na: int, nb: int, nc: int, seed: int = 11) -> Dict[str, np.ndarray]:
    rng = np.random.default_rng(seed)
    return {
        "f_fka": rng.integers(1, na + 1, nf).astype(np.int32),
        "f_fkb": rng.integers(1, nb + 1, nf).astype(np.int32),
        "f_price": rng.integers(90000, 10495001, nf).astype(np.float64) / 100.0,
        "f_discount": rng.integers(0, 11, nf).astype(np.float64) / 100.0,
        "a_key": (rng.permutation(na) + 1).astype(np.int32),
        "a_cat": rng.integers(1, 6, na).astype(np.uint8),
        "b_key": (rng.permutation(nb) + 1).astype(np.int32),
        "b_fkc": rng.integers(1, nc + 1, nb).astype(np.int32),
        "c_key": (rng.permutation(nc) + 1).astype(np.int32),
    }


# Filter constants of the workloads (days since 1990-01-01).
SHIP_DATE_MAX = 2470      # lineitem: ship_date <= 2470 (~97% pass)
BUILD_DATE_LT = 1170      # join build: date < 1170 (~45%)
PROBE_DATE_GT = 1170      # join probe: date > 1170 (~54%)
STAR_CATEGORY = 1         # star: dim A category == 1 (~20%)


def batch_specs(n_instances: int = 64, seed: int = 0, rows=(10_000, 10_000_000), card=(4, 1_000_000)):
    """Uneven instance shapes: half filter+group-by, half join+aggregate+top-10;
    rows and group cardinality log-uniform over the given ranges."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_instances):
        n = int(np.exp(rng.uniform(np.log(rows[0]), np.log(rows[1]))))
        g = int(np.exp(rng.uniform(np.log(card[0]), np.log(card[1]))))
        specs.append({"kind": "groupby" if i % 2 == 0 else "join", "rows": n, "groups": max(1, g), "seed": seed * 1000 + i})
    return specs


def groupby_instance_tables(rows: int, groups: int, seed: int):
    """lineitem-like table whose (flag, status) key domain has about `groups` tuples."""
    t = lineitem(rows, seed)
    a = int(np.ceil(np.sqrt(groups)))
    b = int(np.ceil(groups / a))
    rng = np.random.default_rng(seed + 1)
    kd = np.uint8 if max(a, b) <= 255 else np.int32
    t["flag"] = rng.integers(0, a, rows).astype(kd)
    t["status"] = rng.integers(0, b, rows).astype(kd)
    return t, (a, b)
