"""The compiled reference (oracle/_ref, oracle/reference.py) on the CPU.

It is what bench.py times as the reference arm and what generated tests/golden/; here it must
import from oracle/_ref alone and reproduce committed golden fixtures exactly."""
import copy
import sys
from pathlib import Path

import numpy as np
import pytest
import torch

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from oracle import reference  # noqa: E402
from golden_io import load  # noqa: E402


@pytest.fixture(scope="module")
def ref():
    ok, why = reference.available()
    if not ok:
        pytest.skip(why)
    return reference.load()


def test_modules_come_from_the_compiled_tree(ref):
    for name in ("filter", "hashjoin", "aggregate", "sort", "project", "scan", "variable", "pinned_mem"):
        assert getattr(ref, name).__file__.startswith(str(reference.BUNDLE))
        assert isinstance(getattr(ref, name).__loader__, reference._BundleImporter)


def test_join_aggregate_topk_reproduces_its_golden_fixture(ref):
    ins, outs, args = load("join_agg_topk_unique")
    V = ref.variable.Variable
    tg = {c: V(torch.from_numpy(np.ascontiguousarray(ins[c])), args["types"][str(c)]) for c in ins}
    pool = reference.CpuPool()
    with reference.cpu_mode():
        for f in args["filters"]:
            ref.filter.tqp_filter(False, tg, copy.deepcopy(f), None, None, pool, "f")
        j = copy.deepcopy(args["join"])
        j["mask map"] = {int(k): v for k, v in j["mask map"].items()}
        ref.hashjoin.join_vortex(False, tg, j, 11, 21, [], "inner", None, pool, "j")
        torch.manual_seed(1)
        ref.aggregate.tqp_hash_aggregate(False, tg, copy.deepcopy(args["aggregate"]), pool, None, "a")
        np.testing.assert_array_equal(tg[11].tensor.numpy(), outs["agg_key"])
        np.testing.assert_array_equal(tg[302].tensor.numpy(), outs["agg_revenue"])
        ref.sort.tqp_sort(False, tg, copy.deepcopy(args["topk"]), True, "t")
    np.testing.assert_array_equal(tg[11].tensor.numpy(), outs["top_key"])
    np.testing.assert_array_equal(tg[302].tensor.numpy(), outs["top_revenue"])


def test_cpu_mode_restores_torch():
    sync = torch.cuda.synchronize
    with reference.cpu_mode():
        assert torch.cuda.synchronize is not sync
        assert torch.zeros(2, device="cuda").device.type == "cpu"
    assert torch.cuda.synchronize is sync
