"""Generated query kernels compile for sm_103a (NVRTC runs without a GPU) and keep
their launch-bound literals out of the code."""
import numpy as np
import pytest
import torch

from tqpk import _lib as L
from tqpk.expr import compile_aggregate
from tqpk.predicate import compile_filter

jit = pytest.importorskip("tqpk.jit")


@pytest.fixture(scope="module", autouse=True)
def nvrtc():
    from tqpk import build
    build.build()
    if not L.load().tqpk_jit_available():
        pytest.skip("NVRTC is not available")


LINEITEM_AGG = ["flag#5", "status#6",
                [[["sum", ["quantity#1"]], "#", "101"], "AS", "a#201"],
                [[["sum", [["price#2", "*", ["1.0", "-", "discount#3"]]]], "#", "103"], "AS", "c#203"],
                [[["avg", ["discount#3"]], "#", "107"], "AS", "g#207"],
                [[["min", ["price#2"]], "#", "109"], "AS", "m#209"],
                [[["max", ["status#6"]], "#", "110"], "AS", "x#210"],
                [[["count", ["1"]], "#", "108L"], "AS", "h#208"]]


def _lineitem(n=64):
    from tqpk import datagen
    t = datagen.lineitem(n, 1)
    ids = {"quantity": 1, "price": 2, "discount": 3, "tax": 4, "flag": 5, "status": 6, "ship_date": 7}
    return {ids[k]: torch.from_numpy(v) for k, v in t.items()}


def _join_cols(n=64):
    from tqpk import datagen
    return {k: torch.from_numpy(v) for k, v in datagen.join_tables(16, n, 1).items()}


def test_groupby_kernel_compiles_for_each_table_mode():
    d = _lineitem()
    prog = compile_aggregate({"is partial": False, "keys": ["flag#5", "status#6"], "input ids": [1, 2, 3, 5, 6],
                              "results": LINEITEM_AGG, "out agg ids": [201, 203, 207, 209, 210, 208]}, d)
    pred = compile_filter([[["ship_date#7", "<=", "2470"], "AND", ["price#2", ">=", "1000.5"]], "OR",
                           ["discount#3", "=", "0.05"]], {7: d[7], 2: d[2], 3: d[3]})
    for mode in (L.GB_DENSE_PRIVATE, L.GB_DENSE_SHARED, L.GB_DENSE_GLOBAL):
        plan = L.GbPlan()
        plan.mode, plan.threads, plan.slots = mode, 256, 6
        plan.key_stride[0], plan.key_stride[1] = 2, 1
        src, name, T, smem = jit.groupby_source(prog.spec, pred.struct, plan)
        ok, log = jit.check_compiles(src)
        assert ok, log[:2000]
        assert "2470" not in src and "1000.5" not in src    # literals are bound at launch
        assert "atomicCAS(err, 0, -1)" in src                # keys outside the plan's domain
    # float32 registers (an integer column with a Python float, integer true division, CASE with
    # a float literal beside integers) in the generated accumulation and projection kernels
    q = {1: torch.zeros(64, dtype=torch.int64), 2: torch.zeros(64, dtype=torch.int64), 5: d[5]}
    res32 = ["flag#5", [[["sum", [["q#1", "*", "1.5"]]], "#", "1"], "AS", "a#11"],
             [[["max", [["q#1", "/", "d#2"]]], "#", "2"], "AS", "b#12"],
             [[["sum", ["CASE", "WHEN", ["q#1", ">", "25"], "THEN", "1.0", "ELSE", "0", "END"]], "#", "3"], "AS", "c#13"]]
    p32 = compile_aggregate({"is partial": False, "keys": ["flag#5"], "input ids": [1, 2, 5], "results": res32,
                             "out agg ids": [11, 12, 13]}, q, derived=True)
    plan = L.GbPlan()
    plan.mode, plan.threads, plan.slots = L.GB_DENSE_PRIVATE, 256, 3
    plan.key_stride[0] = 1
    src, name, T, smem = jit.groupby_source(p32.spec, None, plan)
    ok, log = jit.check_compiles(src)
    assert ok, log[:2000]
    assert "__fmul_rn" in src and "__fdiv_rn" in src and "__ll2float_rn" in src


def test_probe_kernels_compile_with_and_without_build_filter():
    j = _join_cols()
    pcols = {22: j["p_date"], 23: j["p_price"], 24: j["p_discount"]}
    prog = compile_aggregate({"keys": None, "results": [[[["sum", [["p#23", "*", ["1.0", "-", "d#24"]]]], "#", "1"],
                                                         "AS", "v#1"]]}, pcols)
    vreg = prog.spec.accs[prog.outputs[0][2]].reg
    pp = compile_filter([["pd#22", ">", "1170"]], {22: j["p_date"]})
    bp = compile_filter([["bd#12", "<", "1170"]], {12: j["b_date"]})
    for p, b in ((pp, None), (pp, bp), (None, bp), (None, None)):
        src, _ = jit.join_probe_source(prog.spec, vreg, p.struct if p else None, b.struct if b else None)
        ok, log = jit.check_compiles(src)
        assert ok, log[:2000]
    cat = compile_filter([["cat#32", "=", "1"]], {32: torch.zeros(8, dtype=torch.uint8)})
    for f, a in ((None, cat), (pp, cat), (None, None)):
        src, _ = jit.star_probe_source(prog.spec, vreg, f.struct if f else None, a.struct if a else None)
        ok, log = jit.check_compiles(src)
        assert ok, log[:2000]
    for early, cs in ((True, False), (True, True), (False, True)):
        src, _ = jit.star_probe_source(prog.spec, vreg, pp.struct, cat.struct, early_fb=early, stream_cs=cs)
        ok, log = jit.check_compiles(src)
        assert ok, log[:2000]
        assert ("#define TQPK_LD(p) __ldcs" in src) == cs
    for cs, st in ((True, False), (False, True), (True, True)):
        src, _ = jit.join_probe_source(prog.spec, vreg, pp.struct, None, stream_cs=cs, stage_vals=st)
        ok, log = jit.check_compiles(src)
        assert ok, log[:2000]
        assert ("cp_async16(&q_v" in src) == st
    for b in (bp, None):                     # the fused join's generated bitmap build
        src, name = jit.join_build_bits_source(b.struct if b else None)
        ok, log = jit.check_compiles(src)
        assert ok, log[:2000]
        assert name == "tqpk_q_join_build_bits" and "red.global.or.b32" in src


def test_generated_batch_kernel_compiles_and_record_layout_matches():
    from tqpk import jitbatch as QB
    d = _lineitem()
    prog = compile_aggregate({"is partial": False, "keys": ["flag#5", "status#6"], "input ids": [1, 2, 3, 5, 6],
                              "results": LINEITEM_AGG, "out agg ids": [201, 203, 207, 209, 210, 208]}, d)
    pred = compile_filter([["ship_date#7", "<=", "2470"]], {7: d[7]})
    j = _join_cols()
    pcols = {22: j["p_date"], 23: j["p_price"], 24: j["p_discount"]}
    jprog = compile_aggregate({"keys": None, "results": [[[["sum", [["p#23", "*", ["1.0", "-", "d#24"]]]], "#", "1"],
                                                          "AS", "v#1"]]}, pcols)
    vreg = jprog.spec.accs[jprog.outputs[0][2]].reg
    pp = compile_filter([["pd#22", ">", "1170"]], {22: j["p_date"]})
    bp = compile_filter([["bd#12", "<", "1170"]], {12: j["b_date"]})
    src = QB.batch_source([(prog.spec, pred.struct, prog.outputs), (prog.spec, None, prog.outputs)],
                          [(jprog.spec, vreg, pp.struct, bp.struct), (jprog.spec, vreg, None, None)])
    probe = src + "\nstatic_assert(sizeof(QInst) == %d, \"record size\");\n" % C_sizeof(QB.QInst)
    ok, log = jit.check_compiles(probe)
    assert ok, log[:3000]
    # group keys checked against the instance's domain; global tables updated by reductions; the
    # persistent kernel's 4 CTAs per SM; the result-packing kernel of results_host
    assert ">= (u64)kr0" in src and "set_err(err, -1)" in src and "gred_add(" in src
    assert f"__launch_bounds__(256, {QB.MIN_CTAS}) tqpk_qb_run" in src
    ok, log = jit.check_compiles(QB._PACK_SRC)
    assert ok, log[:2000]


def C_sizeof(t):
    import ctypes
    return ctypes.sizeof(t)


def test_projection_kernel_compiles():
    from tqpk.expr import compile_projection
    d = _lineitem()
    prog = compile_projection([[[["price#2", "*", ["1", "-", "discount#3"]], "AS", "a#11"]],
                               [[["flag#5", "+", "status#6"], "AS", "b#12"]], "quantity#1"], d)
    assert [dt for _, dt in prog.outputs] == [torch.float64, torch.uint8]
    from tqpk.dtypes import code_of
    src, _ = jit.project_source(prog.spec, [(r, code_of(dt)) for r, dt in prog.outputs])
    ok, log = jit.check_compiles(src)
    assert ok, log[:2000]


def test_expression_forms_compile_case_year_and_post_arithmetic():
    """CASE WHEN / conditions / year() / arithmetic over aggregates compile (the golden
    aggregate_expressions trees): conditions become bool mask columns, calls inside a
    result expression become hidden outputs, the generated kernels compile."""
    import json
    from pathlib import Path
    from tqpk.expr import compile_projection
    z = np.load(Path(__file__).parent / "golden" / "aggregate_expressions.npz")
    args = json.loads(str(z["args"]))
    cols = {int(k[3:]): torch.from_numpy(z[k]) for k in z.files if k.startswith("in_")}
    pp = compile_projection(args["project"]["used expr"], cols, derived=True)
    assert [dt for _, dt in pp.outputs] == [torch.int64, torch.float64, torch.float64, torch.bool]
    assert len(pp.masks) == 2
    src, name = jit.project_source(pp.spec, [(r, L.I64 if dt != torch.float64 else L.F64) for r, dt in pp.outputs])
    ok, log = jit.check_compiles(src)
    assert ok, log[:2000]
    cols[20] = torch.from_numpy(z["out_p20"])
    prog = compile_aggregate(args["aggregate"], cols, derived=True)
    assert [(o, dt) for o, _, dt in prog.post] == [(403, torch.float64), (404, torch.float64)]
    assert len({o[0] for o in prog.outputs}) == len(prog.outputs)
    plan = L.GbPlan()
    plan.mode, plan.threads, plan.slots = L.GB_DENSE_SHARED, 256, 30
    plan.key_stride[0], plan.key_stride[1] = 10, 1
    src, name, T, smem = jit.groupby_source(prog.spec, None, plan)
    assert "tqpk_year(" in src and " ? " in src
    ok, log = jit.check_compiles(src)
    assert ok, log[:2000]
    with pytest.raises(NotImplementedError):          # fused pipelines keep to plain calls
        compile_aggregate(args["aggregate"], cols)


def test_fused_sum_of_product_and_kernel_shape_key():
    """A float sum whose value is a product read nowhere else becomes one FMA in the private
    group-by; the generated-kernel memo key ignores pointers and comparison literals but not
    the predicate's shape or the expression constants."""
    d = _lineitem()
    prog = compile_aggregate({"is partial": False, "keys": ["flag#5", "status#6"], "input ids": [1, 2, 3, 4, 5, 6],
                              "results": LINEITEM_AGG, "out agg ids": [201, 203, 207, 209, 210, 208]}, d)
    fused = jit._fusable_products(prog.spec)
    # sum(price * (1 - discount)) is fused; its product is not used by another accumulator
    assert len(fused) == 1
    (a, (x, y)), = fused.items()
    assert prog.spec.expr[prog.spec.accs[a].reg].op == L.X_MUL
    plan = L.GbPlan()
    plan.mode, plan.threads, plan.slots = L.GB_DENSE_PRIVATE, 128, 6
    plan.key_stride[0], plan.key_stride[1] = 2, 1
    src, *_ = jit.groupby_source(prog.spec, None, plan)
    assert src.count("__fma_rn(") == 1
    p1 = compile_filter([["ship_date#7", "<=", "2470"]], {7: d[7]})
    p2 = compile_filter([["ship_date#7", "<=", "100"]], {7: d[7]})
    p3 = compile_filter([["ship_date#7", ">", "2470"]], {7: d[7]})
    k1, k2, k3 = (jit._shape_key(prog.spec, p.struct, plan) for p in (p1, p2, p3))
    assert k1 == k2 and k1 != k3
    d2 = {c: t.clone() for c, t in d.items()}
    prog2 = compile_aggregate({"is partial": False, "keys": ["flag#5", "status#6"], "input ids": [1, 2, 3, 4, 5, 6],
                               "results": LINEITEM_AGG, "out agg ids": [201, 203, 207, 209, 210, 208]}, d2)
    assert jit._shape_key(prog2.spec, p1.struct, plan) == k1          # other column buffers, same kernel
    plan2 = L.GbPlan.from_buffer_copy(plan)
    plan2.n_rows, plan2.ws_bytes = 12345, 999
    assert jit._shape_key(prog.spec, p1.struct, plan2) == k1
    plan2.slots = 7
    assert jit._shape_key(prog.spec, p1.struct, plan2) != k1


def test_wait_ready_without_events_is_a_no_op():
    from tqpk.variable import Variable, wait_ready
    v = Variable(torch.zeros(3), "float")
    assert v.ready is None
    wait_ready(v, None, type("RefVar", (), {"tensor": torch.zeros(1)})())
