"""Fused query pipelines over device-resident columns (no host sync inside).

``JoinAggTopK`` runs the plan main.py executes as Filter(build),
Filter(probe), Join, Aggregate(sum(expr) group by build key), take ordered
(limit k) -- the shape of the filtered equi-join + aggregate + top-10
workload -- as tqpk_pipeline_join_agg_topk: build, probe+aggregate, top-k.
The same trees and argument dicts as the operators are accepted, so a plan
can be routed here when its build key is a primary key (unique); if the
kernel finds a repeated build key it reports it and ``result()`` raises, so
the caller can run the operator path instead.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Optional

import numpy as np
import torch

from . import _lib as L
from .dtypes import code_of
from .expr import compile_aggregate, require_f64_outputs
from .predicate import compile_filter


# The generated probe tests the build side's membership bitmap (1 bit per key; the group slot is
# the key), which the build stage writes directly (stage bit 4), instead of reading its row
# directory, while the bitmap can stay in L1, and then leaves shared memory (no value stage) and
# L1 (value loads that bypass it) to the bitmap.  GB300, 1.5 M build keys (188 KB), 6,001,215
# probe rows: probe 34.9-37.3 us; with the value stage as well 39.4 us; the row directory with
# the value stage 41.0-41.6 us; a 10% / 72% shared-memory split 37.6 / 42.3 us.  Whole step
# (graph replay): 91.3-93.3 us, 93.4-96.4 us with the bitmap made from the row directory by a
# second pass, 95.4-97.4 us with the row directory.
JOIN_DIR_BITS = True
JOIN_BITS_MAX_BYTES = 256 << 10
JOIN_SHARED_PERCENT = None
JOIN_JIT_BUILD = True         # the bitmap build with its predicate compiled in (tqpk.jit.join_build_bits_source)


class JoinAggTopK:
    def __init__(self, build_keys: torch.Tensor, key_min: int, key_max: int, probe_fk: torch.Tensor,
                 build_cols: Dict[int, torch.Tensor], build_filter, probe_cols: Dict[int, torch.Tensor],
                 probe_filter, value_tree, k: int = 10, descending: bool = True):
        self.lib = L.load()
        self.dev = build_keys.device
        self.bk = build_keys.contiguous()
        self.pk = probe_fk.contiguous()
        self.key_min, self.key_max = int(key_min), int(key_max)
        self.bpred = compile_filter(build_filter, build_cols) if build_filter is not None else None
        self.ppred = compile_filter(probe_filter, probe_cols) if probe_filter is not None else None
        prog = compile_aggregate({"keys": None, "results": [[[["sum", value_tree], "#", "1"], "AS", "v#1"]]},
                                 probe_cols)
        self.prog = prog
        require_f64_outputs(prog, "JoinAggTopK")
        self.value_reg = prog.spec.accs[prog.outputs[0][2]].reg
        if not 1 <= k <= 256:
            raise NotImplementedError("the fused top-k handles k <= 256")
        self.k, self.desc = int(k), bool(descending)
        nbytes = self.lib.tqpk_pipeline_join_agg_topk_workspace_bytes(self.key_min, self.key_max)
        self.ws = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=self.dev)
        self.out_keys = torch.empty(self.k, dtype=torch.int64, device=self.dev)
        self.out_vals = torch.empty(self.k, dtype=torch.float64, device=self.dev)
        self.out_count = torch.zeros(1, dtype=torch.int64, device=self.dev)
        self.groups = torch.zeros(1, dtype=torch.int64, device=self.dev)

    @property
    def workspace_bytes(self) -> int:
        return int(self.ws.numel())

    def _stages(self, stages, s):
        L.check(self.lib.tqpk_pipeline_join_agg_topk_stages(
            stages, self.bk.data_ptr() if self.bk.numel() else None, code_of(self.bk.dtype), self.bk.numel(),
            C.byref(self.bpred.struct) if self.bpred else None, self.key_min, self.key_max,
            self.pk.data_ptr() if self.pk.numel() else None, code_of(self.pk.dtype), self.pk.numel(),
            C.byref(self.ppred.struct) if self.ppred else None, C.byref(self.prog.spec), self.value_reg,
            self.k, int(self.desc), self.ws.data_ptr(), self.ws.numel(), self.out_keys.data_ptr(),
            self.out_vals.data_ptr(), self.out_count.data_ptr(), self.groups.data_ptr(), s),
            "tqpk_pipeline_join_agg_topk")

    def _tma_ok(self) -> bool:
        """The TMA-staged probe (TQPK_TMA=1): every staged column 16-byte aligned and at least one
        full chunk.  Off by default: on GB300 the register probe measured 46.7 us against 49.9 us
        (2 stages per warp) and 55.8 us (4 stages) for the 6,001,215-row probe."""
        import os
        from . import jit
        cols = [self.pk] + list(self.prog.tensors) + (list(self.ppred.tensors) if self.ppred else [])
        return (os.environ.get("TQPK_TMA", "0") == "1" and self.pk.numel() >= jit.TMA_ROWS
                and self.pk.dtype in (torch.int32, torch.int64) and all(t.data_ptr() % 16 == 0 for t in cols))

    def _probe_uses_bits(self) -> bool:
        slots = self.key_max - self.key_min + 1
        return bool(JOIN_DIR_BITS and not self._tma_ok() and (slots + 31) // 32 * 4 <= JOIN_BITS_MAX_BYTES)

    def _jit_probe(self, s):
        """The probe + aggregate pass as a query-specialised kernel."""
        from . import jit
        if not hasattr(self, "_probe_handle"):
            pp = self.ppred.struct if self.ppred else None
            self._bits = self._probe_uses_bits()
            self._probe_smem = 0
            if self._tma_ok():
                import os
                src, name, self._probe_smem = jit.join_probe_tma_source(
                    self.prog.spec, self.value_reg, pp, None, code_of(self.pk.dtype),
                    ST=int(os.environ.get("TQPK_TMA_STAGES", "2")))
            else:
                # evict-first probe columns; with the row directory, value columns staged by cp.async
                # (42.3-42.7 -> 41.4 us on the 6,001,215-row probe, this pipeline's timing)
                src, name = jit.join_probe_source(self.prog.spec, self.value_reg, pp, stream_cs=True,
                                                  stage_vals=not self._bits, occ_sentinel=True,
                                                  dir_bits=self._bits)
            self._probe_handle = jit.compile_kernel(src, name)
            if self._bits and JOIN_SHARED_PERCENT is not None:
                L.check(self.lib.tqpk_jit_prefer_shared(self._probe_handle, JOIN_SHARED_PERCENT),
                        "tqpk_jit_prefer_shared")
            d, su, oc = C.c_void_p(), C.c_void_p(), C.c_void_p()
            L.check(self.lib.tqpk_pipeline_join_tables(self.ws.data_ptr(), self.ws.numel(), self.key_min,
                                                       self.key_max, C.byref(d), C.byref(su), C.byref(oc)),
                    "tqpk_pipeline_join_tables")
            self._probe_args = jit.join_probe_args(
                jit._Args(), self.prog.spec, pp, None, self.pk,
                self.pk.numel(), self.key_min, self.key_max - self.key_min + 1, d.value, su.value, oc.value,
                pred_tensors=self.ppred.tensors if self.ppred else (), col_tensors=self.prog.tensors)
            if self._probe_smem:
                self._probe_err = torch.zeros(1, dtype=torch.int32, device=self.dev)
                self._probe_args.ptr(self._probe_err.data_ptr())
                # one warp per 128-row chunk at a time: enough CTAs for every chunk, at most one wave
                self._probe_grid = jit.occupancy_grid(self._probe_handle, 256, self._probe_smem,
                                                      max(1, self.pk.numel() // jit.TMA_ROWS) * 32)
            else:
                self._probe_grid = jit.occupancy_grid(self._probe_handle, 256, 0, jit.probe_units(self.pk.numel()))
        jit.launch(self._probe_handle, self._probe_grid, 256, self._probe_smem, self._probe_args, s,
                   L.KID_PIPE_PROBE)

    def _jit_build(self, s):
        """The membership-bitmap build as a query-specialised kernel (stage bit 5: the library's
        reset stage clears the header and the bitmap, this kernel does the rest)."""
        from . import jit
        if not hasattr(self, "_build_handle"):
            bp = self.bpred.struct if self.bpred else None
            src, name = jit.join_build_bits_source(bp)
            self._build_handle = jit.compile_kernel(src, name)
            d, su, oc = C.c_void_p(), C.c_void_p(), C.c_void_p()
            L.check(self.lib.tqpk_pipeline_join_tables(self.ws.data_ptr(), self.ws.numel(), self.key_min,
                                                       self.key_max, C.byref(d), C.byref(su), C.byref(oc)),
                    "tqpk_pipeline_join_tables")
            er, ps = C.c_void_p(), C.c_void_p()
            L.check(self.lib.tqpk_pipeline_join_words(self.ws.data_ptr(), self.ws.numel(), self.key_min,
                                                      self.key_max, C.byref(er), C.byref(ps)),
                    "tqpk_pipeline_join_words")
            slots = self.key_max - self.key_min + 1
            self._build_args = jit.join_build_bits_args(
                jit._Args(), bp, self.bk, self.bk.numel(), self.key_min, slots, d.value, su.value, ps.value, er.value,
                pred_tensors=self.bpred.tensors if self.bpred else ())
            self._build_grid = jit.occupancy_grid(self._build_handle, 256, 0,
                                                  max((self.bk.numel() + 3) // 4, slots // 2, 1))
        jit.launch(self._build_handle, self._build_grid, 256, 0, self._build_args, s, L.KID_PIPE_BUILD)

    def run(self, stream=None, before_probe=None):
        """Queues the whole query on `stream` (default: the current stream).  before_probe, when
        given, is called between the build stage and the probe (e.g. to make the stream wait for
        probe columns still being copied, so the build overlaps their copies)."""
        from . import jit
        s = (stream or torch.cuda.current_stream(self.dev)).cuda_stream
        from .predicate import has_strings
        if (jit.available() and jit.probe_supported(code_of(self.pk.dtype)) and self.pk.numel() > 0
                and not has_strings(self.ppred.struct if self.ppred else None)):
            sent = 0 if self._tma_ok() else 8      # the generated register probe keeps occupancy in the sums
            bits = 16 if self._probe_uses_bits() else 0   # the build stage writes the membership bitmap
            if bits and JOIN_JIT_BUILD and not has_strings(self.bpred.struct if self.bpred else None):
                self._stages(1 | sent | bits | 32, s)      # reset only; the generated build follows
                self._jit_build(s)
            else:
                self._stages(1 | sent | bits, s)
            if before_probe is not None:
                before_probe()
            self._jit_probe(s)
            self._stages(4 | sent | bits, s)
            self._sentinel = bool(sent)
        else:
            if before_probe is not None:
                before_probe()
            self._stages(7, s)
            self._sentinel = False

    def result_device(self, key_dtype=None):
        """(keys [m], sums float64[m], m) as device tensors after the last run, with one host
        read (the count and the error word together); keys as int64, or cast on the device to
        key_dtype before that read.  The same read brings the k result rows to pinned host
        memory: `result_host` is then (keys, sums) as numpy arrays of m rows.  A repeated build
        key raises NotImplementedError (TQPK_EUNSUPPORTED), an out-of-domain one ValueError."""
        if getattr(self, "_probe_smem", 0):
            self.check_error()                      # the TMA-staged probe keeps its own error word
        keys = self.out_keys if key_dtype in (None, torch.int64) else self.out_keys.to(key_dtype)
        if not hasattr(self, "_hdr_host"):
            self._hdr_host = torch.empty(16, dtype=torch.int32, pin_memory=True)
            self._vals_host = torch.empty(self.k, dtype=torch.float64, pin_memory=True)
        if getattr(self, "_keys_host", None) is None or self._keys_host.dtype != keys.dtype:
            self._keys_host = torch.empty(self.k, dtype=keys.dtype, pin_memory=True)
        hdr = self._hdr_host
        cur = torch.cuda.current_stream(self.dev)
        hdr[:4].copy_(self.ws[:16].view(torch.int32), non_blocking=True)       # hdr[2] = error word
        hdr[4:6].copy_(self.out_count.view(torch.int32), non_blocking=True)
        self._keys_host.copy_(keys, non_blocking=True)
        self._vals_host.copy_(self.out_vals, non_blocking=True)
        cur.synchronize()
        err, m = int(hdr[2]), int(hdr[4:6].view(torch.int64)[0])
        if err:
            L.check(err, "fused join pipeline (repeated or out-of-domain build key)")
        self.result_host = (self._keys_host[:m].numpy().copy(), self._vals_host[:m].numpy().copy())
        return keys[:m], self.out_vals[:m], m


    def capture(self):
        """Records one run (every memset and launch, no host synchronisation inside) in a CUDA
        graph; replay() then re-runs the whole query with one graph launch."""
        self.run()
        torch.cuda.synchronize(self.dev)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.run()
        return self.graph

    def replay(self):
        self.graph.replay()

    def check_error(self, stream=None):
        s = (stream or torch.cuda.current_stream(self.dev)).cuda_stream
        if getattr(self, "_probe_smem", 0):
            e = int(self._probe_err.item())
            if e:
                L.check(e, "TMA-staged probe (a stage wait expired)")
        err = C.c_int(0)
        L.check(self.lib.tqpk_pipeline_error(self.ws.data_ptr(), C.byref(err), s), "tqpk_pipeline_error")
        if err.value:
            L.check(err.value, "fused join pipeline (repeated or out-of-domain build key)")

    def group_table(self):
        """Every group of the last run, not only the top k: (build keys int64[G] ascending,
        sums float64[G]), read from the slot table (synchronises)."""
        self.check_error()
        d, su, oc = C.c_void_p(), C.c_void_p(), C.c_void_p()
        L.check(self.lib.tqpk_pipeline_join_tables(self.ws.data_ptr(), self.ws.numel(), self.key_min, self.key_max,
                                                   C.byref(d), C.byref(su), C.byref(oc)), "tqpk_pipeline_join_tables")
        slots = self.key_max - self.key_min + 1
        base = self.ws.data_ptr()
        sums = self.ws[su.value - base: su.value - base + 8 * slots].view(torch.float64)
        if getattr(self, "_sentinel", False):      # an empty slot keeps the bits of -0.0
            occ = sums.view(torch.int64) != torch.iinfo(torch.int64).min
        else:
            occ = self.ws[oc.value - base: oc.value - base + 4 * slots].view(torch.int32) != 0
        idx = torch.nonzero(occ).reshape(-1)
        return (idx + self.key_min).cpu().numpy(), sums[idx].cpu().numpy()

    def result(self):
        """(keys int64[m], sums float64[m], groups) after the last run (synchronises)."""
        self.check_error()
        m = int(self.out_count.item())
        return (self.out_keys[:m].cpu().numpy(), self.out_vals[:m].cpu().numpy(), int(self.groups.item()))


STAR_A_BITS_MAX_BYTES = 256 << 10
STAR_SHARED_PERCENT = 20


class StarAggTopK:
    """Fact -> A (filtered) -> B -> C star join, sum(expr) and count(*) by the C key, top-k.

    Dimension key domains are table statistics ([min, max] of each primary
    key, computed once when the tables are loaded)."""

    def __init__(self, f_fka, f_fkb, fact_cols: Dict[int, torch.Tensor], fact_filter, value_tree,
                 a_key, a_cols: Dict[int, torch.Tensor], a_filter, a_dom, b_key, b_fkc, b_dom, c_key, c_dom,
                 k: int = 100, descending: bool = True):
        self.lib = L.load()
        self.dev = f_fka.device
        self.t = [x.contiguous() for x in (f_fka, f_fkb, a_key, b_key, b_fkc, c_key)]
        self.fpred = compile_filter(fact_filter, fact_cols) if fact_filter is not None else None
        self.apred = compile_filter(a_filter, a_cols) if a_filter is not None else None
        self.prog = compile_aggregate({"keys": None, "results": [[[["sum", value_tree], "#", "1"], "AS", "v#1"]]},
                                      fact_cols)
        self.value_reg = self.prog.spec.accs[self.prog.outputs[0][2]].reg
        require_f64_outputs(self.prog, "StarAggTopK")
        if not 1 <= k <= 256:
            raise NotImplementedError("the fused top-k handles k <= 256")
        self.k, self.desc = int(k), bool(descending)
        self.doms = [tuple(map(int, d)) for d in (a_dom, b_dom, c_dom)]
        (amn, amx), (bmn, bmx), (cmn, cmx) = self.doms
        nbytes = self.lib.tqpk_pipeline_star_workspace_bytes(amx - amn + 1, bmx - bmn + 1, cmx - cmn + 1)
        self.ws = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=self.dev)
        self.out_keys = torch.empty(self.k, dtype=torch.int64, device=self.dev)
        self.out_vals = torch.empty(self.k, dtype=torch.float64, device=self.dev)
        self.out_cnts = torch.empty(self.k, dtype=torch.int64, device=self.dev)
        self.out_count = torch.zeros(1, dtype=torch.int64, device=self.dev)
        self.groups = torch.zeros(1, dtype=torch.int64, device=self.dev)

    @property
    def workspace_bytes(self) -> int:
        return int(self.ws.numel())

    def _jit_ok(self) -> bool:
        from . import jit
        fa, fb, ak, bk, bc, ck = self.t
        from .predicate import has_strings
        cmn, cmx = self.doms[2]
        if has_strings(self.fpred.struct if self.fpred else None):
            return False
        return (jit.available() and fa.numel() > 0 and fa.dtype == torch.int32 and fb.dtype == torch.int32
                and all(x.numel() > 0 for x in (ak, bk, ck)) and cmn > -(1 << 31) + 1 and cmx < (1 << 31))

    def _jit_setup(self):
        """Tables of the generated-probe path: row directories for A (its filter applied
        at build) and C, the C-key directory for B, the slot table and top-k scratch."""
        from . import jit
        (amn, amx), (bmn, bmx), (cmn, cmx) = self.doms
        if cmn <= -(1 << 31) + 1:
            # B's directory marks "no row" / "no C row" with the two smallest int32 values
            raise NotImplementedError("C keys at the bottom of the int32 range are reserved as directory markers")
        dev = self.dev
        self.dir_a = torch.empty(amx - amn + 1, dtype=torch.int32, device=dev)
        # A's membership bitmap in place of its row directory while it can stay in L1 (the B
        # lookups and value loads bypass L1, and the kernel asks for a 20% shared-memory split).
        # GB300, generated probe: 2 M A keys (250 KB) 424 us against 442 us with the directory,
        # 600 K keys 117 against 140 us; without the L1 bypass 2 M keys took 467 us, and a 0% /
        # 100% shared split 1585 / 889 us.  TQPK_STAR_ABITS=1/0 forces either form.
        import os
        words = (amx - amn + 32) // 32
        force = os.environ.get("TQPK_STAR_ABITS", "auto")
        self._a_bits = force == "1" or (force == "auto" and words * 4 <= STAR_A_BITS_MAX_BYTES)
        self.bits_a = torch.empty(words if self._a_bits else 1, dtype=torch.int32, device=dev)
        self.dir_b = torch.empty(bmx - bmn + 1, dtype=torch.int32, device=dev)
        self.dir_c = torch.empty(cmx - cmn + 1, dtype=torch.int32, device=dev)
        self.sum = torch.empty(cmx - cmn + 1, dtype=torch.float64, device=dev)
        self.cnt = torch.empty(cmx - cmn + 1, dtype=torch.int32, device=dev)
        self.err = torch.zeros(3, dtype=torch.int32, device=dev)
        self.tws = torch.empty(self.lib.tqpk_dense_topk_workspace_bytes(self.k), dtype=torch.uint8, device=dev)
        # fkB loaded with fkA and evict-first column loads: 529 -> 507 us on the 59,986,052-row star join
        # + B's directory composed with C's (no C lookup in the probe)
        src, name = jit.star_probe_source(self.prog.spec, self.value_reg, self.fpred.struct if self.fpred else None,
                                          None, early_fb=True, stream_cs=True, composed=True, a_bits=self._a_bits)
        self._probe = jit.compile_kernel(src, name)
        if self._a_bits:      # the CTAs' 5 KB of queues per CTA; the rest of the SM's storage as L1
            L.check(self.lib.tqpk_jit_prefer_shared(self._probe, STAR_SHARED_PERCENT), "tqpk_jit_prefer_shared")
        fa, fb = self.t[0], self.t[1]
        a = jit._Args()
        if self.fpred:
            for c in range(self.fpred.struct.n_cols):
                a.ptr(self.fpred.struct.cols[c])
        a.blob(jit.pred_lits(self.fpred.struct if self.fpred else None))
        for c in range(self.prog.spec.n_cols):
            a.ptr(self.prog.spec.cols[c])
        for v in (fa.data_ptr(), fb.data_ptr()):
            a.ptr(v)
        a.i64(fa.numel())
        for mn, mx, d in ((amn, amx, self.bits_a if self._a_bits else self.dir_a), (bmn, bmx, self.dir_b),
                          (cmn, cmx, self.dir_c)):
            a.i64(mn)
            a.i64(mx - mn + 1)
            a.ptr(d.data_ptr())
        a.ptr(self.sum.data_ptr())
        a.ptr(self.cnt.data_ptr())
        a.i32(jit._aligned(*self.fpred.tensors) if self.fpred else 1)
        a.i32(jit._aligned(*self.prog.tensors))
        a.i32(jit._aligned(fa, fb))
        self._probe_args = a
        self._probe_grid = jit.occupancy_grid(self._probe, 256, 0, jit.probe_units(fa.numel()))

    def _run_jit(self, s, before_probe=None):
        from . import jit
        if not hasattr(self, "_probe"):
            self._jit_setup()
        fa, fb, ak, bk, bc, ck = self.t
        (amn, amx), (bmn, bmx), (cmn, cmx) = self.doms
        INT_MIN = -(1 << 31)
        build = self.lib.tqpk_directory_build
        ap = C.byref(self.apred.struct) if self.apred else None
        e = self.err.data_ptr()
        L.check(build(ak.data_ptr(), code_of(ak.dtype), ak.numel(), ap, None, 0, amn, amx - amn + 1, -1, -2,
                      self.dir_a.data_ptr(), e, s), "tqpk_directory_build")
        L.check(build(ck.data_ptr(), code_of(ck.dtype), ck.numel(), None, None, 0, cmn, cmx - cmn + 1, -1, -2,
                      self.dir_c.data_ptr(), e + 8, s), "tqpk_directory_build")
        # B's directory of C keys, composed with C's as it is built (a C key without a C row fails)
        L.check(self.lib.tqpk_directory_build_next(
            bk.data_ptr(), code_of(bk.dtype), bk.numel(), None, bc.data_ptr(), code_of(bc.dtype), bmn, bmx - bmn + 1,
            INT_MIN, INT_MIN + 1, self.dir_c.data_ptr(), cmn, cmx - cmn + 1, self.dir_b.data_ptr(), e + 4, s),
            "tqpk_directory_build_next")
        if self._a_bits:
            L.check(self.lib.tqpk_directory_bits(self.dir_a.data_ptr(), self.dir_a.numel(), self.bits_a.data_ptr(), s),
                    "tqpk_directory_bits")
        self.sum.zero_()
        self.cnt.zero_()
        if before_probe is not None:
            before_probe()
        jit.launch(self._probe, self._probe_grid, 256, 0, self._probe_args, s, L.KID_STAR_PROBE)
        L.check(self.lib.tqpk_dense_topk(self.sum.data_ptr(), self.cnt.data_ptr(), self.sum.numel(), cmn, self.k,
                                         int(self.desc), self.tws.data_ptr(), self.tws.numel(),
                                         self.out_keys.data_ptr(), self.out_vals.data_ptr(), self.out_cnts.data_ptr(),
                                         self.out_count.data_ptr(), self.groups.data_ptr(), s), "tqpk_dense_topk")

    def run(self, stream=None, before_probe=None):
        """Queues the query on `stream` (default: the current stream).  before_probe, when given,
        is called after the dimension directories are queued and before the fact probe (e.g. to
        make the stream wait for fact columns still being copied)."""
        s = (stream or torch.cuda.current_stream(self.dev)).cuda_stream
        self._jit_path = self._jit_ok()
        if self._jit_path:
            with torch.cuda.stream(stream or torch.cuda.current_stream(self.dev)):
                self._run_jit(s, before_probe)
            return
        if before_probe is not None:
            before_probe()
        fa, fb, ak, bk, bc, ck = self.t
        (amn, amx), (bmn, bmx), (cmn, cmx) = self.doms
        L.check(self.lib.tqpk_pipeline_star_agg_topk(
            fa.data_ptr(), code_of(fa.dtype), fb.data_ptr(), code_of(fb.dtype), fa.numel(),
            C.byref(self.fpred.struct) if self.fpred else None, C.byref(self.prog.spec), self.value_reg,
            ak.data_ptr(), code_of(ak.dtype), ak.numel(), C.byref(self.apred.struct) if self.apred else None, amn, amx,
            bk.data_ptr(), code_of(bk.dtype), bc.data_ptr(), code_of(bc.dtype), bk.numel(), bmn, bmx,
            ck.data_ptr(), code_of(ck.dtype), ck.numel(), cmn, cmx, self.k, int(self.desc),
            self.ws.data_ptr(), self.ws.numel(), self.out_keys.data_ptr(), self.out_vals.data_ptr(),
            self.out_cnts.data_ptr(), self.out_count.data_ptr(), self.groups.data_ptr(), s),
            "tqpk_pipeline_star_agg_topk")

    def capture(self):
        """Records one run in a CUDA graph (see JoinAggTopK.capture)."""
        self.run()
        torch.cuda.synchronize(self.dev)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.run()
        return self.graph

    def replay(self):
        self.graph.replay()

    def result_device(self):
        """(C keys [m], sums float64[m], counts int64[m], m) as device tensors after the last run,
        with one host read: the error words, the row count and the k result rows together
        (`result_host` then holds the rows as numpy arrays).  A repeated dimension key raises
        NotImplementedError, an out-of-domain one ValueError."""
        cur = torch.cuda.current_stream(self.dev)
        if not hasattr(self, "_hdr_host"):
            self._hdr_host = torch.empty(8, dtype=torch.int64, pin_memory=True)
            self._rows_host = [torch.empty(self.k, dtype=t.dtype, pin_memory=True)
                               for t in (self.out_keys, self.out_vals, self.out_cnts)]
        hdr = self._hdr_host
        if getattr(self, "_jit_path", False):        # the three directory builds' error words
            hdr[:3].copy_(self.err.to(torch.int64), non_blocking=True)
        else:                                         # the library pipeline's error word (header int 2)
            hdr[1:3] = 0
            hdr[:1].copy_(self.ws[8:12].view(torch.int32).to(torch.int64), non_blocking=True)
        hdr[3:4].copy_(self.out_count, non_blocking=True)
        for h, t in zip(self._rows_host, (self.out_keys, self.out_vals, self.out_cnts)):
            h.copy_(t, non_blocking=True)
        cur.synchronize()
        errs = [int(x) for x in hdr[:3].tolist() if x]
        if errs:
            L.check(errs[0], "star pipeline (repeated or out-of-domain dimension key)")
        m = int(hdr[3])
        self.result_host = tuple(h[:m].numpy().copy() for h in self._rows_host)
        return self.out_keys[:m], self.out_vals[:m], self.out_cnts[:m], m

    def group_table(self):
        """Every group of the last run (generated-probe path): (C keys int64[G] ascending,
        sums float64[G], counts int64[G]) (synchronises)."""
        if not getattr(self, "_jit_path", False):
            raise NotImplementedError("the group table is read on the generated-probe path only")
        self.result()                                  # raises on a recorded error
        idx = torch.nonzero(self.cnt != 0).reshape(-1)
        cmn = self.doms[2][0]
        return ((idx + cmn).cpu().numpy(), self.sum[idx].cpu().numpy(), self.cnt[idx].to(torch.int64).cpu().numpy())

    def result(self):
        s = torch.cuda.current_stream(self.dev).cuda_stream
        err = C.c_int(0)
        if getattr(self, "_jit_path", False):
            errs = [int(x) for x in self.err.cpu().tolist() if x]
            err.value = errs[0] if errs else 0
        else:
            L.check(self.lib.tqpk_pipeline_error(self.ws.data_ptr(), C.byref(err), s), "tqpk_pipeline_error")
        if err.value:
            L.check(err.value, "star pipeline (repeated or out-of-domain dimension key)")
        m = int(self.out_count.item())
        return (self.out_keys[:m].cpu().numpy(), self.out_vals[:m].cpu().numpy(),
                self.out_cnts[:m].cpu().numpy(), int(self.groups.item()))


class GroupByPipeline:
    """Filter + group-by whose key domains are known ahead (table statistics), with no
    host synchronisation: the accumulator table is reset, the generated filter +
    accumulation kernel runs, and the occupied groups are counted and written on the
    device (tqpk_groupby_emit_async).  The same groups, in the same key order, as
    tqp_hash_aggregate over the filtered rows; capture()/replay() as a CUDA graph."""

    def __init__(self, args: dict, columns: Dict[int, torch.Tensor], filter_tree, filter_cols: Dict[int, torch.Tensor],
                 key_domains):
        from . import jit
        from .dtypes import dtype_of
        from .predicate import has_strings
        if not jit.available():
            raise NotImplementedError("the group-by pipeline needs the runtime compiler (NVRTC)")
        self.lib = L.load()
        first = next(iter(columns.values()))
        self.dev, self.n = first.device, int(first.shape[0])
        a = dict(args)
        a.pop("mask map", None)
        self.prog = compile_aggregate(a, columns)
        require_f64_outputs(self.prog, "GroupByPipeline")
        self.pred = compile_filter(filter_tree, filter_cols) if filter_tree is not None else None
        if self.pred is not None and has_strings(self.pred.struct):
            raise NotImplementedError("string predicates run on the operator path")
        S = self.prog.spec
        nk = S.n_keys
        kmin = (C.c_int64 * max(nk, 1))(*[int(d[0]) for d in key_domains])
        kmax = (C.c_int64 * max(nk, 1))(*[int(d[1]) for d in key_domains])
        self.plan = L.GbPlan()
        L.check(self.lib.tqpk_groupby_plan_domains(C.byref(S), kmin, kmax, self.n, C.byref(self.plan)),
                "tqpk_groupby_plan_domains")
        if self.plan.mode == L.GB_HASH:
            raise NotImplementedError("a sparse key domain takes the operator path (hash group-by)")
        K = int(self.plan.slots)
        self.ws = torch.empty(max(int(self.plan.ws_bytes), 256), dtype=torch.uint8, device=self.dev)
        self.keys = [torch.empty(K, dtype=dtype_of(S.key_dtypes[k]), device=self.dev) for k in range(nk)]
        self.outs = [torch.empty(K, dtype=dt, device=self.dev) for (_, _, _, _, dt) in self.prog.outputs]
        self.groups = torch.zeros(1, dtype=torch.int64, device=self.dev)
        ops = []
        for (_, op, a_, b_, dt) in self.prog.outputs:
            ops += [op, a_, b_, code_of(dt)]
        self._ops = (C.c_int32 * max(len(ops), 1))(*ops)
        self._kp = (C.c_void_p * max(nk, 1))(*[k.data_ptr() for k in self.keys])
        self._oc = (C.c_void_p * max(len(self.outs), 1))(*[o.data_ptr() for o in self.outs])
        P = self.pred.struct if self.pred is not None else None
        src, name, self.T, self.smem = jit.groupby_source(S, P, self.plan)
        self.kernel = jit.compile_kernel(src, name)
        self.args = jit._Args()
        if P is not None:
            for c in range(P.n_cols):
                self.args.ptr(P.cols[c])
        self.args.blob(jit.pred_lits(P))
        for k in range(nk):
            self.args.ptr(S.keys[k])
        for c in range(S.n_cols):
            self.args.ptr(S.cols[c])
        self.args.i64(self.n)
        self.args.ptr(self.lib.tqpk_groupby_table(self.ws.data_ptr()))
        self.args.i32(jit._aligned(*self.pred.tensors) if self.pred is not None else 1)
        self.args.i32(jit._aligned(*self.prog.tensors[:nk]))
        self.args.i32(jit._aligned(*self.prog.tensors[nk:]))
        self.err = torch.zeros(1, dtype=torch.int32, device=self.dev)    # a key outside its domain
        self.args.ptr(self.err.data_ptr())
        self.grid = jit.occupancy_grid(self.kernel, self.T, self.smem, (self.n + 3) // 4)

    def run(self, stream=None):
        from . import jit
        s = (stream or torch.cuda.current_stream(self.dev)).cuda_stream
        S = self.prog.spec
        L.check(self.lib.tqpk_groupby_prepare(C.byref(S), C.byref(self.plan), self.ws.data_ptr(), self.ws.numel(), s),
                "tqpk_groupby_prepare")
        with torch.cuda.stream(stream or torch.cuda.current_stream(self.dev)):
            self.err.zero_()
        if self.n > 0:
            jit.launch(self.kernel, self.grid, self.T, self.smem, self.args, s, L.KID_GROUPBY)
        L.check(self.lib.tqpk_groupby_emit_async(C.byref(S), C.byref(self.plan), self.ws.data_ptr(), self._kp,
                                                 len(self.outs), self._ops, self._oc, self.groups.data_ptr(), s),
                "tqpk_groupby_emit_async")

    def capture(self):
        self.run()
        torch.cuda.synchronize(self.dev)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.run()
        return self.graph

    def replay(self):
        self.graph.replay()

    def result(self):
        """(key columns [G], {out id: column [G]}, G) after the last run (synchronises).  A key
        outside its declared domain raises ValueError (TQPK_EINVAL)."""
        G = int(self.groups.item())
        if G < 0:
            L.check(G, "group-by emit")
        e = int(self.err.item())
        if e:
            L.check(e, "group-by (a key outside its declared domain)")
        return ([k[:G] for k in self.keys], {oid: o[:G] for (oid, *_), o in zip(self.prog.outputs, self.outs)}, G)
