"""libtqpk.so builds, loads without a GPU and exports every include/tqpk.h symbol."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    from tqpk import build, _lib
    build.build()
    return _lib.load()


def declared_functions():
    text = (ROOT / "include" / "tqpk.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tqpk_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("tqpk_filter_mask", "tqpk_compact", "tqpk_groupby_plan", "tqpk_groupby_run", "tqpk_groupby_emit",
                 "tqpk_argsort_stable", "tqpk_topk_stable", "tqpk_join_plan_build", "tqpk_join_build",
                 "tqpk_join_probe", "tqpk_gather"):
        assert must in names


def test_every_declared_symbol_is_exported(lib):
    raw = ctypes.CDLL(str(Path(lib._name)))
    missing = [n for n in declared_functions() if not hasattr(raw, n)]
    assert not missing, missing


def test_binding_covers_header():
    from tqpk import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES), set(declared_functions()) - set(_lib.SIGNATURES)


def test_struct_layouts_match(lib):
    # load() already compared every ctypes struct size with the library's sizeof()
    from tqpk import _lib
    sizes = (ctypes.c_int64 * 7)()
    assert lib.tqpk_abi_sizes(sizes, 7) == 7
    assert sizes[0] == ctypes.sizeof(_lib.PredInsn) == 40


def test_status_strings(lib):
    from tqpk import _lib
    assert lib.tqpk_status_string(_lib.OK) == b"ok"
    assert lib.tqpk_status_string(_lib.ETIMEOUT) == b"bounded device wait expired"
    with pytest.raises(TimeoutError):
        _lib.check(_lib.ETIMEOUT, "x")
    with pytest.raises(NotImplementedError):
        _lib.check(_lib.EUNSUPPORTED, "x")


def test_invalid_arguments_rejected_without_gpu(lib):
    # argument checks run before any CUDA call
    from tqpk import _lib
    p = _lib.Predicate()
    p.n_insn = 1
    p.n_cols = 0
    p.insn[0] = _lib.PredInsn(_lib.P_CMP, 3, _lib.LE, _lib.DOM_I64, 0, 0.0, 0.0)
    assert lib.tqpk_filter_mask(ctypes.byref(p), 10, 1 << 20, None, None) == _lib.EINVAL
    assert lib.tqpk_filter_mask(None, 10, 1 << 20, None, None) == _lib.EINVAL
    assert lib.tqpk_argsort_stable(1 << 20, 77, 0, None, 10, 1 << 20, 1 << 20, 1 << 30, None) == _lib.EDTYPE
    assert lib.tqpk_gather(1, None, None, None, -1, 0, None, None) == _lib.EINVAL


def test_membership_and_directory_entry_points_check_arguments_without_gpu(lib):
    from tqpk import _lib
    # tqpk_directory_bits: negative slot count, missing buffers
    assert lib.tqpk_directory_bits(None, -1, None, None) == _lib.EINVAL
    assert lib.tqpk_directory_bits(None, 10, 1 << 20, None) == _lib.EINVAL
    assert lib.tqpk_directory_bits(None, 0, None, None) == _lib.OK          # nothing to do
    # tqpk_directory_build_next: the next directory is required
    assert lib.tqpk_directory_build_next(1 << 20, _lib.I32, 10, None, 1 << 20, _lib.I32, 0, 16, -1, -2,
                                         None, 0, 8, 1 << 20, 1 << 20, None) == _lib.EINVAL
    # tqpk_jit_prefer_shared: a kernel handle and a percentage
    assert lib.tqpk_jit_prefer_shared(None, 20) == _lib.EINVAL
    assert lib.tqpk_jit_prefer_shared(1 << 20, 101) == _lib.EINVAL
    assert lib.tqpk_jit_prefer_shared(1 << 20, -1) == _lib.EINVAL


def test_compaction_workspace_and_noalloc_limit_agree(lib):
    # the allocation-free compaction's row limit is the largest input whose workspace (control
    # block + one status word per 4096-row tile) fits its 1 MiB array
    cap = 1 << 20
    rows = lib.tqpk_compact_noalloc_max_rows()
    assert rows > 0 and rows % 4096 == 0
    assert lib.tqpk_compact_workspace_bytes(rows) <= cap
    assert lib.tqpk_compact_workspace_bytes(rows + 4096) > cap
    assert lib.tqpk_compact_workspace_bytes(0) >= 256


def test_compaction_wait_hook_checks_arguments(lib):
    from tqpk import _lib
    assert lib.tqpk_debug_compact_wait(-1, -1) == _lib.EINVAL
    assert lib.tqpk_debug_compact_wait(1 << 22, -1) == _lib.EINVAL
    assert lib.tqpk_debug_compact_wait(16, -2) == _lib.EINVAL
    assert lib.tqpk_debug_compact_wait(1 << 21, -1) == _lib.OK          # the defaults


def test_topk_barrier_hook_checks_arguments(lib):
    from tqpk import _lib
    assert lib.tqpk_debug_topk_barrier(-1, 0) == _lib.EINVAL
    assert lib.tqpk_debug_topk_barrier((1 << 21) + 1, 0) == _lib.EINVAL
    assert lib.tqpk_debug_topk_barrier(100, -1) == _lib.EINVAL
    assert lib.tqpk_debug_topk_barrier(100, 1025) == _lib.EINVAL
    assert lib.tqpk_debug_topk_barrier(1 << 21, 0) == _lib.OK           # the defaults
