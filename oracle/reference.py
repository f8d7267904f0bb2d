"""TQP-Inmem's own operator modules, compiled once and loaded for timing and pinning.

TEST INFRASTRUCTURE ONLY: imported by tests/golden/make_golden.py (to generate the golden
vectors), by bench.py (the reference arm and the reference's torch CUDA path beside the kernels)
and by nothing in the product.

build() compiles the reference's operator path -- ``operators/{filter,like,hashjoin,aggregate,
sort,project,scan}.py``, ``IO/vortex_pipeline.py``, ``IO/pinned_mem.py``, ``variable.py``,
``constants.py``, ``conversion.py``, ``utility/{logger,tensor_utils}.py`` and four functions of
``parsing.py`` -- from a TQP-Inmem source tree into one bundle of code objects,
``oracle/_ref/tqp_inmem.bundle`` (git-ignored; Python's ``marshal`` format, so it is read by the
same Python version only).  The bundle travels with a copy of this repository to a GPU machine,
where the source tree is absent, and load() imports the modules from it through a finder of its
own, unchanged.

Three adaptations make the modules import without pandas, pyspark and pyparsing, and none of them
touches the operators' arithmetic:

1. ``pandas``/``pyspark``/``pyparsing``/``expression`` are stand-in modules.  Only
   ``pd.Timestamp`` is used on the operator path: ``conversion.py`` makes its epoch at import time
   and turns a date literal into days with ``(pd.Timestamp(s) - epoch).days`` (``date_to_float``,
   :26-29).  The stand-in parses an ISO date and gives that day difference, as pandas does for
   two midnight timestamps.
2. ``parsing`` is compiled from the reference's own ``get_id``/``get_name``/``get_literals``/
   ``right_most`` function bodies alone (the rest of that file drives Spark).
3. ``IO/vortex_pipeline.py`` is compiled with assertions off: its two asserts check that the
   input columns are CUDA tensors and that a mask column was passed, and the reference's CPU
   path (``gpu_enable=False``) puts CPU tensors through the same class.

On the CPU, cpu_mode() additionally maps the hard-coded ``device='cuda'`` arguments of
``operators/aggregate.py:100,101,171,320,326`` to the CPU and makes ``torch.cuda.synchronize``
(``operators/sort.py:37``) a no-op, for the duration of a ``with`` block.
"""
from __future__ import annotations

import ast
import contextlib
import importlib.util
import json
import marshal
import os
import sys
import types
from pathlib import Path

OUT = Path(__file__).resolve().parent / "_ref"

# (module path relative to the TQP-Inmem tree, optimisation level)
MODULES = [
    ("constants.py", 0), ("variable.py", 0), ("conversion.py", 0),
    ("utility/__init__.py", 0), ("utility/logger.py", 0), ("utility/tensor_utils.py", 0),
    ("IO/__init__.py", 0), ("IO/vortex_pipeline.py", 1), ("IO/pinned_mem.py", 0),
    ("operators/like.py", 0), ("operators/filter.py", 0), ("operators/hashjoin.py", 0),
    ("operators/aggregate.py", 0), ("operators/sort.py", 0), ("operators/project.py", 0), ("operators/scan.py", 0),
]
PARSING_FUNCTIONS = {"get_id", "get_name", "get_literals", "right_most"}


class ReferenceUnavailable(RuntimeError):
    """The compiled reference modules are missing or were built for another Python."""


BUNDLE = OUT / "tqp_inmem.bundle"


def _module_name(rel: str) -> tuple[str, bool]:
    parts = rel[:-3].split("/")
    if parts[-1] == "__init__":
        return ".".join(parts[:-1]), True
    return ".".join(parts), False


def build(src=None) -> Path | None:
    """Compiles the reference's operator path into oracle/_ref/ when its source tree is present
    (``src``); returns oracle/_ref/, or None when neither the source nor a previous build exists."""
    src = Path(src) if src else None
    if src is None or not (src / "operators" / "aggregate.py").exists():
        return OUT if (OUT / "manifest.json").exists() and BUNDLE.exists() else None
    OUT.mkdir(parents=True, exist_ok=True)
    mods, built = {}, []
    for rel, opt in MODULES:
        code = compile((src / rel).read_text(), f"TQP-Inmem/{rel}", "exec", optimize=opt, dont_inherit=True)
        name, pkg = _module_name(rel)
        mods[name] = (pkg, code)
        built.append(rel)
    mods["operators"] = (True, compile("", "TQP-Inmem/operators", "exec", dont_inherit=True))  # a directory there
    tree = ast.parse((src / "parsing.py").read_text())
    body = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in PARSING_FUNCTIONS]
    imp = ast.parse("import re").body
    mods["parsing"] = (False, compile(ast.Module(body=imp + body, type_ignores=[]), "TQP-Inmem/parsing.py", "exec",
                                      dont_inherit=True))
    built.append("parsing.py (get_id, get_name, get_literals, right_most)")
    BUNDLE.write_bytes(marshal.dumps(mods))
    (OUT / "manifest.json").write_text(json.dumps({"magic": importlib.util.MAGIC_NUMBER.hex(),
                                                   "python": sys.version.split()[0], "modules": built}, indent=1))
    return OUT


class _BundleImporter:
    """Finds and loads the bundle's modules (a meta path finder and loader in one)."""

    def __init__(self, mods):
        self.mods = mods

    def find_spec(self, name, path=None, target=None):
        if name not in self.mods:
            return None
        pkg, _ = self.mods[name]
        spec = importlib.util.spec_from_loader(name, self, origin=f"{BUNDLE}:{name}", is_package=pkg)
        if pkg:
            spec.submodule_search_locations = []
        return spec

    def create_module(self, spec):
        return None

    def exec_module(self, module):
        pkg, code = self.mods[module.__name__]
        module.__file__ = f"{BUNDLE}:{module.__name__}"
        exec(code, module.__dict__)


def _stub(name: str, **attrs) -> types.ModuleType:
    m = sys.modules.get(name)
    if m is None:
        m = types.ModuleType(name)
        sys.modules[name] = m
    for k, v in attrs.items():
        setattr(m, k, v)
    return m


_LOADED = None


def available() -> tuple[bool, str]:
    """(True, '') when load() can import the compiled reference, else (False, why)."""
    man = OUT / "manifest.json"
    if not man.exists() or not BUNDLE.exists():
        return False, "oracle/_ref was not built (the TQP-Inmem source tree was absent when build() ran)"
    magic = json.loads(man.read_text()).get("magic")
    if magic != importlib.util.MAGIC_NUMBER.hex():
        return False, f"oracle/_ref holds bytecode of another Python ({magic})"
    return True, ""


def load() -> types.SimpleNamespace:
    """The reference's modules, imported from oracle/_ref/: filter, hashjoin, aggregate, sort,
    project, scan, variable, pinned_mem."""
    global _LOADED
    if _LOADED is not None:
        return _LOADED
    ok, why = available()
    if not ok:
        raise ReferenceUnavailable(why)

    import datetime

    class _Delta:
        def __init__(self, days):
            self.days = days

    class _Timestamp:                         # ISO dates at midnight: the day difference pandas gives
        def __init__(self, s, *a, **k):
            self.date = datetime.date.fromisoformat(str(s))

        def __sub__(self, other):
            return _Delta((self.date - other.date).days)

    _stub("pandas", Timestamp=_Timestamp, Timedelta=None, DataFrame=None)
    _stub("pyspark")
    _stub("pyspark.sql", SparkSession=None)
    _stub("pyspark.sql.types", StructType=None, DateType=None, StructField=None, IntegerType=None, StringType=None,
          DoubleType=None)
    _stub("pyparsing")
    _stub("expression", parse=None)
    bundle = marshal.loads(BUNDLE.read_bytes())
    sys.meta_path.insert(0, _BundleImporter(bundle))
    import importlib
    mods = {}
    for name in ("constants", "variable", "conversion", "parsing", "utility.logger", "IO.vortex_pipeline",
                 "IO.pinned_mem", "operators.filter", "operators.hashjoin", "operators.aggregate", "operators.sort",
                 "operators.project", "operators.scan"):
        mods[name] = importlib.import_module(name)
    for name, m in mods.items():
        if not isinstance(getattr(m, "__loader__", None), _BundleImporter):
            raise ReferenceUnavailable(f"module {name} resolved outside oracle/_ref ({getattr(m, '__file__', '')})")
    lg = mods["utility.logger"]
    lg.set_perf_logger(None, False)           # as main.py does before running queries
    lg.set_message_logger(None, False)
    _LOADED = types.SimpleNamespace(filter=mods["operators.filter"], hashjoin=mods["operators.hashjoin"],
                                    aggregate=mods["operators.aggregate"], sort=mods["operators.sort"],
                                    project=mods["operators.project"], scan=mods["operators.scan"],
                                    variable=mods["variable"],
                                    pinned_mem=mods["IO.pinned_mem"])
    return _LOADED


class CpuPool:
    """Stands in for IO/pinned_mem.GPUMemory on the CPU path: plain allocations."""

    def malloc_like(self, t):
        import torch
        return 0, torch.empty_like(t)

    def free_all(self):
        pass


@contextlib.contextmanager
def cpu_mode():
    """Runs the reference's CPU path (gpu_enable=False): device='cuda' keyword arguments become
    the CPU and torch.cuda.synchronize is a no-op, inside the block only."""
    import torch
    from torch.overrides import TorchFunctionMode

    class _CudaToCpu(TorchFunctionMode):
        def __torch_function__(self, func, types_, args=(), kwargs=None):
            kwargs = dict(kwargs or {})
            dev = kwargs.get("device")
            if dev is not None and ((isinstance(dev, str) and dev.startswith("cuda"))
                                    or (isinstance(dev, torch.device) and dev.type == "cuda")):
                kwargs["device"] = "cpu"
            return func(*args, **kwargs)

    sync = torch.cuda.synchronize
    torch.cuda.synchronize = lambda *a, **k: None
    try:
        with _CudaToCpu():
            yield
    finally:
        torch.cuda.synchronize = sync
