"""The C ABI library builds, loads without a GPU and exports every symbol that
include/gcpm.h declares; the ctypes table matches the header."""

from __future__ import annotations

import ctypes as C
import re

from conftest import ROOT


def _header_functions():
    text = (ROOT / "include" / "gcpm.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(gc_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_builds_and_exports_header_symbols():
    from galaxy_collision_gb300 import _build

    path = _build.build()
    lib = C.CDLL(str(path))
    names = _header_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"symbols declared in gcpm.h but not exported: {missing}"


def test_ctypes_table_matches_header():
    from galaxy_collision_gb300 import _native

    assert sorted(_native.EXPORTED) == _header_functions()


def test_load_without_gpu_and_abi_version():
    from galaxy_collision_gb300 import _build, _native

    _build.build()
    lib = _native.load()
    assert lib.gc_abi_version() == 1
    p = _native.MGParams()
    lib.gc_mg_default_params(C.byref(p))
    # defaults of MultigridPoissonSolver.__init__ (solver/multigrid.py:301-312)
    assert (p.pre_sweeps, p.post_sweeps, p.coarse_sweeps, p.max_cycles, p.min_cycles) == (2, 2, 40, 20, 1)
    assert p.tol == 1e-3


def test_create_reports_bad_arguments_without_gpu():
    from galaxy_collision_gb300 import _native

    lib = _native.load()
    h = C.c_void_p()
    assert lib.gc_ctx_create(C.byref(h), 1, 1.0, 1.0) == _native.GC_ERR_ARG
    assert b"grid_size" in lib.gc_last_error(None)
    assert lib.gc_ctx_create(C.byref(h), 16, -1.0, 1.0) == _native.GC_ERR_ARG
    assert lib.gc_ctx_destroy(None) == 0
