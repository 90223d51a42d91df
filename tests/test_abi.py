"""The C-ABI library loads without a GPU and exports every function that
include/bolt_gb300.h declares; the ctypes table covers all of them."""
import ctypes as C
import os
import re

import pytest

from bolt_gb300 import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "bolt_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = set(re.findall(r"\b(bolt_[A-Za-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_header_declares_entry_points():
    names = _declared()
    for n in ("bolt_ctx_create", "bolt_cosmo_build", "bolt_source_grid", "bolt_cl", "bolt_plin",
              "bolt_engine_submit", "bolt_source_grid_static", "bolt_host_tables_frozen"):
        assert n in names


def test_library_exports_every_declared_symbol():
    _build.build()
    lib = C.CDLL(_build.LIB)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_table_matches_header():
    assert set(_lib.EXPORTS) == set(_declared())


def test_debug_symbols_not_in_header_are_absent():
    # phase-cycle counters exist only in builds with BOLT_PHASE_TIMERS
    _build.build()
    lib = C.CDLL(_build.LIB)
    with pytest.raises(AttributeError):
        getattr(lib, "bolt_debug_phase_cycles")
