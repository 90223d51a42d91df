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


_STRUCTS = {"bolt_params": "BoltParams", "bolt_grid": "BoltGrid", "bolt_recfast": "BoltRecfast",
            "bolt_hier": "BoltHier", "bolt_opts": "BoltOpts", "bolt_request": "BoltRequest",
            "bolt_engine_cfg": "BoltEngineCfg"}


def _header_structs():
    src = open(os.path.join(ROOT, "include", "bolt_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for body, name in re.findall(r"typedef struct\s*\{(.*?)\}\s*(bolt_[a-z_]+)\s*;", src, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            m = re.match(r"((?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*?)\s*(\**\s*[A-Za-z_]\w*(?:\s*,\s*\**\s*[A-Za-z_]\w*)*)$",
                         decl)
            assert m, decl
            fields += [v.strip().lstrip("*").strip() for v in m.group(2).split(",")]
        out[name] = fields
    return out


def test_ctypes_structs_match_header_layout(tmp_path):
    """Every struct of the header has a ctypes mirror with the same fields,
    offsets and size (compiled with the host C compiler)."""
    structs = _header_structs()
    assert set(structs) == set(_STRUCTS)
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "bolt_gb300.h"', "int main(void) {"]
    for cname, fields in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in fields:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    (tmp_path / "layout.c").write_text("\n".join(lines))
    import subprocess
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(tmp_path / "layout.c"), "-o", str(exe)],
                   check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        s, f, v = line.split()
        got[(s, f)] = int(v)
    for cname, pyname in _STRUCTS.items():
        py = getattr(_lib, pyname)
        assert [f[0] for f in py._fields_] == structs[cname], cname
        assert C.sizeof(py) == got[(cname, "size")], cname
        for f in structs[cname]:
            assert getattr(py, f).offset == got[(cname, f)], (cname, f)


def test_engine_config_validation_without_gpu():
    """bolt_engine_create rejects an invalid objective or landing stride
    before it touches the device."""
    _build.build()
    lib = _lib.load()
    for bad in ({"objective": 2}, {"objective": -1}, {"land_stride": 65}, {"land_stride": -1}):
        cfg = _lib.BoltEngineCfg(0, 2, 0, 0, 150.0, 0, 0, 0.0, 0, 1)
        for k, v in bad.items():
            setattr(cfg, k, v)
        h = C.c_void_p()
        assert lib.bolt_engine_create(C.byref(cfg), C.byref(h)) == -1, bad
        assert not h.value
