"""CPU-only checks of the C-ABI boundary: the shared library loads without a GPU, exports
every entry point declared in include/hybird_gpu.h, and rejects bad parameters before
touching the device (the reference would exit(); here an error code comes back)."""
import ctypes as C
import os
import re

import pytest

from hybird_gb300 import abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _ensure_built():
    if not os.path.exists(abi.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()


def declared_symbols():
    syms = []
    for hdr in os.listdir(os.path.join(REPO, "include")):
        if hdr.endswith(".h"):
            text = open(os.path.join(REPO, "include", hdr)).read()
            syms += re.findall(r"^\s*(?:int|const char\*|void)\s+\**(hb_\w+)\s*\(", text, re.M)
    return sorted(set(syms))


def test_library_exports_every_declared_symbol():
    _ensure_built()
    lib = C.CDLL(abi.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 15, syms
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_params_struct_matches_header_field_order():
    text = open(os.path.join(REPO, "include", "hybird_gpu.h")).read()
    body = text[text.index("typedef struct hb_params {"):text.index("} hb_params;")]
    fields = re.findall(r"^\s*(?:int32_t|int64_t|double)\s+(\w+)", body, re.M)
    assert fields == [f[0] for f in abi.HbParams._fields_]


@pytest.mark.parametrize("field,value,code", [
    ("boundary", (9, 7, 7, 7, 7, 7), abi.STATUS_NAMES and 2),   # curved walls: unsupported
    ("init_visc", 0.0, 1),
    ("precision", 7, 1),
])
def test_create_rejects_bad_parameters_without_gpu(field, value, code):
    _ensure_built()
    lib = C.CDLL(abi.LIB_PATH)
    lib.hb_last_error.restype = C.c_char_p
    p = abi.make_params((8, 8, 8), (7,) * 6)
    if field == "boundary":
        p.boundary[:] = list(value)
    else:
        setattr(p, field, value)
    h = C.c_void_p()
    rc = lib.hb_create(C.byref(p), C.byref(h))
    assert rc == code, (rc, lib.hb_last_error())
    assert not h.value


def test_checkpoint_load_rejects_a_foreign_file_without_gpu(tmp_path):
    """hb_checkpoint_load validates the header before it builds a context."""
    _ensure_built()
    lib = C.CDLL(abi.LIB_PATH)
    lib.hb_last_error.restype = C.c_char_p
    lib.hb_checkpoint_load.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
    bad = tmp_path / "not_a_checkpoint.bin"
    bad.write_bytes(b"HBCKPT99" + bytes(64))
    h = C.c_void_p()
    assert lib.hb_checkpoint_load(str(bad).encode(), C.byref(h)) == abi.HB_ERR_ARG
    assert not h.value
    assert b"checkpoint" in lib.hb_last_error()
    missing = tmp_path / "missing.bin"
    assert lib.hb_checkpoint_load(str(missing).encode(), C.byref(h)) == abi.HB_ERR_ARG


STRUCTS = [("hb_params", "HbParams"), ("hb_elements", "HbElements"), ("hb_objects", "HbObjects"),
           ("hb_status", "HbStatus"), ("hb_export", "HbExport"), ("hb_cylinders", "HbCylinders"),
           ("hb_adjoint_cfg", "HbAdjointCfg")]


def test_ctypes_mirrors_match_the_c_layout(tmp_path):
    """Every struct of the header and its ctypes mirror: same size, same field offsets
    (a C program built from the header prints them)."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "hybird_gpu.h"', "int main(void) {"]
    for cname, pyname in STRUCTS:
        cls = getattr(abi, pyname)
        lines.append(f'printf("{cname} sizeof() %zu\\n", sizeof({cname}));')
        for f in cls._fields_:
            lines.append(f'printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, pyname in STRUCTS:
        cls = getattr(abi, pyname)
        assert got[(cname, "sizeof()")] == C.sizeof(cls), cname
        for f in cls._fields_:
            assert got[(cname, f[0])] == getattr(cls, f[0]).offset, (cname, f[0])


def test_create_rejects_moving_bounce_back_with_free_surface_without_gpu():
    _ensure_built()
    lib = C.CDLL(abi.LIB_PATH)
    lib.hb_last_error.restype = C.c_char_p
    p = abi.make_params((8, 8, 8), (7,) * 6, free_surface=1, gas_box=(0.4, 0.6), coupling=abi.HB_MOVING_BB)
    h = C.c_void_p()
    assert lib.hb_create(C.byref(p), C.byref(h)) == abi.HB_ERR_UNSUPPORTED
    assert b"moving bounce-back" in lib.hb_last_error()
    p.coupling = 7
    assert lib.hb_create(C.byref(p), C.byref(h)) == abi.HB_ERR_ARG
