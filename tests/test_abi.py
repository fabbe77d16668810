"""CPU tests of the C ABI boundary: libgbmg.so builds, loads, and exports every
function include/gbmg.h declares; calls that need no GPU behave.  No kernel is
launched here."""
import ctypes as C
import os
import re
import subprocess

import pytest

from fortrancfd_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "gbmg.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbmg_[a-z_0-9]+)\s*\(", text)))


def test_header_declarations_are_the_binding_exports():
    assert header_functions() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    for name in header_functions():
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.library_path()],
                         capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (gbmg_\w+)", out))
    assert set(header_functions()) <= exported


def test_default_params_and_strerror():
    L = _lib.load()
    prm = _lib.Params()
    L.gbmg_default_params(C.byref(prm))
    assert (prm.precision, prm.nu1, prm.nu2, prm.max_cycles, prm.coarse_max) == (0, 2, 2, 100, 64)
    assert prm.use_graph == 1 and prm.remove_rhs_mean == 1 and prm.device == -1
    assert prm.certify == 1 and prm.stream is None
    for code in range(8):
        assert L.gbmg_strerror(code)
    assert L.gbmg_strerror(1).decode().startswith("not converged")


def test_null_and_invalid_arguments_return_codes():
    L = _lib.load()
    h = C.c_void_p()
    assert L.gbmg_create(None, None, C.byref(h)) == _lib.GBMG_INVALID_ARG
    g = _lib.Grid(0, 4, 4, 1.0, 1.0, 1.0)
    assert L.gbmg_create(C.byref(g), None, C.byref(h)) == _lib.GBMG_INVALID_ARG
    assert L.gbmg_destroy(None) == _lib.GBMG_INVALID_ARG
    assert L.gbmg_kernel_launches(None) == 0


@pytest.mark.parametrize("field,value", [
    ("nu1", -1), ("max_cycles", 0), ("coarse_max", 65), ("precision", 7), ("stop_rule", 3),
    ("zero_wall_faces", 2), ("use_graph", 3), ("inner_cycles", 9), ("split_restarts", -1),
    ("split_restarts", 101)])
def test_invalid_parameters_are_rejected_before_any_device_call(field, value):
    """gbmg_create checks its parameters before it asks for a device, so these
    run without a GPU (and give the same code with one)."""
    L = _lib.load()
    prm = _lib.Params()
    L.gbmg_default_params(C.byref(prm))
    setattr(prm, field, value)
    h = C.c_void_p()
    g = _lib.Grid(8, 8, 8, 0.125, 0.125, 0.125)
    assert L.gbmg_create(C.byref(g), C.byref(prm), C.byref(h)) == _lib.GBMG_INVALID_ARG
    assert not h.value


@pytest.mark.parametrize("combo", [
    {"stop_rule": 2, "krylov": 1},          # the increment rule with a Krylov iteration
    {"stop_rule": 2, "inner_cycles": 2},    # ... or with several FP32 cycles per correction
    {"split_restarts": 5, "krylov": 2}])    # the split driver's restarts with a Krylov iteration
def test_invalid_parameter_combinations_are_rejected(combo):
    L = _lib.load()
    prm = _lib.Params()
    L.gbmg_default_params(C.byref(prm))
    for k, v in combo.items():
        setattr(prm, k, v)
    h = C.c_void_p()
    g = _lib.Grid(8, 8, 8, 0.125, 0.125, 0.125)
    assert L.gbmg_create(C.byref(g), C.byref(prm), C.byref(h)) == _lib.GBMG_INVALID_ARG


def test_create_without_device_reports_no_device():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    L = _lib.load()
    h = C.c_void_p()
    g = _lib.Grid(8, 8, 8, 0.125, 0.125, 0.125)
    assert L.gbmg_create(C.byref(g), None, C.byref(h)) == _lib.GBMG_NO_DEVICE
    assert not h.value


def test_fortran_module_binds_every_entry_point():
    text = open(os.path.join(ROOT, "include", "gbmg.f90")).read()
    bound = set(re.findall(r'bind\(c,\s*name="(gbmg_\w+)"\)', text))
    assert bound == set(header_functions())


def test_struct_layouts_match_the_header(tmp_path):
    """sizeof and field offsets of the ABI structs as a C compiler lays them
    out from include/gbmg.h, against the ctypes mirrors."""
    structs = {"gbmg_params": _lib.Params, "gbmg_stats": _lib.Stats, "gbmg_field": _lib.Field,
               "gbmg_ns_params": _lib.NSParams, "gbmg_ns_fields": _lib.NSFields,
               "gbmg_ns_stats": _lib.NSStats}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "gbmg.h"', "int main(void) {"]
    for name, cls in structs.items():
        lines.append(f'  printf("{name} sizeof %zu\\n", sizeof({name}));')
        for f, _ in cls._fields_:
            lines.append(f'  printf("{name} {f} %zu\\n", offsetof({name}, {f}));')
    lines.append("  return 0;\n}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    for line in out.splitlines():
        name, field, val = line.split()
        cls = structs[name]
        want = C.sizeof(cls) if field == "sizeof" else getattr(cls, field).offset
        assert int(val) == want, (name, field)
