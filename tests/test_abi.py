"""CPU tests of the C ABI boundary: libspgpu.so builds for sm_103a, loads,
exports every entry point declared in include/spgpu.h, its structures match
the ctypes mirror byte for byte, and argument errors are reported before any
device call."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from spatialpy_gb300 import abi
from spatialpy_gb300 import scenario as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "spgpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sp_[a-z_0-9]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(spgpu_lib):
    names = declared_functions()
    assert set(names) == set(abi.EXPORTED_SYMBOLS), names
    out = subprocess.run(["nm", "-D", "--defined-only", abi.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r"\bT (sp_[a-z_0-9]+)", out))
    for n in names:
        assert n in exported, n
        assert hasattr(spgpu_lib, n)
    assert spgpu_lib.sp_abi_version() == abi.ABI_VERSION


STRUCTS = {"sp_scenario": abi.SpScenario, "sp_options": abi.SpOptions,
           "sp_run_args": abi.SpRunArgs, "sp_outputs": abi.SpOutputs,
           "sp_traj_status": abi.SpTrajStatus, "sp_profile": abi.SpProfile,
           "sp_fno_shape": abi.SpFnoShape}


def test_struct_layout_matches_header(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"',
             "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", str(src), "-o", str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines():
        cname, field, val = ln.split()
        got[(cname, field)] = int(val)
    for cname, py in STRUCTS.items():
        assert got[(cname, "sizeof")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def _create(lib, sc):
    s = (abi.SpScenario * 1)()
    s[0] = abi.scenario_struct(sc)
    h = C.c_void_p()
    rc = lib.sp_create(s, 1, None, C.byref(h))
    msg = lib.sp_last_error(h).decode()
    lib.sp_destroy(h)
    return rc, msg


@pytest.mark.parametrize("mutate,needle", [
    (lambda sc: sc.type.__setitem__(0, 5), "type"),
    (lambda sc: setattr(sc, "h", 0.0), "h (basis function width)"),
    (lambda sc: sc.rho.__setitem__(3, 0.0), "Rho"),
    (lambda sc: sc.output_steps.__setitem__(1, 0), "output steps"),
    (lambda sc: sc.rxn_reactants.__setitem__((1, 0), 7), "reactant"),
])
def test_argument_errors_before_device_calls(spgpu_lib, mutate, needle):
    sc = S.config_birth_death_2d()
    mutate(sc)
    rc, msg = _create(spgpu_lib, sc)
    assert rc == abi.SP_E_INVALID
    assert needle in msg


def test_null_arguments(spgpu_lib):
    h = C.c_void_p()
    assert spgpu_lib.sp_create(None, 1, None, C.byref(h)) == abi.SP_E_INVALID
    assert spgpu_lib.sp_run(None, None, None) == abi.SP_E_INVALID
    assert spgpu_lib.sp_status(None, 0, None) == abi.SP_E_INVALID
    spgpu_lib.sp_destroy(None)


def test_fno_shape_checks_before_device_calls(spgpu_lib):
    """sp_fno_create rejects shapes outside its limits without touching a GPU."""
    good = dict(n=32, width=32, modes=12, layers=4, in_ch=6, out_ch=6, cond=6, hidden=64,
                max_batch=64)
    h = C.c_void_p()
    assert spgpu_lib.sp_fno_create(None, C.byref(h)) == abi.SP_E_INVALID
    for field, bad in [("n", 3), ("n", 65), ("modes", 17), ("modes", 0), ("width", 65),
                       ("layers", 0), ("hidden", 65), ("max_batch", 0), ("in_ch", 17)]:
        sh = abi.SpFnoShape(**{**good, field: bad})
        assert spgpu_lib.sp_fno_create(C.byref(sh), C.byref(h)) == abi.SP_E_INVALID, field
        assert not h.value
    assert spgpu_lib.sp_fno_num_params(None) == -1
    spgpu_lib.sp_fno_destroy(None)


def test_fno_create_without_a_device_fails_cleanly(spgpu_lib):
    """A valid shape on a machine without a CUDA device: an error code, no handle."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    sh = abi.SpFnoShape(n=16, width=8, modes=4, layers=2, in_ch=3, out_ch=2, cond=3, hidden=16,
                        max_batch=4)
    h = C.c_void_p()
    assert spgpu_lib.sp_fno_create(C.byref(sh), C.byref(h)) == abi.SP_E_CUDA
    assert not h.value
    from spatialpy_gb300 import fno
    with pytest.raises(fno.FnoError):
        fno.FnoNet(fno.FnoShape(n=16, width=8, modes=4, layers=2, in_ch=3, out_ch=2, cond=3,
                                hidden=16, max_batch=4))


def test_noalloc_rejects_bad_sizes_before_device_work(spgpu_lib):
    """sp_neighbors_noalloc checks every size before it touches the device
    (these calls run without a GPU): too many particles, a box of more cells
    than its static scratch holds (including one whose cell count overflows
    an int), an inverted or non-finite box, a non-finite h, kmax above 256."""
    err = C.create_string_buffer(256)
    dummy = C.c_void_p(16)

    def box(*v):
        return (C.c_double * 3)(*v)

    def call(n, h, lo, hi, kmax=32):
        return spgpu_lib.sp_neighbors_noalloc(dummy, n, 3, h, dummy, dummy, lo, hi, kmax, dummy,
                                              dummy, None, None, None, None, err, len(err))

    assert call(262145, 0.1, box(0, 0, 0), box(1, 1, 1)) == abi.SP_E_INVALID
    assert b"262,144" in err.value
    assert call(1000, 1e-3, box(0, 0, 0), box(1, 1, 1)) == abi.SP_E_INVALID
    assert b"524,288" in err.value
    assert call(1000, 1.0, box(0, 0, 0), box(1e12, 1, 1)) == abi.SP_E_INVALID
    assert b"524,288" in err.value
    assert call(1000, 1.0, box(0, 0, 0), box(3e9, 3e9, 3e9)) == abi.SP_E_INVALID
    assert call(1000, 1.0, box(0, 0, 0), box(float("inf"), 1, 1)) == abi.SP_E_INVALID
    assert b"finite" in err.value
    assert call(1000, 1.0, box(0, 0, 0), box(float("nan"), 1, 1)) == abi.SP_E_INVALID
    assert call(1000, 1.0, box(0, 2, 0), box(1, 1, 1)) == abi.SP_E_INVALID
    assert b"hi < lo" in err.value
    assert call(1000, float("inf"), box(0, 0, 0), box(1, 1, 1)) == abi.SP_E_INVALID
    assert call(1000, 0.1, box(0, 0, 0), box(1, 1, 1), kmax=257) == abi.SP_E_INVALID
    assert b"256" in err.value
