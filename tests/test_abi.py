"""The C-ABI library loads and exports every symbol include/*.h declares.
No compute call is made here; on a machine without a GPU the availability
probe and context creation must fail cleanly with a status, never crash."""
import ctypes as C
import os
import subprocess

from conftest import ROOT


def test_exports_every_declared_symbol(native_lib):
    from bcgx import _lib
    declared = _lib.declared_symbols(os.path.join(ROOT, "include"))
    assert len(declared) >= 20
    L = C.CDLL(_lib.LIB_PATH)
    missing = [n for n in declared if not hasattr(L, n)]
    assert not missing, missing
    bound = {s[0] for s in _lib.SIGNATURES}
    assert set(declared) <= bound, set(declared) - bound
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    assert set(declared) <= exported


def test_probe_without_gpu_is_a_status(native_lib):
    import bcgx
    ok, why = bcgx.gpu_available()
    assert isinstance(why, str) and why
    if not ok:
        try:
            bcgx.Context(0)
        except bcgx.BCError as e:
            assert e.status == 1  # BC_ERR_NO_DEVICE
        else:
            raise AssertionError("context creation must fail without a GB300")


def test_null_arguments_rejected(native_lib):
    import bcgx
    L = bcgx.lib()
    assert L.bc_create(0, None) == 7  # BC_ERR_INVALID_ARG
    assert L.bc_cancel(None) == 7
    assert L.bc_scene_upload(None, None, 0, 0, 0) == 7
    assert L.bc_raycast(None, None, 0, None, None) == 7
    buf = C.create_string_buffer(64)
    assert L.bc_last_error(None, buf, 64) == 0


def test_struct_layouts_match_the_header(native_lib, tmp_path):
    """The ctypes mirrors of the ABI structs have the C compiler's size and field
    offsets (a field added to the header must be added to the mirror)."""
    from bcgx import _lib
    pairs = [("bc_scene_desc", _lib.SceneDesc), ("bc_camera", _lib.CameraC), ("bc_settings", _lib.SettingsC),
             ("bc_view", _lib.ViewC), ("bc_diff_desc", _lib.DiffDescC), ("bc_post_desc", _lib.PostDescC),
             ("bc_tune_report", _lib.TuneReportC), ("bc_timing", _lib.TimingC)]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "bc_gx.h"', "int main(void) {"]
    for cname, py in pairs:
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f in py._fields_:
            lines.append(f'  printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        name, field, value = line.split()
        got[(name, field)] = int(value)
    for cname, py in pairs:
        assert got[(cname, "sizeof")] == C.sizeof(py), cname
        for f in py._fields_:
            assert got[(cname, f[0])] == getattr(py, f[0]).offset, (cname, f[0])
