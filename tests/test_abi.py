"""CPU checks of the C-ABI boundary: libfdmgpu.so builds for sm_103a, loads,
exports every entry point include/fdmgpu.h declares, and rejects bad
arguments with the documented status codes before touching the GPU."""
import ctypes
import re
from ctypes import byref, c_void_p
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "fdmgpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fdmgpu_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("fdmgpu_lapl_cube_create", "fdmgpu_lapl_cube_solve", "fdmgpu_lapl_cube_solve_device",
                 "fdmgpu_lapl_rect_solve", "fdmgpu_nscube_step", "fdmgpu_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(native):
    from fdm_gb300 import _native
    lib = ctypes.CDLL(str(_native.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding declares exactly the header's functions
    assert sorted(_native.EXPORTED) == declared_functions()


def test_status_codes_without_gpu(native):
    from fdm_gb300 import _native as N
    lib = N.load()
    h = c_void_p()
    # n+1 not a power of two: the reference aborts in verify((1<<n) == N)
    assert lib.fdmgpu_lapl_cube_create(byref(h), N.F64, 0, .1, .1, .1, 3.2, 3.2, 3.2, 32, 31, 31) == N.ESIZE
    assert b"verify" in lib.fdmgpu_last_error()
    assert lib.fdmgpu_lapl_cube_create(byref(h), N.F64, 0, .1, .1, .1, 3.2, 3.2, 3.2, 2047, 31, 31) == N.ESIZE
    assert lib.fdmgpu_lapl_cube_create(byref(h), 7, 0, .1, .1, .1, 3.2, 3.2, 3.2, 31, 31, 31) == N.EINVAL
    # mixed boundary flags are not instantiated by the reference
    assert lib.fdmgpu_lapl_cube_create(byref(h), N.F64, 3, .1, .1, .1, 3.2, 3.2, 3.2, 31, 31, 31) == N.ENOTSUP
    # all periodic: n must be a power of two
    assert lib.fdmgpu_lapl_cube_create(byref(h), N.F64, 7, .1, .1, .1, 3.2, 3.2, 3.2, 31, 32, 32) == N.ESIZE
    assert lib.fdmgpu_lapl_cube_create(None, N.F64, 0, .1, .1, .1, 3.2, 3.2, 3.2, 31, 31, 31) == N.EINVAL
    assert lib.fdmgpu_lapl_cube_create(byref(h), N.F64, 0, -.1, .1, .1, 3.2, 3.2, 3.2, 31, 31, 31) == N.EINVAL
    assert lib.fdmgpu_lapl_rect_create(byref(h), N.F64, 0, .1, .1, 3.2, 3.2, 20, 62) == N.ESIZE
    assert lib.fdmgpu_lapl_rect_create(byref(h), N.F64, 1, .1, .1, 3.2, 3.2, 20, 63) == N.ESIZE
    assert lib.fdmgpu_nscube_create(byref(h), N.F64, 64, 63, -1, -1, -1, 1, 1, 1, 1, 250, .01) == N.ESIZE
    assert lib.fdmgpu_nscube_create(byref(h), 7, 63, 63, -1, -1, -1, 1, 1, 1, 1, 250, .01) == N.EINVAL
    assert lib.fdmgpu_sine_device(N.F64, 12, 1, 1.0, 1, 1, None) == N.ESIZE
    assert lib.fdmgpu_lapl_cube_solve(None, None, None) == N.EINVAL
    assert lib.fdmgpu_lapl_cube_destroy(None) == N.OK


def test_python_errors_carry_status(native):
    from fdm_gb300 import FdmError, LaplCube
    with pytest.raises(FdmError) as e:
        LaplCube(0.1, 0.1, 0.1, 3.2, 3.2, 3.2, 32, 31, 31)
    assert e.value.status == 2


def test_server_stats_struct_layout(tmp_path):
    """ctypes' ServerStats has the C struct's size and field offsets."""
    import shutil
    import subprocess
    from fdm_gb300 import _native as N
    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    names = [n for n, _ in N.ServerStats._fields_]
    src = tmp_path / "layout.c"
    src.write_text("#include <stdio.h>\n#include <stddef.h>\n#include \"fdmgpu.h\"\nint main(void){\n"
                   "printf(\"%zu\\n\", sizeof(fdmgpu_server_stats_t));\n"
                   + "".join("printf(\"%%zu\\n\", offsetof(fdmgpu_server_stats_t, %s));\n" % n for n in names)
                   + "return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert vals[0] == ctypes.sizeof(N.ServerStats)
    assert vals[1:] == [getattr(N.ServerStats, n).offset for n in names]


def test_server_arguments_without_gpu(native):
    from fdm_gb300 import _native as N
    lib = N.load()
    h = c_void_p()
    assert lib.fdmgpu_server_create(byref(h), 0.0, 8, 8) == N.EINVAL
    assert lib.fdmgpu_server_create(byref(h), 1e9, 0, 8) == N.EINVAL
    assert lib.fdmgpu_server_create(byref(h), 1e9, 8, 65) == N.EINVAL
    assert lib.fdmgpu_server_create(None, 1e9, 8, 8) == N.EINVAL
    assert lib.fdmgpu_server_destroy(None) == N.OK
    assert lib.fdmgpu_server_cancel(None, 1) == N.EINVAL
    assert lib.fdmgpu_server_set_admission(None, 0, 0.0) == N.EINVAL


def test_shared_steps_arguments_without_gpu(native):
    from ctypes import c_int
    from fdm_gb300 import FdmError, NSCube
    from fdm_gb300 import _native as N
    lib = N.load()
    assert lib.fdmgpu_nscube_step_many(None, None, 0) == N.EINVAL
    hs = (c_void_p * 2)(None, None)
    ks = (c_int * 2)(1, 1)
    assert lib.fdmgpu_nscube_step_many(hs, ks, 0) == N.EINVAL
    assert lib.fdmgpu_nscube_step_many(hs, ks, 2) == N.EINVAL  # null handles
    with pytest.raises(FdmError) as e:
        NSCube.step_many([], [])
    assert e.value.status == N.EINVAL
