"""The header-only C++ shims (include/fdm_gb300/*.h) as a reference caller
uses them: a program written against fdm::LaplCube / fdm::NSCube compiles
and links against libfdmgpu.so with only the include and link line changed
(CPU), and gives the reference's answers (GPU)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from tests.helpers import rel_l2

ROOT = Path(__file__).resolve().parents[1]


def _build(tmp_path, native) -> Path:
    if not shutil.which("g++"):
        pytest.skip("g++ not found")
    exe = tmp_path / "shim_solve"
    lib = ROOT / "fdm_gb300"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), str(ROOT / "tests/cpp/shim_solve.cpp"),
                    "-o", str(exe), "-L", str(lib), "-lfdmgpu", "-Wl,-rpath," + str(lib)], check=True)
    return exe


def test_shim_program_compiles_and_links(tmp_path, native):
    exe = _build(tmp_path, native)
    assert exe.exists()


@pytest.mark.gpu
def test_shim_program_matches_reference(tmp_path, native, cuda, golden):
    exe = _build(tmp_path, native)
    g = golden("lapl_cube")
    rhs = g["aniso_rhs"]
    (tmp_path / "rhs").write_bytes(np.ascontiguousarray(rhs).tobytes())
    subprocess.run([str(exe), "dirichlet", "15", "15", "7", *[repr(float(v)) for v in g["aniso_args"]],
                    str(tmp_path / "rhs"), str(tmp_path / "ans")], check=True)
    ans = np.frombuffer((tmp_path / "ans").read_bytes()).reshape(rhs.shape)
    assert rel_l2(ans, g["aniso_ans"]) <= 1e-12
    p = golden("lapl_cube_periodic")
    rhs = p["rhs_a8x16x32"]
    (tmp_path / "prhs").write_bytes(np.ascontiguousarray(rhs).tobytes())
    subprocess.run([str(exe), "periodic", "32", "16", "8", *[repr(float(v)) for v in p["args_a8x16x32"]],
                    str(tmp_path / "prhs"), str(tmp_path / "pans")], check=True)
    ans = np.frombuffer((tmp_path / "pans").read_bytes()).reshape(rhs.shape)
    assert rel_l2(ans, p["ans_a8x16x32"]) <= 1e-12
    ns = golden("ns_cube")
    subprocess.run([str(exe), "nscube", "15", "20", str(tmp_path / "u")], check=True)
    u = np.frombuffer((tmp_path / "u").read_bytes())
    ref = ns["n15_s20_u"]
    assert np.abs(u - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["double", "float"])
def test_shim_cavity_driver_matches_reference(tmp_path, native, cuda, golden, dtype):
    """A caller written like the reference's cavity driver (reads ns.dx,
    ns.u.vec, ns.time_index and ns.u[i][k][j]) compiles against the NSCube
    shim unchanged and gives the reference's fields after 20 steps, for
    NSCube<double> and NSCube<float>."""
    exe = _build(tmp_path, native)
    ns = golden("ns_cube")
    out = subprocess.run([str(exe), "nsdriver", dtype, "15", "20", str(tmp_path / "drv")], check=True,
                         capture_output=True, text=True)
    assert "It took me" in out.stdout
    o = np.frombuffer((tmp_path / "drv").read_bytes())
    assert o[0] == 20 and o[4] == 20  # time_index, steps
    assert o[1] == o[2] == o[3] == 2 * np.pi / 15  # dx = (x2 - x1) / nx
    u = o[6:]
    ref64 = ns["n15_s20_u"]
    assert u.size == ref64.size
    if dtype == "double":
        assert np.abs(u - ref64).max() <= 1e-12 * max(1.0, np.abs(ref64).max())
    else:
        # the float cavity's own criterion (test_ns_cube_gpu.py): within ten
        # times the reference's float-vs-double gap
        ref32 = ns["f32_n15_s20_u"].astype(np.float64)
        gap = np.linalg.norm(ref32 - ref64)
        assert np.linalg.norm(u - ref32) <= 10 * gap + 1e-6 * np.linalg.norm(ref64)
    assert o[5] == u[(16 * 17 + 3) * 18 + 4]  # ns.u[nz+1][3][3]: z 16, y 3, x 3 (x runs from -1, 18 wide)


@pytest.mark.gpu
def test_shim_cylindrical_matches_reference(tmp_path, native, cuda, golden):
    """fdm::LaplCyl3FFT2 and fdm::NSCyl through the C++ shims against the
    reference's own answers (Dirichlet and periodic z)."""
    exe = _build(tmp_path, native)
    g = golden("lapl_cyl")
    for name, pz, shape in (("d16x15x20", 0, (16, 15, 20)), ("p8x16x12", 1, (8, 16, 12))):
        nphi, nz, nr = shape
        rhs = g["rhs_" + name]
        (tmp_path / "crhs").write_bytes(np.ascontiguousarray(rhs).tobytes())
        subprocess.run([str(exe), "cyl", str(pz), str(nr), str(nz), str(nphi),
                        *[repr(float(v)) for v in g["args_" + name]], str(tmp_path / "crhs"),
                        str(tmp_path / "cans")], check=True)
        ans = np.frombuffer((tmp_path / "cans").read_bytes()).reshape(rhs.shape)
        assert rel_l2(ans, g["ans_" + name]) <= 1e-12, name
    for name, pz, (nr, nz, nphi) in (("d16x15x16", 0, (16, 15, 16)), ("p16x16x8", 1, (16, 16, 8))):
        subprocess.run([str(exe), "nscyl", str(pz), str(nr), str(nz), str(nphi), "20", str(tmp_path / "cu")],
                       check=True)
        u = np.frombuffer((tmp_path / "cu").read_bytes())
        ref = g["ns_%s_s20_u" % name]
        assert np.abs(u - ref).max() <= 1e-11 * max(1.0, np.abs(ref).max()), name


def test_dd_conversions_host_build(tmp_path):
    """fdm_gb300/csrc/dd.cuh built for the host with the CUDA intrinsics
    given their IEEE meaning: the integer FP64 <-> float conversions of the
    mixed solver agree with the host's IEEE conversions and FP64 addition over
    the whole exponent range (tests/cpp/dd_host_check.cpp).  The GPU build is
    checked against the device's conversions in test_kernels_gpu.py."""
    if not shutil.which("g++"):
        pytest.skip("g++ not found")
    exe = tmp_path / "dd_host_check"
    subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", str(ROOT / "tests/cpp/dd_host_check.cpp"),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
