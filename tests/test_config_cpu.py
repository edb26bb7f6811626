"""fdm_gb300.Config against the reference's own Config (src/config.cpp,
compiled into oracle/_ref): INI sections, comments, separators, CRLF line
ends, `--section:key=value` overrides and typed reads with defaults.  CPU
only; skipped where the reference tree was not compiled."""
import pytest

from fdm_gb300 import Config
from oracle.oracle import reference

INI = (
    "# cavity driver settings\n"
    "[ns]\n"
    "nx = 63\n"
    "nz=31 ; trailing comment\n"
    "Re\t250.5\n"
    "dt = 1e-2   # not a comment marker for the value\n"
    "u0 = 1.0x\n"
    "name = cube_run\n"
    "; whole-line comment\n"
    "empty =\n"
    "[plot] ; a section with a comment\n"
    "interval = 100\r\n"
    "vtk = 1\r\n"
    "[solver]\n"
    "datatype = float\n"
    "steps = 12.7\n"
    "bad = abc\n"
    "[ spaced ]\n"
    "k = v\n"
    "[open\n"
    "a = b\n"
)

ARGV = ["--ns:nx=127", "--plot:png=1", "notanoverride", "--nosection=1", "--ns:noequals", "--new:key=7=8"]

QUERIES = [
    ("ns", "nx", 0), ("ns", "nz", 0), ("ns", "Re", 0.0), ("ns", "dt", 0.0), ("ns", "u0", 0.0),
    ("ns", "name", ""), ("ns", "empty", "dflt"), ("ns", "missing", 5), ("ns", "missing", 2.5),
    ("plot", "interval", 0), ("plot", "vtk", 0), ("plot", "png", 0), ("solver", "datatype", "double"),
    ("solver", "steps", 0), ("solver", "steps", 0.0), ("solver", "bad", 3), ("spaced", "k", ""), ("", "k", ""),
    ("op", "a", ""), ("ope", "a", ""), ("space", "k", ""), ("solver", "[", ""), ("new", "key", ""),
    ("nosection", "x", 1), ("missing", "x", 0.125),
]


@pytest.fixture(scope="module")
def ref():
    r = reference()
    if r is None:
        pytest.skip("the compiled reference (oracle/_ref) is not built here")
    return r


def test_config_matches_reference(ref, tmp_path):
    path = tmp_path / "run.ini"
    path.write_bytes(INI.encode())
    c = Config()
    c.open(str(path))
    c.rewrite(["prog"] + ARGV)
    for sec, key, dflt in QUERIES:
        want = ref.config_get(path, ARGV, sec, key, dflt)
        got = c.get(sec, key, dflt)
        assert type(got) is type(want) and got == want, (sec, key, dflt, got, want)


def test_config_missing_file_keeps_overrides(ref, tmp_path):
    path = tmp_path / "absent.ini"
    c = Config()
    c.open(str(path))
    c.rewrite(["prog", "--ns:Re=400"])
    assert c.get("ns", "Re", 250.0) == ref.config_get(path, ["--ns:Re=400"], "ns", "Re", 250.0) == 400.0
    assert c.get("ns", "nx", 31) == ref.config_get(path, [], "ns", "nx", 31) == 31
