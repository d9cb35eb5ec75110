"""Host-side logic of the C++ driver, without a GPU: the reference's known answers for
InputParser::splitString (tests/InputParserTest.cpp) and TimeConverter::convertToEarthDays
(tests/TimeConverterTest.cpp), CSV reading, and the command line's error behaviour."""

import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "n-body-simulation_gb300", "_build")
EXE = os.path.join(BUILD, "nbody_sim")


@pytest.fixture(scope="module")
def host():
    path = os.path.join(BUILD, "libnbody_host.so")
    if not os.path.exists(path):
        pytest.skip("host library not built")
    L = ctypes.CDLL(path)
    L.nbh_split_string.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
    L.nbh_convert_to_earth_days.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)]
    L.nbh_parse_input_count.restype = ctypes.c_longlong
    L.nbh_parse_input_count.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)]
    return L


def split(L, s):
    n = L.nbh_split_string(s.encode(), -1, None, 0)
    out = []
    for k in range(n):
        buf = ctypes.create_string_buffer(256)
        L.nbh_split_string(s.encode(), k, buf, 256)
        out.append(buf.value.decode())
    return out


def test_split_string_known_answers(host, kats):
    tests = kats["InputParserTest.cpp"]
    assert len(tests) == 2
    for t in tests:
        fields = split(host, t["split_inputs"][0])
        for e in t["expects"]:
            if e.get("array") == "result":
                assert fields[e["index"]] == str(e["value"]) if not isinstance(e["value"], str) \
                    else fields[e["index"]] == e["value"]
            else:
                assert e["expr"] == "result.size()" and len(fields) == e["value"]


def test_time_converter_known_answers(host, kats):
    tests = kats["TimeConverterTest.cpp"]
    assert len(tests) == 8
    for t in tests:
        out = ctypes.c_double(0)
        rc = host.nbh_convert_to_earth_days(t["strings"]["input"].encode(), ctypes.byref(out))
        if t["throws"]:
            assert rc == 1, t
        else:
            assert rc == 0
            assert out.value == pytest.approx(t["expects"][0]["value"], rel=1e-7), t


def test_csv_round_trip(host, tmp_path):
    from nbody import generators
    d = generators.heliocentric_disc(50, seed=3)
    p = tmp_path / "bodies.csv"
    generators.write_csv(str(p), d)
    row = (ctypes.c_double * 7)()
    assert host.nbh_parse_input_count(str(p).encode(), row) == 50
    np.testing.assert_array_equal(np.array(row[:]), [d[k][0] for k in ("m", "x", "y", "z", "vx", "vy", "vz")])
    bad = tmp_path / "bad.csv"
    bad.write_text("id,name\n0,a,b,notanumber,1,2,3,4,5,6\n")
    assert host.nbh_parse_input_count(str(bad).encode(), None) == -1


@pytest.mark.parametrize("args,message", [
    (["--algorithm=foo"], "Algorithm must either be <naive> or <BarnesHut>"),
    (["--algorithm=naive", "--opt_stage=3"], "Optimization stage must be 0,1 or 2"),
    (["--algorithm=naive", "--bogus=1"], "unknown option --bogus"),
])
def test_cli_errors(tmp_path, args, message):
    if not os.path.exists(EXE):
        pytest.skip("driver not built")
    from nbody import generators
    p = tmp_path / "b.csv"
    generators.write_csv(str(p), generators.heliocentric_disc(20, seed=1))
    base = [EXE, f"--file={p}", "--dt=1h", "--t_end=1d", "--vs=1d", f"--vs_dir={tmp_path}"]
    r = subprocess.run(base + args, capture_output=True, text=True)
    assert r.returncode == 1 and message in r.stderr, r.stderr
