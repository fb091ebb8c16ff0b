"""The C++ facade (include/poutre_gb300/poutre.hpp): compiles without a GPU; on a GPU it replays
every known-answer test of the reference through poutre-named C++ calls (tests/cpp/facade_test.cpp)."""
import os
import subprocess

import pytest

from tests.kats import load_cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "facade_test.cpp")
CUDA = "/usr/local/cuda"


def _img(d):
    tok = {"uint8": "GUINT8", "int32": "GINT32", "int64": "GINT64", "float32": "F32", "float64": "D64"}[d["dtype"]]
    vals = " ".join(str(v) for v in d["values"])
    return f"Scalar {tok} {len(d['shape'])} " + " ".join(str(s) for s in d["shape"]) + " " + vals


def _compile(out, syntax_only=False):
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"), SRC]
    if syntax_only:
        cmd += ["-fsyntax-only"]
    else:
        lib = os.path.join(ROOT, "poutre2_gb300", "_build")
        cmd += ["-o", out, "-L", lib, "-lpoutre_gb300", "-L", os.path.join(CUDA, "lib64"), "-lcudart",
                f"-Wl,-rpath,{lib}", f"-Wl,-rpath,{os.path.join(CUDA, 'lib64')}"]
    subprocess.check_call(cmd)


def test_facade_compiles():
    _compile(None, syntax_only=True)


@pytest.mark.gpu
def test_facade_replays_reference_kats(tmp_path):
    from poutre2_gb300 import build
    build.build()
    exe = str(tmp_path / "facade_test")
    _compile(exe)
    lines = []
    for c in load_cases():
        if c["op"] == "compare":
            se = c["cmp"]
            param = "|".join(f"#{o['image']}" if "image" in o else str(o["scalar"]) for o in c["operands"])
        else:
            se, param = c.get("se") or "", c.get("half", c.get("h", ""))
        lines.append(";".join([c["op"], se, "" if param is None else str(param), _img(c["expected"])]
                              + [_img(i) for i in c["inputs"]]))
    cases = tmp_path / "cases.txt"
    cases.write_text("\n".join(lines) + "\n")
    r = subprocess.run([exe, str(cases)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "116 cases, 0 failed" in r.stdout
