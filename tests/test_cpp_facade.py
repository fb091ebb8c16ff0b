"""The C++ facade (include/poutre_gb300/poutre.hpp).

* Standalone: compiles without a GPU; on a GPU it replays every known-answer test of the reference
  through poutre-named C++ calls (tests/cpp/facade_test.cpp).
* Inside poutre2 (POUTRE_GB300_WITH_POUTRE2, tests/cpp/dispatch_test.cpp): compiled against poutre2's own
  headers and linked with poutre2 itself (oracle/_ref), the dispatcher branch forwards a
  poutre::IInterface& that holds a device image to the C ABI and any other image to poutre2's own code;
  the known answers pass through both paths (the host path runs without a GPU)."""
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


def _cases_file(tmp_path):
    """Every known answer as one line: op;se;param;expected;input1[;input2;...]."""
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
    return cases


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
    r = subprocess.run([exe, str(_cases_file(tmp_path))], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "116 cases, 0 failed" in r.stdout


# ----------------------------------------------------------------------------- inside poutre2
DISPATCH = os.path.join(ROOT, "tests", "cpp", "dispatch_test.cpp")
REF = os.path.join(ROOT, "oracle", "_ref")


def _ref_ready():
    from oracle import ref
    return ref.available() and os.path.isdir(os.path.join(REF, "src", "include", "poutre"))


def _compile_dispatch(out):
    from poutre2_gb300 import build
    build.build()
    lib = os.path.join(ROOT, "poutre2_gb300", "_build")
    cmd = ["g++", "-std=c++23", "-O1", "-w", "-DPOUTRE_GB300_WITH_POUTRE2",
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(REF, "src", "include"),
           "-I", os.path.join(ROOT, "oracle", "ref", "shim"), "-I", os.path.join(CUDA, "include"),
           "-include", "cstring", "-include", "mutex", "-include", "cmath", DISPATCH, "-o", out,
           "-L", REF, "-lpoutre_ref", "-L", lib, "-lpoutre_gb300", "-L", os.path.join(CUDA, "lib64"), "-lcudart",
           f"-Wl,-rpath,{REF}", f"-Wl,-rpath,{lib}", f"-Wl,-rpath,{os.path.join(CUDA, 'lib64')}"]
    subprocess.check_call(cmd)


@pytest.mark.skipif(not _ref_ready(), reason="poutre2 (oracle/_ref) not built")
def test_dispatcher_branch_compiles_against_poutre2_and_keeps_its_cpu_path(tmp_path):
    exe = str(tmp_path / "dispatch_test")
    _compile_dispatch(exe)
    r = subprocess.run([exe, "--host-only", str(_cases_file(tmp_path))], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "host 116 cases" in r.stdout


@pytest.mark.gpu
@pytest.mark.skipif(not _ref_ready(), reason="poutre2 (oracle/_ref) not built")
def test_dispatcher_branch_forwards_device_images_to_the_c_abi(tmp_path):
    exe = str(tmp_path / "dispatch_test")
    _compile_dispatch(exe)
    r = subprocess.run([exe, str(_cases_file(tmp_path))], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "host 116 cases, device 116 cases, 0 failed" in r.stdout
