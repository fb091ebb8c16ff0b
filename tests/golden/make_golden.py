"""Extract the reference's known-answer tests into tests/golden/reference_kats.json.

Reads poutre2's Catch2 test sources *as text* (no reference code is built or run):
every test case there parses its inputs with ``poutre::ImageFromString``, calls one
hot-path (or labelling) entry point and compares ``ImageToString(out)`` with an expected string.
This script records, per case, the source file:line, the entry point, its
structuring element / scalar parameter, the input images and the expected image.

Usage (from the repository root, where the poutre2 tree is available):
    python tests/golden/make_golden.py /root/reference
"""
from __future__ import annotations

import json
import os
import re
import sys

FILES = [
    "test/low_level_morpho/ero_dil_static_se_t.cpp",
    "test/low_level_morpho/ero_dil_runtime_se.cpp",
    "test/low_level_morpho/ero_dil_line_se.cpp",
    "test/geodesy/mreconstruct.cpp",
    "test/geodesy/extrema.cpp",
    "test/geodesy/leveling.cpp",
    "test/label/label_binary.cpp",
    "test/label/label_flat_zones.cpp",
    "test/label/label_extrema.cpp",
]

# image-string tokens -> numpy dtype names (src/base/types.cpp:295-341)
PTYPES = {"GUINT8": "uint8", "GINT32": "int32", "GINT64": "int64", "F32": "float32", "D64": "float64"}

OPS = (
    r"t_DilateX|t_ErodeX|t_DilateY|t_ErodeY|t_Dilate|t_Erode|Reconstruction|h_minima|h_maxima|h_convex|h_concave|"
    r"dynamic_pseudo_opening|dynamic_pseudo_closing|low_leveling|high_leveling|leveling|label_binary|label_flat_zones|"
    r"label_minima|label_maxima"
)

TOKEN = re.compile(
    r'R"\((?P<raw>.*?)\)"'                      # raw string literal
    r'|"(?P<str>(?:[^"\\]|\\.|\\\n)*)"'         # ordinary literal (may hold backslash-newline)
    r"|(?P<op>\b(?:" + OPS + r"))\s*\((?P<args>[^;]*)\)\s*;"
    r"|static_cast<poutre::p\w+>\((?P<const>-?\d+)\)"
    r"|(?P<tc>TEST_CASE)\s*\(",
    re.S,
)


def parse_image(s: str):
    toks = s.replace("\\\n", " ").split()
    assert toks[0] == "Scalar", s
    dtype = PTYPES[toks[1]]
    rank = int(toks[2])
    shape = [int(t) for t in toks[3:3 + rank]]
    vals = toks[3 + rank:]
    n = 1
    for d in shape:
        n *= d
    # ImageFromString reads exactly prod(shape) values and ignores trailing tokens
    # (src/base/image_interface.cpp:407-425); one leveling test relies on that.
    assert len(vals) >= n, (shape, len(vals))
    vals = vals[:n]
    conv = float if dtype.startswith("float") else int
    return {"dtype": dtype, "shape": shape, "values": [conv(v) for v in vals]}


def parse_op(op: str, args: str, const):
    args = " ".join(args.split())
    se = None
    m = re.search(r"Common_NL_SE::(\w+)", args)
    if m:
        se, kind = m.group(1), "static"
    else:
        m = re.search(r"poutre::se::(SE\w+)", args)
        if m:
            se, kind = m.group(1), "nl"
    rec = {"op": op}
    if op in ("t_Dilate", "t_Erode"):
        rec["op"] = ("dilate" if op == "t_Dilate" else "erode") + "_" + kind
        rec["se"] = se
    elif op in ("t_DilateX", "t_ErodeX", "t_DilateY", "t_ErodeY"):
        rec["op"] = op[2:].lower()
        rec["half"] = int(args.split(",")[1])
    elif op == "Reconstruction":
        rec["op"] = "reconstruct_" + ("dilate" if "reconstruction_type::dilate" in args else "erode")
        rec["se"] = se
    elif op in ("h_minima", "h_maxima", "h_convex", "h_concave", "dynamic_pseudo_opening", "dynamic_pseudo_closing"):
        rec["se"] = se
        rec["h"] = const
    else:
        rec["se"] = se
    return rec


def extract(root: str):
    cases = []
    for rel in FILES:
        text = open(os.path.join(root, rel)).read()
        name, inputs, op, const = None, [], None, None
        for m in TOKEN.finditer(text):
            line = text.count("\n", 0, m.start()) + 1
            if m.group("tc"):
                nm = re.match(r'TEST_CASE\s*\(\s*"([^"]*)"', text[m.start():])
                name, inputs, op, const = nm.group(1), [], None, None
            elif m.group("const") is not None:
                const = int(m.group("const"))
            elif m.group("op"):
                op = parse_op(m.group("op"), m.group("args"), const)
                op_line = line
            else:
                s = m.group("raw") if m.group("raw") is not None else m.group("str")
                if not s.lstrip().startswith("Scalar"):
                    continue
                img = parse_image(s)
                if op is None:
                    inputs.append(img)
                else:
                    cases.append({"name": name, "file": rel, "line": op_line, **op, "inputs": inputs,
                                  "expected": img})
                    inputs, op = [], None
    return cases


# poutre2's compare tests (test/pixel_processing/compare.cpp) call the template layer
# (t_CompareImage_xyz / ViewCompare_xyz_func_helper) on images built by ImageFromString, named
# scalars (`const poutre::pINT32 valcomp = 5;`) and literals; x, y, z say whether the comparand,
# the true value and the false value are a scalar (s) or an image (i).  Cases on sections of an
# image are skipped.
COMP_OPS = {"CompOpEqual": "equal", "CompOpDiff": "diff", "CompOpSup": "sup", "CompOpSupEqual": "sup_equal",
            "CompOpInf": "inf", "CompOpInfEqual": "inf_equal"}
COMPARE_FILE = "test/pixel_processing/compare.cpp"


def _string_literal(text: str, start: int):
    m = re.compile(r'"((?:[^"\\]|\\.|\\\n)*)"', re.S).search(text, start)
    return m.group(1), m.end()


def extract_compare(root: str):
    text = open(os.path.join(root, COMPARE_FILE)).read()
    starts = [m.start() for m in re.finditer(r"TEST_CASE\s*\(", text)] + [len(text)]
    cases = []
    for a, b in zip(starts, starts[1:]):
        body = text[a:b]
        name = re.match(r'TEST_CASE\s*\(\s*"([^"]*)"', body).group(1)
        call = re.search(r"(?:t_CompareImage_|ViewCompare_)(?P<form>[si]{3})\w*\((?P<args>[^;]*)\)\s*;", body)
        if call is None or "section" in body:
            continue
        images, alias, scalars = {}, {}, {}
        for m in re.finditer(r"(?:const\s+)?auto\s+(\w+)\s*=\s*poutre::ImageFromString\(", body):
            lit, _ = _string_literal(body, m.end())
            images[m.group(1)] = parse_image(lit)
        for m in re.finditer(r"(?:const\s+)?auto\s*\*?\s*(\w+)\s*=\s*dynamic_cast<[^>]*>\((\w+)\.get\(\)\)", body):
            alias[m.group(1)] = m.group(2)
        for m in re.finditer(r"auto\s+(\w+)\s*=\s*poutre::details::view\(\*?(\w+)\)", body):
            alias[m.group(1)] = m.group(2)
        for m in re.finditer(r"const\s+poutre::p\w+\s+(\w+)\s*=\s*(-?[\d.]+)\s*;", body):
            scalars[m.group(1)] = m.group(2)
        out = re.search(r"image_t<poutre::(p\w+)>\s+imgout", body).group(1)

        def resolve(tok):
            tok = tok.strip().lstrip("*")
            while tok in alias:
                tok = alias[tok]
            return tok

        args = [re.sub(r"//\S*", "", x).strip() for x in call.group("args").split(",")]
        op = COMP_OPS[args[1].split("::")[-1]]
        src = resolve(args[0])
        inputs = [images[src]]
        operands = []
        for kind, tok in zip(call.group("form"), args[2:5]):
            if kind == "s":
                v = scalars.get(tok, tok)
                operands.append({"scalar": float(v) if "." in v else int(v)})
            else:
                inputs.append(images[resolve(tok)])
                operands.append({"image": len(inputs) - 1})
        lit, _ = _string_literal(body, body.index("expected", call.end()))
        cases.append({"name": name, "file": COMPARE_FILE, "line": text.count("\n", 0, a + call.start()) + 1,
                      "op": "compare", "cmp": op, "form": call.group("form"), "operands": operands,
                      "out_ptype": out, "inputs": inputs, "expected": parse_image(lit)})
    return cases


def main():
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <poutre2 source tree>")
    root = sys.argv[1]
    cases = extract(root) + extract_compare(root)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")
    with open(out, "w") as f:
        json.dump({"source": "poutre2 Catch2 tests (test/low_level_morpho, test/geodesy, test/label, test/pixel_processing/compare.cpp)", "cases": cases},
                  f, indent=1)
    print(f"wrote {len(cases)} cases to {out}")


if __name__ == "__main__":
    main()
