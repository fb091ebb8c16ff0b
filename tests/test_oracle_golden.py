"""The CPU oracle reproduces every known-answer test of the reference's own test-suite
(test/low_level_morpho/*.cpp, test/geodesy/*.cpp, test/label/*.cpp, test/pixel_processing/compare.cpp),
before it is trusted as the checker."""
import numpy as np
import pytest

import oracle
from tests.kats import OUT_PTYPES, case_id, compare_operands, load_cases, to_array

CASES = load_cases()


def run_oracle(c):
    ins = [to_array(i) for i in c["inputs"]]
    op = c["op"]
    if op in ("dilate_static", "erode_static"):
        return oracle.erode_dilate_static(ins[0], c["se"], 1, op.startswith("dilate"))
    if op in ("dilate_nl", "erode_nl"):
        from poutre2_gb300.se import predefined_offsets
        return oracle.erode_dilate_nl(ins[0], predefined_offsets(c["se"]), op.startswith("dilate"))
    if op in ("dilatex", "erodex", "dilatey", "erodey"):
        return oracle.line(ins[0], c["half"], op[-1], op.startswith("dilate"))
    if op.startswith("reconstruct_"):
        return oracle.reconstruct(ins[0], ins[1], c["se"], op.endswith("dilate"))
    if op in ("h_minima", "h_maxima", "h_convex", "h_concave", "dynamic_pseudo_opening", "dynamic_pseudo_closing"):
        return getattr(oracle, op)(ins[0], c["h"], c["se"])
    if op in ("low_leveling", "high_leveling", "leveling"):
        return getattr(oracle, op)(ins[0], ins[1], c["se"])
    if op in ("label_binary", "label_flat_zones"):
        return oracle.label(ins[0], c["se"], op == "label_flat_zones")[0]
    if op in ("label_minima", "label_maxima"):
        return oracle.label_extrema(ins[0], c["se"], op == "label_maxima")[0]
    if op == "compare":
        return oracle.compare(ins[0], c["cmp"], *compare_operands(c, ins), OUT_PTYPES[c["out_ptype"]])
    raise AssertionError(op)


@pytest.mark.parametrize("case", CASES, ids=[case_id(c) for c in CASES])
def test_oracle_matches_reference_kat(case):
    got = run_oracle(case)
    exp = to_array(case["expected"])
    assert got.dtype == exp.dtype and got.shape == exp.shape
    np.testing.assert_array_equal(got, exp)


def test_kat_count():
    # 20 static + 20 runtime-neighbour-list + 6 line + 4 reconstruction + 6 extrema + 4 leveling
    # + 4 binary labelling + 2 flat-zone labelling + 2 labelled extrema + 48 whole-image compares
    assert len(CASES) == 116


def test_oracle_dilate_y_rejects_non_square():
    # t_DilateY on a non-square image throws in the reference (transpose_op_t.hpp:59).
    with pytest.raises(oracle.OracleError):
        oracle.line(np.zeros((4, 6), np.uint8), 1, "y", True)
