"""Loader for the reference known-answer tests (tests/golden/reference_kats.json)."""
import json
import os

import numpy as np

_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_kats.json")


def load_cases():
    with open(_PATH) as f:
        return json.load(f)["cases"]


def to_array(img):
    return np.array(img["values"], dtype=img["dtype"]).reshape(img["shape"])


# poutre pixel-type names of the compare tests' output images -> numpy dtype names
OUT_PTYPES = {"pUINT8": "uint8", "pINT32": "int32", "pINT64": "int64", "pFLOAT": "float32", "pDOUBLE": "float64"}


# compare-case operation names -> poutre::CompOpType values (types.hpp:443-452)
COMP_VALUES = {"equal": 1, "diff": 2, "sup": 4, "sup_equal": 8, "inf": 16, "inf_equal": 32}


def compare_operands(case, ins):
    """The comparand / true / false operands of a compare case: input images or scalars."""
    return [ins[o["image"]] if "image" in o else o["scalar"] for o in case["operands"]]


def case_id(c):
    return f"{os.path.basename(c['file'])}:{c['line']}:{c['name']}"
