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


def case_id(c):
    return f"{os.path.basename(c['file'])}:{c['line']}:{c['name']}"
