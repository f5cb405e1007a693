"""Loader for the golden fixtures written by tests/golden/make_golden.py."""
import glob
import json
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names(zero_gradient=True):
    """Step fixtures (make_golden.py); the io_* fixtures hold output formats.
    zero_gradient=False leaves out the cases with zero_gradient edges (the AA
    layout and the adjoint refuse them)."""
    names = sorted(os.path.splitext(os.path.basename(p))[0]
                   for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz"))
                   if not os.path.basename(p).startswith("io_"))
    if not zero_gradient:
        names = [n for n in names if not n.startswith("zero_gradient")]
    return names


def load_golden(name):
    """Returns (case dictionaries, npz data).  ``array`` initial fields in the
    case JSON are re-attached from the fixture."""
    data = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    case = json.loads(str(data["case_json"]))
    for region, rd in case["initial_fields_dict"].items():
        for fname, spec in rd["fluid"].items():
            if spec["type"] == "array":
                spec["value"] = data[f"init_{region}_{fname}"]
    return case, data
