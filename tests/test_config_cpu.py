"""Case validation against the reference's own classes: every mutation of a
valid golden case in tests/golden/config_validation.json (made by
tests/golden/make_config_golden.py from the reference's State,
CollisionOperator and ForceOperator) is rejected by pylabolt_gb300's Case
with the message the reference prints after "FATAL ERROR!"."""
import copy
import json
import os

import pytest

from _golden import GOLDEN_DIR, load_golden
from pylabolt_gb300.config import Case

with open(os.path.join(GOLDEN_DIR, "config_validation.json")) as f:
    ENTRIES = json.load(f)

# The reference rejects these through an incidental Python error (its own
# message is the TypeError text); Case rejects them with a message of its own.
INCIDENTAL = {"gravity a scalar": "gravity must be a list (gx, gy) in forcing dict"}


def _apply(case, ops):
    c = copy.deepcopy(case)
    for op in ops:
        node = c
        for k in op[1][:-1]:
            node = node[k]
        if op[0] == "del":
            del node[op[1][-1]]
        else:
            node[op[1][-1]] = copy.deepcopy(op[2])
    return c


def test_fixture_covers_every_section():
    assert len(ENTRIES) >= 60
    assert all(e["reference"] for e in ENTRIES)   # the reference rejects every mutation


@pytest.mark.parametrize("entry", ENTRIES, ids=[e["name"] for e in ENTRIES])
def test_same_message_as_reference(entry):
    case = _apply(load_golden(entry["base"])[0], entry["ops"])
    with pytest.raises(ValueError) as e:
        Case(case)
    want = INCIDENTAL.get(entry["name"], entry["reference"])
    assert str(e.value) == want


def test_unmutated_bases_are_valid():
    for name in {e["base"] for e in ENTRIES}:
        Case(load_golden(name)[0])
