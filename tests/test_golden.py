"""The oracle against the literal known answers of the reference's own tests
(tests/golden/known_answers.json, extracted by tests/golden/make_golden.py from
test/test_clebsch_gordan.jl)."""

import json
import math
from pathlib import Path

import pytest

import oracle as O

RECORDS = json.loads((Path(__file__).parent / "golden" / "known_answers.json").read_text())


def test_golden_file_is_not_empty():
    assert len(RECORDS) >= 10


@pytest.mark.parametrize("rec", RECORDS, ids=[r["source"] for r in RECORDS])
def test_oracle_matches_reference_known_answer(rec):
    got = getattr(O, rec["func"])(*rec["args"])
    if rec["op"] == "==":
        assert got == rec["expected"]
    else:
        atol = rec.get("atol", 0.0)
        rtol = rec.get("rtol", math.sqrt(2.2e-16) if not atol else 0.0)
        assert abs(got - rec["expected"]) <= atol + rtol * abs(rec["expected"])
