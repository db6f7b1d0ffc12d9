"""Loader of the reference known-answer fixture (tests/golden/)."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "reference_known_answers.json")


def load():
    with open(FIXTURE) as f:
        return json.load(f)["cases"]


def cplx(pairs):
    return np.array([complex(a, b) for a, b in pairs], np.complex128)


def init_state(case):
    n = case["n"]
    if case.get("init") is None:
        s = np.zeros(1 << n, np.complex128)
        s[0] = 1
        return s
    return cplx(case["init"])


def tolerance(case):
    # C++ Catch2 goldens are quoted to 1e-7..1e-8; the Python tables are exact expressions.
    return 1e-7 if "src/tests" in case["source"] else 1e-12


def case_id(case):
    ops = case.get("ops") or []
    return "%s-%s" % (case["kind"], "-".join(o[0] for o in ops)[:40])
