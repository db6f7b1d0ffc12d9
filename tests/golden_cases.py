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


_NAMED = {"Identity": np.eye(2), "PauliX": np.array([[0, 1], [1, 0]], complex),
          "PauliY": np.array([[0, -1j], [1j, 0]]), "PauliZ": np.diag([1.0 + 0j, -1.0]),
          "Hadamard": np.array([[1, 1], [1, -1]], complex) / np.sqrt(2)}


def observable_matrix(factors):
    """(matrix, wires) of a tensor product of named (or explicit Hermitian)
    one-wire factors, the first factor's wire the most significant bit."""
    m, wires = np.array([[1.0 + 0j]]), []
    for f in factors:
        name, w = f[0], f[1]
        mat = cplx(f[2]).reshape(2, 2) if len(f) > 2 else _NAMED[name]
        m = np.kron(m, mat)
        wires.extend(w)
    return m, wires


def oracle_observable(obs):
    """A fixture observable [is_hamiltonian, [[coeff, [[name, wires, matrix_or_None], ...]], ...]]
    in the oracle's form."""
    is_h, terms = obs
    return (is_h, [(c, [(f[0], f[1], None if f[2] is None else cplx(f[2]).reshape(2, 2)) for f in fs])
                   for c, fs in terms])


def pennylane_order(p, k):
    """Probabilities of the engine's order (bit j of the index is wires[j])
    in PennyLane's order (wires[0] most significant), as the device returns them."""
    return np.asarray(p).reshape([2] * k).transpose().reshape(-1)


def tolerance(case):
    # C++ Catch2 goldens are quoted to 1e-7..1e-8; the Python tables are exact
    # expressions, unless the case carries the reference test's own tolerance.
    if "tol" in case:
        return case["tol"]
    return 1e-7 if "src/tests" in case["source"] else 1e-12


def case_id(case):
    ops = case.get("ops") or []
    return "%s-%s" % (case["kind"], "-".join(o[0] for o in ops)[:40])
