"""Pin the oracle to the reference's own known answers (tests/golden/)."""
import numpy as np
import pytest

import golden_cases as G

CASES = G.load()


@pytest.mark.parametrize("case", CASES, ids=[G.case_id(c) for c in CASES])
def test_oracle_matches_reference_golden(oracle, case):
    psi = G.init_state(case)
    ops = [(o[0], o[1], o[2], o[3], None) for o in case.get("ops") or []]
    tol = G.tolerance(case)
    if case["kind"] == "state":
        out = oracle.apply_ops(psi, ops)
        assert np.max(np.abs(out - G.cplx(case["expected"]))) < tol
    elif case["kind"] == "expval_matrix":
        if ops:
            psi = oracle.apply_ops(psi, ops)
        mat = G.cplx(case["matrix"]).reshape(1 << len(case["wires"]), -1)
        r = oracle.expval_matrix(psi, mat, case["wires"])
        assert abs(r - complex(*case["expected"])) < tol
    elif case["kind"] == "expval_sparse":
        if ops:
            psi = oracle.apply_ops(psi, ops)
        r = oracle.expval_sparse(psi, case["indptr"], case["indices"], G.cplx(case["data"]))
        assert abs(r - case["expected"][0]) < tol
    elif case["kind"] == "measure":
        psi = oracle.apply_ops(psi, ops)
        for (kind, factors), want in zip(case["measure"], case["expected"]):
            m, wires = G.observable_matrix(factors)
            mean = oracle.expval_matrix(psi, m, wires).real
            got = mean if kind == "expval" else oracle.expval_matrix(psi, m @ m, wires).real - mean ** 2
            assert abs(got - want) < tol, (kind, factors, got, want)
    elif case["kind"] == "observable":
        psi = oracle.apply_ops(psi, ops) if ops else psi
        for step in case["steps"]:
            if step["ops"]:
                psi = oracle.apply_ops(psi, [(o[0], o[1], o[2], o[3], None) for o in step["ops"]])
            psi = oracle.apply_observable(psi, G.oracle_observable(step["obs"]))
            assert np.max(np.abs(psi - G.cplx(step["expected"]))) < tol
    elif case["kind"] == "probs":
        psi = oracle.apply_ops(psi, ops)
        k = len(case["wires"])
        got = G.pennylane_order(oracle.probs(psi, case["wires"]), k)
        assert np.max(np.abs(got - np.array(case["expected"]))) < tol
    elif case["kind"] == "adjoint":
        final = oracle.apply_ops(psi, ops)
        obs = [(h, [(c, [(f[0], f[1], None) for f in fs]) for c, fs in terms]) for h, terms in case["obs"]]
        jac = oracle.adjoint_jacobian(final, ops, obs, case["tp"])
        assert np.max(np.abs(jac - np.array(case["expected"]))) < tol


def test_fixture_covers_reference_tests():
    kinds = {c["kind"] for c in CASES}
    assert kinds == {"state", "expval_matrix", "expval_sparse", "adjoint", "measure", "probs", "observable"}
    assert len(CASES) >= 150
    sources = {c["source"].split(":")[0] for c in CASES}
    for rel in ("tests/test_apply.py", "tests/test_expval.py", "tests/test_var.py", "tests/test_probs.py",
                "tests/test_hamiltonian_sparse.py", "tests/test_adjoint_jacobian.py"):
        assert rel in sources, rel
