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
        r = oracle.expval_sparse(psi, case["indptr"], case["indices"], G.cplx(case["data"]))
        assert abs(r - case["expected"][0]) < tol
    elif case["kind"] == "adjoint":
        final = oracle.apply_ops(psi, ops)
        obs = [(h, [(c, [(f[0], f[1], None) for f in fs]) for c, fs in terms]) for h, terms in case["obs"]]
        jac = oracle.adjoint_jacobian(final, ops, obs, case["tp"])
        assert np.max(np.abs(jac - np.array(case["expected"]))) < tol


def test_fixture_covers_reference_tests():
    kinds = {c["kind"] for c in CASES}
    assert kinds == {"state", "expval_matrix", "expval_sparse", "adjoint"}
    assert len(CASES) >= 90
