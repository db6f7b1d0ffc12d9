"""Generate tests/golden/reference_known_answers.json from the reference's own
test files (run in the build container, where the reference checkout is
mounted; the GPU machine never reads the reference).

Sources:
  1. C++ Catch2 known answers: the numeric literals are read from the cited
     line ranges of the reference test files; the circuit around them is
     restated here (initial state, operation, wires, parameters).
  2. The Python test tables of tests/test_apply.py (lists of
     (operation, input state, expected state) tuples), evaluated from the
     reference source with a stub namespace in which ``qml.<Op>`` is the
     operation's name; no reference code runs.
  3. The closed forms of tests/test_expval.py and tests/test_var.py: each
     test body (its assignments, ``dev.apply`` and ``assert np.allclose``
     statements) is evaluated against recording stubs of ``qml`` and the
     device at the module's THETA / PHI / VARPHI rows.
  4. The ObservableGPU applyInPlace states of Test_ObservablesGPU.cpp
     (named, Hermitian, tensor-product and Hamiltonian observables).
  5. The parametrize tables of tests/test_probs.py and
     tests/test_hamiltonian_sparse.py, and the closed-form gradients of
     tests/test_adjoint_jacobian.py (test_ry_gradient, test_rx_gradient,
     test_multiple_rx_gradient), with the short circuits restated and
     checked against the test source text.

Usage:  python tests/golden/make_golden.py /path/to/reference
        (or set LGPU_REFERENCE_ROOT to the checkout of the reference)
"""
import ast
import json
import math
import os
import re
import sys

import numpy as np

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LGPU_REFERENCE_ROOT")
if __name__ == "__main__" and not REF:
    sys.exit("usage: make_golden.py /path/to/reference (or set LGPU_REFERENCE_ROOT)")
HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "reference_known_answers.json")
CPP_TESTS = "pennylane_lightning_gpu/src/tests"
NUM = re.compile(r"-?\d+(?:\.\d+)?(?:[eE][-+]?\d+)?")
ISING = re.compile(r"expected_results(?:_adj)?\[(\d+)\]\[(\d+)\] = \{([^,]+), ([^}]+)\}")


def lines(rel, a, b):
    with open(os.path.join(REF, rel)) as f:
        src = f.read().splitlines()
    return "\n".join(src[a - 1:b])


def numbers(rel, a, b):
    """All numeric literals on lines a..b (1-based, inclusive) of a reference file."""
    txt = lines(rel, a, b)
    txt = re.sub(r"//.*", "", txt)
    return [float(x) for x in NUM.findall(txt)]


def pairs(vals):
    assert len(vals) % 2 == 0, vals
    return [[vals[i], vals[i + 1]] for i in range(0, len(vals), 2)]


def cpp_cases():
    P = CPP_TESTS + "/Test_StateVectorCudaManaged_Param.cpp"
    N = CPP_TESTS + "/Test_StateVectorCudaManaged_NonParam.cpp"
    A = CPP_TESTS + "/Test_AdjointDiffGPU.cpp"
    cases = []
    # --- RX on |0>: angles line 34, expected lines 35-40, adjoint 42-46
    ang = numbers(P, 34, 34)
    exp = pairs(numbers(P, 35, 40))
    exp_adj = pairs(numbers(P, 42, 46))
    for i, a in enumerate(ang):
        for adj, e in ((False, exp), (True, exp_adj)):
            cases.append({"kind": "state", "source": "%s:34-46" % P, "n": 1, "init": None,
                          "ops": [["RX", [0], [a], adj]], "expected": e[2 * i:2 * i + 2]})
    # --- RY from an explicit initial state: angles 99, expected 101-106, adj 108-113, init 115-116
    ang = numbers(P, 99, 99)
    exp = pairs(numbers(P, 100, 106))
    exp_adj = pairs(numbers(P, 107, 113))
    init = pairs(numbers(P, 115, 116))
    for i, a in enumerate(ang):
        for adj, e in ((False, exp), (True, exp_adj)):
            cases.append({"kind": "state", "source": "%s:96-160" % P, "n": 1, "init": init,
                          "ops": [["RY", [0], [a], adj]], "expected": e[2 * i:2 * i + 2]})
    # --- IsingXX on |000>: angles 443, sparse expected 448-470 (wires {0,1} -> idx 6, {0,2} -> idx 5)
    ang = numbers(P, 443, 443)
    for (a, b), adj in (((448, 458), False), ((463, 473), True)):
        entries = ISING.findall(lines(P, a, b))
        for k in range(4):
            wires = [0, 1] if k < 2 else [0, 2]
            e = [[0.0, 0.0] for _ in range(8)]
            for kk, idx, re_, im_ in entries:
                if int(kk) == k:
                    e[int(idx)] = [float(re_), float(im_)]
            cases.append({"kind": "state", "source": "%s:437-528" % P, "n": 3, "init": None,
                          "ops": [["IsingXX", wires, [ang[k % 2]], adj]], "expected": e})
    # --- IsingYY on |000>: angles 536, expected 541-551, adjoint 556-566 (same layout as IsingXX)
    ang = numbers(P, 536, 536)
    for (a, b), adj in (((541, 551), False), ((556, 566), True)):
        entries = ISING.findall(lines(P, a, b))
        assert len(entries) == 8
        for k in range(4):
            wires = [0, 1] if k < 2 else [0, 2]
            e = [[0.0, 0.0] for _ in range(8)]
            for kk, idx, re_, im_ in entries:
                if int(kk) == k:
                    e[int(idx)] = [float(re_), float(im_)]
            cases.append({"kind": "state", "source": "%s:530-621" % P, "n": 3, "init": None,
                          "ops": [["IsingYY", wires, [ang[k % 2]], adj]], "expected": e})
    # --- IsingZZ on |000>: angles 629, expected 634-635, adjoint 639-640, wires {0,1} and {0,2}
    ang = numbers(P, 629, 629)
    for (a, b), adj in (((634, 635), False), ((639, 640), True)):
        entries = ISING.findall(lines(P, a, b))
        assert len(entries) == 2
        for kk, idx, re_, im_ in entries:
            for wires in ([0, 1], [0, 2]):
                e = [[0.0, 0.0] for _ in range(8)]
                e[int(idx)] = [float(re_), float(im_)]
                cases.append({"kind": "state", "source": "%s:623-694" % P, "n": 3, "init": None,
                              "ops": [["IsingZZ", wires, [ang[int(kk)]], adj]], "expected": e})
    # --- excitations and MultiRZ on |0...0>: every apply<Gate>({wires}, adjoint, angles[index])
    # call of the test block, checked against expected_results[_adj][index] (phases of |0...0>
    # for the Minus/Plus forms and MultiRZ) or against the unchanged |0...0> (SingleExcitation,
    # DoubleExcitation)
    for name, a, b in (("SingleExcitation", 695, 740), ("SingleExcitationMinus", 741, 815),
                       ("SingleExcitationPlus", 816, 890), ("DoubleExcitation", 891, 926),
                       ("DoubleExcitationMinus", 927, 981), ("DoubleExcitationPlus", 982, 1036),
                       ("MultiRZ", 1037, 1108)):
        text = lines(P, a, b)
        assert ("LightningGPU::apply%s\"" % name) in text
        nq = int(re.search(r"num_qubits = (\d+);", text).group(1))
        ang = [float(x) for x in re.search(r"angles\{([^}]*)\}", text).group(1).split(",")]
        table = {False: {}, True: {}}
        for m in re.finditer(r"expected_results(_adj)?\[(\d+)\]\[(\d+)\] = \{([^,]+), ([^}]+)\}", text):
            table[m.group(1) is not None].setdefault(int(m.group(2)), {})[int(m.group(3))] = [float(m.group(4)),
                                                                                            float(m.group(5))]
        calls = re.findall(r"apply%s\(\s*\{([0-9, ]+)\},\s*(true|false),\s*angles\[index\]" % name, text)
        assert calls, name
        for wires_s, adj_s in calls:
            wires = [int(x) for x in wires_s.split(",")]
            adj = adj_s == "true"
            for k, theta in enumerate(ang):
                e = [[0.0, 0.0] for _ in range(1 << nq)]
                if table[adj]:
                    for idx, v in table[adj][k].items():
                        e[idx] = v
                else:
                    assert re.search(r"expected_results\[0\] = \{1\.0, 0\.0\}", text)
                    e[0] = [1.0, 0.0]
                cases.append({"kind": "state", "source": "%s:%d-%d" % (P, a, b), "n": nq, "init": None,
                              "ops": [[name, wires, [theta], adj]], "expected": e})
    # --- PauliY / PauliZ / S / T on |+++> (NonParam): the expected_results rows are tables of
    # two symbols per target wire; the symbols' values are restated from their definitions
    s2 = 1.0 / math.sqrt(2.0)
    for name, (da, db), (ra, rb), sym, must in (
            ("PauliY", (193, 197), (199, 202), {"p": 0.5j * s2, "m": -0.5j * s2}, "IMAG"),
            ("PauliZ", (238, 240), (242, 245), {"p": 0.5 * s2, "m": -0.5 * s2}, "INVSQRT2"),
            ("S", (279, 281), (283, 286), {"r": 0.5 * s2, "i": 0.5j * s2}, "IMAG"),
            ("T", (321, 322), (324, 327), {"r": 1.0 / (2.0 * math.sqrt(2.0)), "i": 0.25 + 0.25j}, "1.0 / 4")):
        assert must in lines(N, da, db), name
        rows = re.findall(r"\{([a-z, ]+)\}", lines(N, ra, rb))
        assert len(rows) == 3, (name, rows)
        for index, row in enumerate(rows):
            vals = [sym[x.strip()] for x in row.split(",")]
            assert len(vals) == 8
            block = {"PauliY": "182-226", "PauliZ": "228-268", "S": "270-309", "T": "311-352"}[name]
            cases.append({"kind": "state", "source": "%s:%s" % (N, block), "n": 3, "init": None,
                          "ops": [["Hadamard", [0], [], False], ["Hadamard", [1], [], False],
                                  ["Hadamard", [2], [], False], [name, [index], [], False]],
                          "expected": [[float(np.real(v)), float(np.imag(v))] for v in vals]})
    # --- dense expval (1.263 - 1.011i) with a non-normalised state: NonParam 866-889
    init = pairs(numbers(N, 867, 869))
    mat = pairs(numbers(N, 874, 886))
    assert len(mat) == 64
    exp = numbers(N, 890, 890)
    cases.append({"kind": "expval_matrix", "source": "%s:863-893" % N, "n": 3, "init": init, "wires": [0, 1, 2],
                  "matrix": mat, "expected": exp})
    # --- identity expval on a GHZ state: NonParam 838-861
    cases.append({"kind": "expval_matrix", "source": "%s:838-861" % N, "n": 3, "init": None,
                  "ops": [["Hadamard", [0], [], False], ["CNOT", [0, 1], [], False], ["CNOT", [1, 2], [], False]],
                  "wires": [0, 1, 2], "matrix": [[1.0 if i % 9 == 0 else 0.0, 0.0] for i in range(64)],
                  "expected": [1.0, 0.0]})
    # --- sparse expval = 1: NonParam 903-925
    init = pairs(numbers(N, 903, 905))
    offs = [int(x) for x in numbers(N, 913, 913)[1:]]
    cols = [int(x) for x in numbers(N, 914, 915)[1:]]
    vals = pairs(numbers(N, 917, 920))
    assert len(offs) == 9 and len(cols) == 16 and len(vals) == 16
    cases.append({"kind": "expval_sparse", "source": "%s:897-932" % N, "n": 3, "init": init, "indptr": offs,
                  "indices": cols, "data": vals, "expected": [1.0]})
    # --- adjoint Jacobians (Test_AdjointDiffGPU.cpp)
    p = [-math.pi / 7, math.pi / 5, 2 * math.pi / 3]  # lines 201 / 237: {-M_PI / 7, M_PI / 5, 2 * M_PI / 3}
    assert "{-M_PI / 7, M_PI / 5, 2 * M_PI / 3}" in lines(A, 201, 201) and "M_PI / 7" in lines(A, 237, 237)
    exp = numbers(A, 228, 230)[0::4]  # CHECK(value == Approx(jacobian[0][i]).margin(m))
    cases.append({"kind": "adjoint", "source": "%s:198-232" % A, "n": 3,
                  "ops": [["RX", [0], [p[0]], False], ["RX", [1], [p[1]], False], ["RX", [2], [p[2]], False]],
                  "obs": [[False, [[1.0, [["PauliZ", [0]], ["PauliZ", [1]], ["PauliZ", [2]]]]]]],
                  "tp": [0, 1, 2], "expected": [exp]})
    exp = numbers(A, 272, 277)[0::4]
    ops = [["RZ", [0], [p[0]], False], ["RY", [0], [p[1]], False], ["RZ", [0], [p[2]], False],
           ["CNOT", [0, 1], [], False], ["CNOT", [1, 2], [], False], ["RZ", [1], [p[0]], False],
           ["RY", [1], [p[1]], False], ["RZ", [1], [p[2]], False]]
    cases.append({"kind": "adjoint", "source": "%s:234-279" % A, "n": 3, "ops": ops,
                  "obs": [[False, [[1.0, [["PauliX", [0]], ["PauliX", [1]], ["PauliX", [2]]]]]]],
                  "tp": [0, 1, 2, 3, 4, 5], "expected": [exp]})
    lp = numbers(A, 350, 351)
    assert len(lp) == 9
    exp = numbers(A, 401, 401)
    names = ["Hadamard", "RX", "CNOT", "RZ", "RY", "RZ", "RZ", "RY", "RZ", "RZ", "RY", "CNOT"]
    wires = [[0], [0], [0, 1], [0], [0], [0], [0], [0], [0], [0], [1], [0, 1]]
    ops, k = [], 0
    for nm, w in zip(names, wires):
        if nm in ("Hadamard", "CNOT"):
            ops.append([nm, w, [], False])
        else:
            ops.append([nm, w, [lp[k]], False])
            k += 1
    cases.append({"kind": "adjoint", "source": "%s:339-407" % A, "n": 2, "ops": ops,
                  "obs": [[False, [[1.0, [["PauliX", [0]], ["PauliZ", [1]]]]]]], "tp": [1, 2, 3],
                  "expected": [exp]})
    return cases


CPAIR = re.compile(r"\{\s*(-?[0-9.]+(?:[eE][-+]?\d+)?)\s*,\s*(-?[0-9.]+(?:[eE][-+]?\d+)?)\s*\}")


def cpairs(rel, a, b):
    """The {re, im} literals on lines a..b of a reference file, in order."""
    return [[float(x), float(y)] for x, y in CPAIR.findall(lines(rel, a, b))]


def observable_cases():
    """ObservableGPU::applyInPlace known answers (Test_ObservablesGPU.cpp):
    a 4-qubit state, optional Hadamards, then observables applied in turn,
    the state checked after each.  Amplitudes are read from the cited lines;
    the observables are restated (a named observable with a parameter, RX
    on wire 1 at 0.245, is given as its matrix, as is the test's rotation
    matrix passed as a Hermitian)."""
    O = CPP_TESTS + "/Test_ObservablesGPU.cpp"
    h = cpairs(O, 93, 96)
    assert len(h) == 4 and abs(h[0][0] - 0.7071067811865475) < 1e-16
    assert "std::cos(0.1234)" in lines(O, 97, 97) and "-std::sin(0.1234)" in lines(O, 98, 98)
    c, s_ = math.cos(0.1234), math.sin(0.1234)
    ry = [[c, 0.0], [-s_, 0.0], [s_, 0.0], [c, 0.0]]  # lines 97-100, row-major
    assert '"RX", {1}, {0.245}' in lines(O, 35, 35)
    c2, s2 = math.cos(0.245 / 2), math.sin(0.245 / 2)
    rx = [[c2, 0.0], [0.0, -s2], [0.0, -s2], [c2, 0.0]]  # RX(0.245)

    def named(name, w):
        return [name, [w], None]

    def mat(m, w):
        return ["Hermitian", [w], m]

    def single(*factors):
        return [False, [[1.0, list(factors)]]]

    had = lambda ws: [["Hadamard", [w], [], False] for w in ws]
    cases = []
    r1, r2 = cpairs(O, 58, 59), cpairs(O, 61, 63)
    assert len(r1) == 16 and len(r2) == 16
    cases.append({"kind": "observable", "source": "%s:52-81" % O, "n": 4, "init": None, "ops": [],
                  "steps": [{"ops": [], "obs": single(named("PauliX", 3)), "expected": r1},
                            {"ops": [], "obs": single(mat(rx, 1)), "expected": r2}]})
    r1, r2 = cpairs(O, 119, 134), cpairs(O, 136, 139)
    assert len(r1) == 16 and len(r2) == 16
    assert "applyHadamard({1}" in lines(O, 148, 148) and "applyHadamard({2}" in lines(O, 149, 149)
    cases.append({"kind": "observable", "source": "%s:114-158" % O, "n": 4, "init": None, "ops": [],
                  "steps": [{"ops": [], "obs": single(mat(h, 0)), "expected": r1},
                            {"ops": had([1, 2]), "obs": single(mat(ry, 2)), "expected": r2}]})
    r1, r2 = cpairs(O, 221, 224), cpairs(O, 235, 242)
    assert len(r1) == 16 and len(r2) == 16
    cases.append({"kind": "observable", "source": "%s:189-250" % O, "n": 4, "init": None, "ops": had([1, 2]),
                  "steps": [{"ops": [], "obs": single(mat(h, 0), mat(ry, 2)), "expected": r1},
                            {"ops": [], "obs": single(named("PauliX", 3), mat(rx, 1)), "expected": r2}]})
    assert "{0.165, 0.13, 0.5423}" in lines(O, 281, 281) and "{0.8545, 0.3222}" in lines(O, 285, 285)
    r1, r2 = cpairs(O, 324, 327), cpairs(O, 338, 342)
    assert len(r1) == 16 and len(r2) == 16
    ham1 = [True, [[0.165, [mat(h, 0)]], [0.13, [named("PauliX", 2)]], [0.5423, [named("PauliX", 2)]]]]
    ham2 = [True, [[0.8545, [mat(h, 0), named("PauliX", 2)]], [0.3222, [named("PauliX", 2), named("PauliX", 3)]]]]
    cases.append({"kind": "observable", "source": "%s:258-352" % O, "n": 4, "init": None, "ops": had([0, 1, 2]),
                  "steps": [{"ops": [], "obs": ham1, "expected": r1}, {"ops": [], "obs": ham2, "expected": r2}]})
    return cases


class _Qml:
    def __getattr__(self, name):
        return name


def python_cases():
    rel = "tests/test_apply.py"
    with open(os.path.join(REF, rel)) as f:
        tree = ast.parse(f.read())
    ns = {"qml": _Qml(), "math": math, "np": np}
    wanted = {"test_data_no_parameters": 1, "test_data_two_wires_no_parameters": 2,
              "test_data_three_wires_no_parameters": 3, "test_data_single_wire_with_parameters": 1,
              "test_data_two_wires_with_parameters": 2}
    cases = []
    for node in ast.walk(tree):
        if isinstance(node, ast.Assign) and len(node.targets) == 1 and isinstance(node.targets[0], ast.Name):
            name = node.targets[0].id
            if name not in wanted:
                continue
            table = eval(compile(ast.Expression(node.value), rel, "eval"), ns)
            for row in table:
                if len(row) == 3:
                    op, inp, out = row
                    par = []
                else:
                    op, inp, out, par = row
                nw = wanted[name]
                cases.append({"kind": "state", "source": "%s:%d (%s)" % (rel, node.lineno, name), "n": nw,
                              "init": [[float(np.real(x)), float(np.imag(x))] for x in np.asarray(inp, complex)],
                              "ops": [[op, list(range(nw)), [float(x) for x in np.atleast_1d(par)], False]],
                              "expected": [[float(np.real(x)), float(np.imag(x))] for x in np.asarray(out, complex)]})
    return cases


class _Obs:
    """An operation or observable of a reference test, recorded by name:
    ``name`` (or a list of names for a tensor product), wires, parameters and
    an explicit matrix for Hermitian factors."""

    def __init__(self, name, params, wires, matrix=None):
        self.factors = [(name, [int(w) for w in np.atleast_1d(wires)], [float(p) for p in params], matrix)]

    def __matmul__(self, other):
        out = _Obs.__new__(_Obs)
        out.factors = self.factors + other.factors
        return out

    def diagonalizing_gates(self):
        return []  # the reference device ignores rotations in apply()

    def as_op(self):
        (name, wires, params, _), = self.factors
        return [name, wires, params, False]

    def as_obs(self):
        return [[f[0], f[1]] + ([[[float(np.real(x)), float(np.imag(x))] for x in np.ravel(f[3])]]
                                if f[3] is not None else []) for f in self.factors]


class _Ham:
    def __init__(self, coeffs, obs):
        self.coeffs, self.obs = [float(c) for c in coeffs], obs

    def sparse_matrix(self):
        return self


class _QmlObs:
    """Stub of the ``qml`` namespace: constructors record operations and
    observables; ``qml.device`` returns a recording device."""

    def __getattr__(self, name):
        def make(*args, wires=None, **kw):
            if name == "SparseHamiltonian":
                return args[0]
            if name == "Hermitian":
                return _Obs(name, [], wires, np.asarray(args[0], complex))
            if wires is None:
                args, wires = args[:-1], args[-1]
            return _Obs(name, args, wires)
        return make

    def Hamiltonian(self, coeffs, obs):  # noqa: N802 (the reference's name)
        return _Ham(coeffs, obs)

    def device(self, *a, **kw):
        return _RecDev()


class _RecDev:
    def __init__(self):
        self.ops = []

    def apply(self, ops, **kw):
        self.ops.extend(o.as_op() for o in ops)

    def syncH2D(self, state):
        self.state = np.asarray(state)

    def expval(self, obs):
        if isinstance(obs, _Ham):
            return _Meas("expval", obs)
        return _Meas("expval", obs.as_obs())

    def var(self, obs):
        return _Meas("var", obs.as_obs())


class _Meas:
    """A recorded measurement (kept opaque so that ``np.array([...])`` of
    several measurements stays a one-dimensional object array)."""

    def __init__(self, kind, obs):
        self.rec = [kind, obs]


def _decorator_params(node, ns):
    """(names, rows) of a ``pytest.mark.parametrize(names, rows)`` decorator."""
    for d in node.decorator_list:
        if isinstance(d, ast.Call) and getattr(d.func, "attr", "") == "parametrize":
            names = [s.strip() for s in ast.literal_eval(d.args[0]).split(",")]
            rows = eval(compile(ast.Expression(d.args[1]), "<param>", "eval"), ns)
            if len(names) == 1:
                return names, [(r,) for r in rows]
            return names, [tuple(r) for r in rows]
    return None, None


def _run_body(fn, rel, ns):
    """Evaluate a reference test body against the stubs; every
    ``assert np.allclose(res, expected, ...)`` becomes a recorded pair."""
    recorded = []

    def record(res, expected, *a, **kw):
        recorded.append((res, expected))
        return True

    body = []
    for st in fn.body:
        if isinstance(st, ast.Assert) and isinstance(st.test, ast.Call) and \
                getattr(st.test.func, "attr", "") == "allclose":
            st = ast.Expr(ast.Call(ast.Name("_record", ast.Load()), st.test.args, st.test.keywords))
        if isinstance(st, (ast.Assign, ast.Expr)):
            body.append(st)
    mod = ast.fix_missing_locations(ast.Module(body, []))
    local = dict(ns, _record=record)
    exec(compile(mod, rel, "exec"), local)
    return recorded, local


def python_measure_cases():
    """Closed-form expectation values and variances of the reference's
    tests/test_expval.py and tests/test_var.py (TestExpval, TestTensorExpval,
    TestVar, TestTensorVar): each test body is evaluated with the recording
    stubs at the module's THETA / PHI / VARPHI rows; the expected values are
    the reference's own expressions."""
    cases = []
    for rel in ("tests/test_expval.py", "tests/test_var.py"):
        with open(os.path.join(REF, rel)) as f:
            tree = ast.parse(f.read())
        ns = {"np": np, "qml": _QmlObs(), "math": math}
        for node in tree.body:
            if isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Name) and \
                    node.targets[0].id in ("THETA", "PHI", "VARPHI"):
                ns[node.targets[0].id] = eval(compile(ast.Expression(node.value), rel, "eval"), ns)
        for cls in tree.body:
            if not isinstance(cls, ast.ClassDef):
                continue
            names, rows = _decorator_params(cls, ns)
            if names is None:
                continue
            for fn in cls.body:
                if not (isinstance(fn, ast.FunctionDef) and fn.name.startswith("test_")):
                    continue
                for row in rows:
                    dev = _RecDev()
                    env = dict(ns, tol=1e-4, qubit_device_3_wires=dev, dev=dev, **dict(zip(names, row)))
                    recorded, local = _run_body(fn, rel, env)
                    dev = local["dev"]
                    for res, expected in recorded:
                        meas = [r.rec for r in (res if isinstance(res, (list, np.ndarray)) else [res])]
                        exp = np.atleast_1d(np.asarray(expected, float)).tolist()
                        if len(exp) == 1 and len(meas) > 1:
                            exp = exp * len(meas)
                        cases.append({"kind": "measure", "source": "%s:%d (%s.%s)" % (rel, fn.lineno, cls.name,
                                                                                     fn.name),
                                      "n": 3, "init": None, "ops": dev.ops, "measure": meas, "expected": exp})
    return cases


def python_probs_sparse_cases():
    """Known answers of tests/test_probs.py (probabilities of fixed 2-wire
    circuits, PennyLane order) and tests/test_hamiltonian_sparse.py (sparse
    Hamiltonian expectation values): the numbers are the reference's
    parametrize tables; the circuits are restated from the test bodies."""
    cases = []
    rel = "tests/test_probs.py"
    with open(os.path.join(REF, rel)) as f:
        tree = ast.parse(f.read())
    circuits = {
        # test_probs_tape_wire0: RX(0.4), Rot(0.5, 0.3, -0.7), RY(-0.2) on wire 0
        "test_probs_tape_wire0": [["RX", [0], [0.4], False], ["Rot", [0], [0.5, 0.3, -0.7], False],
                                  ["RY", [0], [-0.2], False]],
        # test_probs_tape_wire01: RX(0.5) on wire 0, RY(0.3) on wire 1
        "test_probs_tape_wire01": [["RX", [0], [0.5], False], ["RY", [1], [0.3], False]],
    }
    for cls in [c for c in tree.body if isinstance(c, ast.ClassDef)]:
        for fn in cls.body:
            if isinstance(fn, ast.FunctionDef) and fn.name in circuits:
                src = ast.get_source_segment(open(os.path.join(REF, rel)).read(), fn)
                for op in circuits[fn.name]:
                    assert "qml.%s(" % op[0] in src, (fn.name, op)
                _, rows = _decorator_params(fn, {"np": np})
                for (row,) in rows:
                    wires, expected = row
                    cases.append({"kind": "probs", "source": "%s:%d (%s)" % (rel, fn.lineno, fn.name), "n": 2,
                                  "init": None, "ops": circuits[fn.name], "wires": [int(w) for w in np.atleast_1d(wires)],
                                  "expected": [float(x) for x in expected]})
    rel = "tests/test_hamiltonian_sparse.py"
    with open(os.path.join(REF, rel)) as f:
        text = f.read()
    tree = ast.parse(text)
    ns = {"np": np, "qml": _QmlObs()}
    for cls in [c for c in tree.body if isinstance(c, ast.ClassDef)]:
        for fn in cls.body:
            if not isinstance(fn, ast.FunctionDef):
                continue
            src = ast.get_source_segment(text, fn)
            if fn.name in ("test_sparse_Pauli_words", "test_sparse_arbitrary"):
                assert "qml.RX(0.4, wires=[0])" in src and "qml.RY(-0.2, wires=[1])" in src
                _, rows = _decorator_params(fn, ns)
                for (row,) in rows:
                    obs, expected = row
                    cases.append({"kind": "expval_sparse", "source": "%s:%d (%s)" % (rel, fn.lineno, fn.name),
                                  "n": 2, "init": None,
                                  "ops": [["RX", [0], [0.4], False], ["RY", [1], [-0.2], False]],
                                  **_csr([1.0], [obs], 2), "expected": [float(expected)]})
            elif fn.name == "test_hamiltonian_expectation":
                recorded, local = _run_body(fn, rel, dict(ns, qubit_device_3_wires=_RecDev(), tol=1e-4,
                                                          _record=None))
                sv = local["state_vector"]
                ham = local["Hmat"]
                cases.append({"kind": "expval_sparse", "source": "%s:%d (%s)" % (rel, fn.lineno, fn.name),
                              "n": 3, "init": [[float(np.real(x)), float(np.imag(x))] for x in sv],
                              **_csr(ham.coeffs, ham.obs, 3), "expected": [float(local["expected"])],
                              # the test's state is complex64 (norm 1 to 4e-8), checked by np.allclose
                              "tol": 1e-6})
    return cases


_PAULI = {"Identity": np.eye(2), "PauliX": np.array([[0, 1], [1, 0]]), "PauliY": np.array([[0, -1j], [1j, 0]]),
          "PauliZ": np.diag([1, -1])}


def _csr(coeffs, obs_list, n):
    """CSR of sum_k c_k O_k on n wires (wire 0 the most significant bit), the
    matrix that ``qml.Hamiltonian(...).sparse_matrix()`` builds."""
    h = np.zeros((1 << n, 1 << n), complex)
    for c, o in zip(coeffs, obs_list):
        per = [np.eye(2)] * n
        for name, wires, _, mat in o.factors:
            assert len(wires) == 1
            per[wires[0]] = mat if mat is not None else _PAULI[name]
        m = np.array([[1.0]])
        for p in per:
            m = np.kron(m, p)
        h += c * m
    indptr, indices, data = [0], [], []
    for r in range(1 << n):
        for col in np.nonzero(h[r])[0]:
            indices.append(int(col))
            data.append([float(h[r, col].real), float(h[r, col].imag)])
        indptr.append(len(indices))
    return {"indptr": indptr, "indices": indices, "data": data}


def python_adjoint_cases():
    """Closed-form adjoint Jacobians of tests/test_adjoint_jacobian.py:
    test_ry_gradient (d<X>/d par = cos par over its parametrize list),
    test_rx_gradient (-sin a) and test_multiple_rx_gradient (-diag(sin p));
    the parameters and expected expressions are evaluated from the test
    bodies, the one-gate circuits are restated."""
    rel = "tests/test_adjoint_jacobian.py"
    with open(os.path.join(REF, rel)) as f:
        text = f.read()
    tree = ast.parse(text)
    cases = []
    fns = {fn.name: fn for fn in ast.walk(tree) if isinstance(fn, ast.FunctionDef)}

    def assigned(fn, env, names):
        for st in fn.body:
            if isinstance(st, ast.Assign) and isinstance(st.targets[0], ast.Name) and st.targets[0].id in names:
                env[st.targets[0].id] = eval(compile(ast.Expression(st.value), rel, "eval"), env)
        return env

    fn = fns["test_ry_gradient"]
    src = ast.get_source_segment(text, fn)
    assert "qml.RY(par, wires=[0])" in src and "qml.PauliX(0)" in src
    _, rows = _decorator_params(fn, {"np": np})
    for (par,) in rows:
        env = assigned(fn, {"np": np, "par": par}, {"exact"})
        cases.append({"kind": "adjoint", "source": "%s:%d (test_ry_gradient)" % (rel, fn.lineno), "n": 1,
                      "ops": [["RY", [0], [float(par)], False]], "obs": [[False, [[1.0, [["PauliX", [0]]]]]]],
                      "tp": [0], "expected": [[float(env["exact"])]]})
    fn = fns["test_rx_gradient"]
    src = ast.get_source_segment(text, fn)
    assert "qml.RX(a, wires=0)" in src and "qml.PauliZ(0)" in src
    env = assigned(fn, {"np": np}, {"a", "expected_jacobian"})
    cases.append({"kind": "adjoint", "source": "%s:%d (test_rx_gradient)" % (rel, fn.lineno), "n": 1,
                  "ops": [["RX", [0], [float(env["a"])], False]], "obs": [[False, [[1.0, [["PauliZ", [0]]]]]]],
                  "tp": [0], "expected": [[float(env["expected_jacobian"])]]})
    fn = fns["test_multiple_rx_gradient"]
    src = ast.get_source_segment(text, fn)
    assert "qml.RX(params[2], wires=2)" in src and "qml.expval(qml.PauliZ(idx))" in src
    env = assigned(fn, {"np": np}, {"params", "expected_jacobian"})
    p = [float(x) for x in env["params"]]
    cases.append({"kind": "adjoint", "source": "%s:%d (test_multiple_rx_gradient)" % (rel, fn.lineno), "n": 3,
                  "ops": [["RX", [w], [p[w]], False] for w in range(3)],
                  "obs": [[False, [[1.0, [["PauliZ", [w]]]]]] for w in range(3)], "tp": [0, 1, 2],
                  "expected": np.asarray(env["expected_jacobian"], float).tolist()})
    return cases


def main():
    cases = cpp_cases() + python_cases() + python_measure_cases() + python_probs_sparse_cases() + \
        python_adjoint_cases() + observable_cases()
    with open(OUT, "w") as f:
        json.dump({"reference": "PennyLane-Lightning-GPU 0.33.0-dev", "cases": cases}, f, indent=1)
    print("wrote %d cases to %s" % (len(cases), OUT))


if __name__ == "__main__":
    main()
