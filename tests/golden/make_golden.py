"""Generate tests/golden/reference_known_answers.json from the reference's own
test files (run in the build container, where the reference checkout is
mounted; the GPU machine never reads the reference).

Two sources:
  1. C++ Catch2 known answers: the numeric literals are read from the cited
     line ranges of the reference test files; the circuit around them is
     restated here (initial state, operation, wires, parameters).
  2. The Python test tables of tests/test_apply.py (lists of
     (operation, input state, expected state) tuples), evaluated from the
     reference source with a stub namespace in which ``qml.<Op>`` is the
     operation's name; no reference code runs.

Usage:  python tests/golden/make_golden.py [/path/to/reference]
"""
import ast
import json
import math
import os
import re
import sys

import numpy as np

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
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


def main():
    cases = cpp_cases() + python_cases()
    with open(OUT, "w") as f:
        json.dump({"reference": "PennyLane-Lightning-GPU 0.33.0-dev", "cases": cases}, f, indent=1)
    print("wrote %d cases to %s" % (len(cases), OUT))


if __name__ == "__main__":
    main()
