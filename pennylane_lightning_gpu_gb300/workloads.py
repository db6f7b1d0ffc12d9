"""Seeded synthetic workloads shaped like the reference's benchmark configs.

Operations are tuples ``(name, wires, params, inverse)``; Hamiltonians are
lists of ``(coeff, word, wires)`` Pauli terms.  Every generator takes an
explicit ``numpy.random.Generator`` or seed so that the GPU path, the oracle
and the CPU baseline see identical inputs.
"""
import numpy as np

TWO_PI = 2.0 * np.pi


def layered_ansatz(n, layers, rng):
    """RX, RY, RZ on every wire, then a CNOT ring (i -> i+1 mod n), per layer.

    The 12-qubit, 4-layer instance is the CPU-path configuration (144 params).
    """
    ops = []
    for _ in range(layers):
        for w in range(n):
            for g in ("RX", "RY", "RZ"):
                ops.append((g, [w], [float(rng.uniform(0, TWO_PI))], False))
        if n > 1:
            for w in range(n):
                ops.append(("CNOT", [w, (w + 1) % n], [], False))
    return ops


def random_circuit(n, layers, rng, rot_per_layer=None, ent_per_layer=None):
    """Random single-qubit rotations (RX/RY/RZ/Rot) on random wires plus
    CNOT/CZ/CRY on random distinct pairs.  Per layer: n rotations and n/2
    two-qubit gates unless given."""
    rot_per_layer = n if rot_per_layer is None else rot_per_layer
    ent_per_layer = n // 2 if ent_per_layer is None else ent_per_layer
    ops = []
    for _ in range(layers):
        for _ in range(rot_per_layer):
            g = ("RX", "RY", "RZ", "Rot")[int(rng.integers(4))]
            w = int(rng.integers(n))
            if g == "Rot":
                ops.append((g, [w], [float(x) for x in rng.uniform(0, TWO_PI, 3)], False))
            else:
                ops.append((g, [w], [float(rng.uniform(0, TWO_PI))], False))
        for _ in range(ent_per_layer):
            g = ("CNOT", "CZ", "CRY")[int(rng.integers(3))]
            a, b = (int(x) for x in rng.choice(n, size=2, replace=False))
            ops.append((g, [a, b], [float(rng.uniform(0, TWO_PI))] if g == "CRY" else [], False))
    return ops


def random_pauli_hamiltonian(n, terms, rng, max_wires=6):
    """`terms` Pauli words, each on 1..max_wires distinct wires with uniform
    X/Y/Z letters and N(0, 1) coefficients."""
    ham = []
    for _ in range(terms):
        k = int(rng.integers(1, min(max_wires, n) + 1))
        wires = sorted(int(x) for x in rng.choice(n, size=k, replace=False))
        word = "".join("XYZ"[int(rng.integers(3))] for _ in range(k))
        ham.append((float(rng.normal()), word, wires))
    return ham


def ry_rz_cz_ansatz(n, layers, rng):
    """RY, RZ on every wire, then a CZ ladder (i, i+1), per layer."""
    ops = []
    for _ in range(layers):
        for w in range(n):
            ops.append(("RY", [w], [float(rng.uniform(0, TWO_PI))], False))
            ops.append(("RZ", [w], [float(rng.uniform(0, TWO_PI))], False))
        for w in range(n - 1):
            ops.append(("CZ", [w, w + 1], [], False))
    return ops


def sum_z_hamiltonian(n):
    return [(1.0, "Z", [w]) for w in range(n)]


def random_state(n, rng, dtype=np.complex128):
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    v /= np.linalg.norm(v)
    return v.astype(dtype)


def sum_z_hamiltonian_terms(n):
    """sum_i Z_i as (coeff, word, wires) terms."""
    return [(1.0, "Z", [w]) for w in range(n)]


def circuit_28q_workload(n=28, seed=11, layers=20):
    """The 28-qubit circuit workload at any width n: `layers` layers of 28
    random rotations (RX/RY/RZ/Rot) and 14 random CNOT/CZ/CRY (840 operations
    for 20 layers, whatever n is), then a 100-term random Pauli Hamiltonian
    (1..6 wires per word, N(0, 1) coefficients).  n = 28 with seed 11 is the
    benchmarked instance; smaller n keep the operation count for oracle
    comparisons."""
    rng = np.random.default_rng(seed)
    ops = random_circuit(n, layers, rng, rot_per_layer=28, ent_per_layer=14)
    terms = random_pauli_hamiltonian(n, 100, rng, max_wires=6)
    return ops, terms


def adjoint_24q_workload(n=24, layers=8, seed=13):
    """The differentiation workload: RY, RZ on every wire plus a CZ ladder per
    layer (2 n layers parameters: 384 at n = 24, 8 layers), a 50-term random
    Pauli Hamiltonian and uniform angles, all from one seed."""
    rng = np.random.default_rng(seed)
    terms = random_pauli_hamiltonian(n, 50, rng, max_wires=6)
    params = rng.uniform(0, TWO_PI, 2 * n * layers)
    return terms, params
