"""Gate generators against central differences of the gates themselves.

The reference checks each applyGenerator<Gate> against the generator matrix
applied directly (Test_Generators.cpp:19-1371); the adjoint method relies on
d/dtheta U(theta)|psi> = i s G U(theta)|psi>, with s the scale factor
returned with the generator (AdjointDiffGPU.hpp:58-114: -1/2 for rotations,
+1 for phase shifts).  Here that identity is checked for every parametric
gate: G from ``ApplyGeneratorOf`` on U(theta)|psi>, the derivative by central
differences of U (h = 1e-4, complex128, agreement 1e-7), on random states of
4 and 5 qubits and every target placement class (low, high, mixed wires).
"""
import zlib

import numpy as np
import pytest

from helpers import random_state

pytestmark = pytest.mark.gpu

GATES = [("RX", 1), ("RY", 1), ("RZ", 1), ("PhaseShift", 1), ("IsingXX", 2), ("IsingYY", 2), ("IsingZZ", 2),
         ("CRX", 2), ("CRY", 2), ("CRZ", 2), ("ControlledPhaseShift", 2), ("SingleExcitation", 2),
         ("SingleExcitationMinus", 2), ("SingleExcitationPlus", 2), ("DoubleExcitation", 4),
         ("DoubleExcitationMinus", 4), ("DoubleExcitationPlus", 4), ("MultiRZ", 3)]


def _applied(native, psi, name, wires, theta):
    sv = native.LightningGPU_C128(np.ascontiguousarray(psi, np.complex128))
    sv.apply(name, list(wires), False, [float(theta)], np.zeros(0, np.complex128))
    return sv


@pytest.mark.parametrize("n", [4, 5])
@pytest.mark.parametrize("name,k", GATES, ids=[g[0] for g in GATES])
def test_generator_is_the_derivative_of_the_gate(native, name, k, n):
    rng = np.random.default_rng(zlib.crc32(("%s/%d" % (name, n)).encode()))
    h = 1e-4
    placements = [list(range(k)), list(range(n - k, n)), list(rng.permutation(n)[:k])]
    for wires in placements:
        psi = random_state(n, rng)
        theta = float(rng.uniform(-np.pi, np.pi))
        plus = _applied(native, psi, name, wires, theta + h).GetState()
        minus = _applied(native, psi, name, wires, theta - h).GetState()
        fd = (plus - minus) / (2 * h)
        sv = _applied(native, psi, name, wires, theta)
        s = sv.ApplyGeneratorOf(name, list(wires), False)
        dev = 1j * s * sv.GetState()
        assert np.max(np.abs(dev - fd)) < 1e-7, (name, wires, np.max(np.abs(dev - fd)))
