"""torch.autograd adjoint against central differences and the oracle adjoint.

Tolerances: adjoint vs central differences (h = 1e-4, complex128) 1e-7;
adjoint vs the oracle's adjoint 1e-10.
"""
import numpy as np
import pytest

from pennylane_lightning_gpu_gb300 import workloads

pytestmark = pytest.mark.gpu


def test_autograd_matches_fd_and_oracle(oracle):
    torch = pytest.importorskip("torch")
    from pennylane_lightning_gpu_gb300.lightning_gpu import LightningGPU
    from pennylane_lightning_gpu_gb300 import torch_adjoint as TA

    n, layers = 8, 3
    rng = np.random.default_rng(3)
    terms = workloads.random_pauli_hamiltonian(n, 12, rng, max_wires=4)
    H = TA.pauli_hamiltonian(terms)
    template = TA.ry_rz_cz_template(n, layers)
    dev = LightningGPU(n)
    f = TA.expval_function(template, [H], dev)
    p = torch.tensor(rng.uniform(0, 2 * np.pi, 2 * n * layers), dtype=torch.float64, requires_grad=True)
    y = f(p)
    y.sum().backward()
    grad = p.grad.numpy()
    fd = TA.central_differences(template, [H], dev, p.detach().numpy(), h=1e-4)[0]
    assert np.max(np.abs(grad - fd)) < 1e-7
    # oracle adjoint on the same ops and observable
    ops = template(p.detach().numpy())
    oops = [(o.name, o.wires, o.parameters, False, None) for o in ops]
    final = oracle.run(n, oops)
    obs = [(True, [(c, [(("Pauli" + ch) if ch != "I" else "Identity", [w], None) for ch, w in zip(word, wires)])
                   for c, word, wires in terms])]
    ref = oracle.adjoint_jacobian(final, oops, obs, list(range(p.numel())))[0]
    assert np.max(np.abs(grad - ref)) < 1e-10


def test_autograd_multiple_outputs_vjp():
    torch = pytest.importorskip("torch")
    from pennylane_lightning_gpu_gb300 import ops as Q
    from pennylane_lightning_gpu_gb300 import torch_adjoint as TA
    from pennylane_lightning_gpu_gb300.lightning_gpu import LightningGPU

    n = 4
    template = TA.ry_rz_cz_template(n, 2)
    obs = [Q.PauliZ(0), Q.PauliX(2) @ Q.PauliZ(3)]
    dev = LightningGPU(n)
    f = TA.expval_function(template, obs, dev)
    p = torch.tensor(np.linspace(0.1, 1.5, 16), dtype=torch.float64, requires_grad=True)
    y = f(p)
    w = torch.tensor([0.3, -1.7], dtype=torch.float64)
    (y * w).sum().backward()
    jac = TA.central_differences(template, obs, dev, p.detach().numpy())
    assert np.allclose(p.grad.numpy(), w.numpy() @ jac, atol=1e-7)
