"""torch.autograd integration: expectation values of a parameterised circuit as
a differentiable torch function whose backward pass is the engine's fused
adjoint-Jacobian sweep (one vector-Jacobian product per backward call, built
from the combined observable sum_k dy_k O_k as in the reference's vjp,
lightning_gpu.py:771-810).

    f = expval_function(template, observables, device)
    y = f(params)            # torch tensor, one value per observable
    y.sum().backward()       # params.grad via the adjoint method

``template(params_numpy) -> list of ops`` must consume the parameters in
order, one per parametric operation (Rot counts three).
"""
import numpy as np
import torch

from . import ops as Q


class AdjointExpval(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, template, observables, device):
        p = params.detach().to("cpu", torch.float64).numpy()
        tape = Q.QuantumTape(template(p), [Q.expval(o) for o in observables])
        res = np.asarray(device.execute(tape), dtype=np.float64)
        ctx.device = device
        ctx.tape = tape
        ctx.nparams = p.size
        # device copy of the final state: the backward sweep starts from it
        # instead of applying the circuit again
        ctx.final = type(device._gpu_state)(device._gpu_state)
        ctx.save_for_backward(params)
        return torch.as_tensor(res, dtype=params.dtype, device=params.device)

    @staticmethod
    def backward(ctx, grad_out):
        (params,) = ctx.saved_tensors
        dy = grad_out.detach().to("cpu", torch.float64).numpy().reshape(-1)
        ctx.device._gpu_state.copyFrom(ctx.final)
        ctx.final = None
        vjp = np.asarray(ctx.device.vjp(ctx.tape.measurements, dy, use_device_state=True)(ctx.tape),
                         dtype=np.float64)
        if vjp.size != ctx.nparams:
            raise RuntimeError("the template must use each parameter exactly once, in order")
        return torch.as_tensor(vjp, dtype=params.dtype, device=params.device), None, None, None


def expval_function(template, observables, device):
    """Differentiable f(params) -> torch tensor of expectation values."""

    def f(params):
        return AdjointExpval.apply(params, template, observables, device)

    return f


def central_differences(template, observables, device, params, h=1e-4, indices=None):
    """Central-difference Jacobian (rows: observables, columns: `indices`)."""
    p0 = np.asarray(params, dtype=np.float64)
    idx = range(p0.size) if indices is None else list(indices)
    cols = []
    for i in idx:
        e = np.zeros_like(p0)
        e[i] = h
        plus = device.execute(Q.QuantumTape(template(p0 + e), [Q.expval(o) for o in observables]))
        minus = device.execute(Q.QuantumTape(template(p0 - e), [Q.expval(o) for o in observables]))
        cols.append((np.asarray(plus) - np.asarray(minus)) / (2 * h))
    return np.stack(cols, axis=1)


def ry_rz_cz_template(n, layers):
    """RY, RZ on every wire then a CZ ladder, per layer (2 n layers params)."""

    def template(p):
        ops = []
        k = 0
        for _ in range(layers):
            for w in range(n):
                ops.append(Q.op("RY", w, p[k]))
                ops.append(Q.op("RZ", w, p[k + 1]))
                k += 2
            for w in range(n - 1):
                ops.append(Q.op("CZ", [w, w + 1]))
        return ops

    return template


def pauli_hamiltonian(terms):
    """(coeff, word, wires) terms -> ops.Hamiltonian of Pauli words."""
    names = {"X": Q.PauliX, "Y": Q.PauliY, "Z": Q.PauliZ, "I": Q.Identity}
    obs = []
    for _, word, wires in terms:
        factors = [names[c](w) for c, w in zip(word, wires)]
        obs.append(factors[0] if len(factors) == 1 else Q.Tensor(*factors))
    return Q.Hamiltonian([t[0] for t in terms], obs)
