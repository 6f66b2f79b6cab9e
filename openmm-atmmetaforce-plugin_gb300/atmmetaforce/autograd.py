"""torch.autograd.Function over the ATM softplus bias energy W.

``atm_softplus_energy(batch, positions, displacements, params, charge, sigma,
epsilon)`` returns W_r for every replica of a ReplicaBatch created with
``{"DifferencePath": 1, "Adjoint": 1}``; its backward pass is the hand-written
adjoint kernel of the library (dW/dx = -s W'(u) (F2 - F1), dW/dd = -s W'(u) F2,
dW/d{q, sigma, eps} from the difference tiles, the exception corrections and
the reciprocal potentials; closed-form dW/d{lambda1, lambda2, alpha, u0, w0}).
Pair terms are recomputed in the evaluation, never stored.

Shapes (N = atoms of all replicas back to back, R = replicas), float64 on the
batch's CUDA device:
    positions, displacements: (N, 3); params: (R, 5); charge, sigma, epsilon: (N,)
The W of the reference is ReferenceATMMetaForceKernels.cpp:88-95; the merge
energy E = e0 + W is available through ReplicaBatch.evaluate.
"""
from __future__ import annotations

import numpy as np
import torch

from ._lib import NUM_RES

RES_W = 3
PARAM_NAMES5 = ("ATMLambda1", "ATMLambda2", "ATMAlpha", "ATMU0", "ATMW0")


class _ATMSoftplusEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, positions, displacements, params, charge, sigma, epsilon, batch, cache):
        R, offs = batch.R, batch.offsets
        d_np = displacements.detach().cpu().numpy()
        p_np = params.detach().cpu().numpy()
        q_np = charge.detach().cpu().numpy()
        s_np = sigma.detach().cpu().numpy()
        e_np = epsilon.detach().cpu().numpy()
        for r in range(R):
            a, b = offs[r], offs[r + 1]
            key_d = d_np[a:b].tobytes()
            if cache.get(("d", r)) != key_d:
                batch.setDisplacements(r, d_np[a:b])
                cache[("d", r)] = key_d
            key_p = q_np[a:b].tobytes() + s_np[a:b].tobytes() + e_np[a:b].tobytes()
            if cache.get(("p", r)) != key_p:
                batch.setNonbondedParameters(r, q_np[a:b], s_np[a:b], e_np[a:b])
                cache[("p", r)] = key_p
            for k, name in enumerate(PARAM_NAMES5):
                batch.setParameter(r, name, float(p_np[r, k]))
        pos = positions.detach().contiguous()
        forces = torch.empty_like(pos)
        results = torch.empty((R, NUM_RES), dtype=torch.float64, device=pos.device)
        stream = torch.cuda.current_stream(pos.device).cuda_stream
        batch.evaluateDevice(pos.data_ptr(), forces.data_ptr(), results.data_ptr(), stream)
        ctx.batch = batch
        ctx.shapes = (positions.shape, R)
        return results[:, RES_W].clone()

    @staticmethod
    def backward(ctx, gW):
        batch = ctx.batch
        pshape, R = ctx.shapes
        dev = gW.device
        g = gW.detach().to(torch.float64).contiguous()
        N = pshape[0]
        dx = torch.empty((N, 3), dtype=torch.float64, device=dev)
        dd = torch.empty((N, 3), dtype=torch.float64, device=dev)
        dq = torch.empty((N,), dtype=torch.float64, device=dev)
        ds = torch.empty((N,), dtype=torch.float64, device=dev)
        de = torch.empty((N,), dtype=torch.float64, device=dev)
        dp = torch.empty((R, 5), dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        batch.backwardDevice(g.data_ptr(), dx.data_ptr(), dd.data_ptr(), dq.data_ptr(), ds.data_ptr(),
                             de.data_ptr(), dp.data_ptr(), stream)
        return dx, dd, dp, dq, ds, de, None, None


def atm_softplus_energy(batch, positions, displacements, params, charge, sigma, epsilon):
    """W per replica (R,), differentiable with respect to every tensor argument."""
    cache = getattr(batch, "_autograd_cache", None)
    if cache is None:
        cache = {}
        batch._autograd_cache = cache
    return _ATMSoftplusEnergy.apply(positions, displacements, params, charge, sigma, epsilon, batch, cache)


def batch_tensors(batch, cases, device="cuda"):
    """Initial (positions, displacements, params, charge, sigma, epsilon) tensors
    of a batch built from synthetic cases, float64 on ``device``."""
    cat = lambda xs: torch.as_tensor(np.ascontiguousarray(np.concatenate(xs)), dtype=torch.float64, device=device)
    pos = cat([c.pos for c in cases])
    displ = cat([c.displ for c in cases])
    params = torch.as_tensor(np.stack([c.params[:5] for c in cases]), dtype=torch.float64, device=device)
    q = cat([c.spec.charge for c in cases])
    s = cat([c.spec.sigma for c in cases])
    e = cat([c.spec.epsilon for c in cases])
    return pos, displ, params, q, s, e
