"""torch.autograd wrappers of the adjoint sensitivities.

SteadyCurrent: theta = (V, Gamma, U, eps) -> lead-1 steady current, with the gradient of
heom_steady_gradient (adjoint solve with the transpose apply).
ChebyshevCurrentIntegral: bias amplitude A -> J = dt sum_n I_1(rho_n) of a Chebyshev run,
with the gradient of heom_td_gradient (reverse pass with checkpoints).

The forward passes run the GPU solver / propagator through the C ABI; torch only carries
the scalars.
"""
import numpy as np
import torch

from . import PREC_FP64_REFINED, Context, Model
from . import models

HBAR = 0.658211928


def _model_for(kind, base, theta):
    V, gamma, U, eps = (float(t) for t in theta)
    build = models.siam if kind == "siam" else models.dqd
    return Model(build(**base, V=V, gamma=gamma, U=U, eps=eps))


class SteadyCurrent(torch.autograd.Function):
    """I_1(theta) for theta = (V, Gamma, U, eps) of the single-orbital ("siam") or double-dot
    ("dqd") model; `base` holds the remaining model arguments (ntier, nmats, T, W, ...)."""

    @staticmethod
    def forward(ctx, theta, kind, base, crit=1e-12):
        th = theta.detach().cpu().numpy().astype(np.float64)
        m = _model_for(kind, base, th)
        nd2 = m.nrho ** 2
        dhs_du = m.get("dhs_du", nd2, np.complex128)
        dhs_deps = m.get("dhs_deps", nd2, np.complex128)
        c = Context(m, dhs=(dhs_du, dhs_deps))
        rho, info = c.solve_tfqmr(crit=crit, precision=PREC_FP64_REFINED, max_refine=16)
        if not info.converged:
            raise RuntimeError("steady state did not converge")
        current = c.current(rho)[0].sum()
        deshift = np.array([[0.5, 0.5], [-0.5, -0.5]]).T.reshape(-1) / HBAR
        dI, _ = c.steady_gradient(rho, deshift=deshift, gamma=float(th[1]), dhs_du=dhs_du, dhs_deps=dhs_deps,
                                  which=0xF, crit=crit)
        ctx.save_for_backward(torch.as_tensor(dI, dtype=theta.dtype, device=theta.device))
        return torch.as_tensor(current, dtype=theta.dtype, device=theta.device)

    @staticmethod
    def backward(ctx, grad_out):
        (dI,) = ctx.saved_tensors
        return grad_out * dI, None, None, None


class ChebyshevCurrentIntegral(torch.autograd.Function):
    """J(A) = dt sum_n I_1(rho_n) for nstep Chebyshev steps from rho0 under the model's
    bias pulse scaled by A (A != 0; the derivative is taken at the given A)."""

    @staticmethod
    def forward(ctx, amp, model, rho0, dt, nstep, checkpoint_every=32):
        a = float(amp.detach().cpu())
        if a == 0.0:
            raise ValueError("the bias amplitude must be nonzero (the derivative is taken along its scale)")
        amps, tchar = model.field()
        c = Context(model, amps=a * amps, tchar=tchar)
        # heom_td_gradient differentiates along the scale s of the context's pulse a * amps:
        # dJ/da = (dJ/ds) / a
        J, dJs = c.td_gradient(rho0, dt, nstep, checkpoint_every=checkpoint_every)
        dJ = dJs / a
        ctx.save_for_backward(torch.as_tensor(dJ, dtype=amp.dtype, device=amp.device))
        return torch.as_tensor(J, dtype=amp.dtype, device=amp.device)

    @staticmethod
    def backward(ctx, grad_out):
        (dJ,) = ctx.saved_tensors
        return grad_out * dJ, None, None, None, None, None


def steady_current(theta, kind="siam", crit=1e-12, **base):
    return SteadyCurrent.apply(theta, kind, base, crit)


def chebyshev_current_integral(amp, model, rho0, dt, nstep, checkpoint_every=32):
    return ChebyshevCurrentIntegral.apply(amp, model, rho0, dt, nstep, checkpoint_every)
