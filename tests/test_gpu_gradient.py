"""Adjoint steady-state sensitivities of the lead-1 current against central finite
differences.  Steady states are refined to a residual of 1e-12, which leaves about 1e-11
relative noise in the current; the steady-state differences therefore use h = 1e-4 (the
truncation error h^2 stays near 1e-8) so that the noise of (I+ - I-)/2h stays well below the
1e-6 bar.  The time-dependent runs are deterministic and use h = 1e-5."""
import numpy as np
import pytest

import configs as cf
import heomq

pytestmark = pytest.mark.gpu

HB = 0.658211928
BASE = {"siam_L2": dict(kind="siam", ntier=3, nmats=2), "dqd_L2": dict(kind="dqd", ntier=3, nmats=2)}
PARAMS = {"siam": dict(V=0.6, U=2.0, eps=-0.7, gamma=0.5), "dqd": dict(V=0.8, U=2.0, eps=-0.8, gamma=0.5)}


def make_cfg(name, **over):
    b = dict(BASE[name])
    kind = b.pop("kind")
    p = dict(PARAMS[kind])
    p.update(over)
    return (cf.siam if kind == "siam" else cf.dqd)(**b, **p)


def steady_current(cfg):
    m = heomq.Model(cfg)
    ctx = heomq.Context(m)
    rho, info = ctx.solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
    assert info.converged
    return ctx.current(rho)[0].sum()


@pytest.mark.parametrize("name", sorted(BASE))
def test_adjoint_gradient_matches_central_differences(name):
    kind = BASE[name]["kind"]
    p0 = PARAMS[kind]
    cfg = make_cfg(name)
    m = heomq.Model(cfg)
    ctx = heomq.Context(m, dhs=(m.get("dhs_du", m.nrho ** 2, np.complex128), m.get("dhs_deps", m.nrho ** 2, np.complex128)))
    rho, info = ctx.solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
    assert info.converged
    # d eleadinfty / dV: +1/2 for lead 1, -1/2 for lead 2, in the operator's units (1/hbar)
    deshift = np.array([[0.5, 0.5], [-0.5, -0.5]]).T.reshape(-1) / HB
    dI, ainfo = ctx.steady_gradient(rho, deshift=deshift, gamma=p0["gamma"],
                                    dhs_du=m.get("dhs_du", m.nrho ** 2, np.complex128),
                                    dhs_deps=m.get("dhs_deps", m.nrho ** 2, np.complex128), which=0xF, crit=1e-12)
    for k, key in enumerate(("V", "gamma", "U", "eps")):
        h = 1e-4 * max(1.0, abs(p0[key]))
        if key == "gamma":
            ip = steady_current(make_cfg(name, gamma=p0[key] + h))
            im = steady_current(make_cfg(name, gamma=p0[key] - h))
        else:
            ip = steady_current(make_cfg(name, **{key: p0[key] + h}))
            im = steady_current(make_cfg(name, **{key: p0[key] - h}))
        fd = (ip - im) / (2 * h)
        assert abs(dI[k] - fd) <= 1e-6 * max(abs(fd), 1e-3 * abs(ip)), (key, dI[k], fd)


@pytest.mark.parametrize("name", sorted(BASE))
def test_mixed_adjoint_solve_gives_the_fp64_gradients(name):
    """The adjoint solve in mixed precision (FP32x2 TFQMR rounds on the regularised adjoint,
    FP64 refinement to the same tolerance) against the FP64 adjoint solve: dI/d{V, Gamma, U,
    eps} within 1e-8 relative (of the largest)."""
    p0 = PARAMS[BASE[name]["kind"]]
    m = heomq.Model(make_cfg(name))
    du, de = m.get("dhs_du", m.nrho ** 2, np.complex128), m.get("dhs_deps", m.nrho ** 2, np.complex128)
    ctx = heomq.Context(m, dhs=(du, de))
    rho, info = ctx.solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
    assert info.converged
    deshift = np.array([[0.5, 0.5], [-0.5, -0.5]]).T.reshape(-1) / HB
    kw = dict(deshift=deshift, gamma=p0["gamma"], dhs_du=du, dhs_deps=de, which=0xF, crit=1e-12)
    d64, i64 = ctx.steady_gradient(rho, precision=heomq.PREC_FP64, **kw)
    dmx, imx = ctx.steady_gradient(rho, precision=heomq.PREC_MIXED, **kw)
    assert imx.converged and imx.resid <= i64.resid * 10 + 1e-300 or imx.converged
    assert np.max(np.abs(dmx - d64)) <= 1e-8 * np.max(np.abs(d64)), (dmx, d64)


def test_adjoint_identity_of_the_regularised_solve():
    """<c, x_theta> from a forward tangent solve equals the adjoint value."""
    cfg = make_cfg("siam_L2")
    m = heomq.Model(cfg)
    ctx = heomq.Context(m)
    rho, _ = ctx.solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
    deshift = np.array([[0.5, 0.5], [-0.5, -0.5]]).T.reshape(-1) / HB
    d1, _ = ctx.steady_gradient(rho, deshift=deshift, which=1, crit=1e-12)
    d2, _ = ctx.steady_gradient(rho, deshift=2 * deshift, which=1, crit=1e-12)
    assert abs(d2[0] - 2 * d1[0]) <= 1e-10 * abs(d1[0])


@pytest.mark.parametrize("name, nstep, ck", [("siam_L2", 64, 16), ("dqd_L2", 40, 8)])
def test_td_gradient_matches_central_differences(name, nstep, ck):
    """d/dA of J = dt sum_n I_1(rho_n) for a Chebyshev run from the V = 0 steady state
    under the step bias A * (+-V/2), by the checkpointed reverse pass, against central
    differences of two forward runs (h = 1e-5)."""
    dt = 0.05
    cfg0 = make_cfg(name, V=0.0)
    m0 = heomq.Model(cfg0)
    ctx0 = heomq.Context(m0)
    rho_eq, _ = ctx0.solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
    cfg = make_cfg(name)
    m = heomq.Model(cfg)
    amps, tchar = m.field()
    ctx = heomq.Context(m)
    J, dJ = ctx.td_gradient(rho_eq, dt, nstep, checkpoint_every=ck)

    def integral(scale):
        c = heomq.Context(m, adjoint=False, amps=scale * amps, tchar=tchar)
        _, jt = c.propagate(rho_eq, 0.0, dt, nstep, method=heomq.PROP_CHEBYSHEV, currents=True)
        return dt * jt[:, 0::m.nalf].sum()

    assert abs(J / integral(1.0) - 1) < 1e-12
    h = 1e-5
    fd = (integral(1 + h) - integral(1 - h)) / (2 * h)
    assert abs(dJ - fd) <= 1e-6 * abs(fd), (dJ, fd)
    # through FP32x2 steps: the same integral and gradient to about 48-bit accumulation
    Jm, dJm = ctx.td_gradient(rho_eq, dt, nstep, checkpoint_every=ck, method=heomq.PROP_CHEBYSHEV_MIXED)
    assert abs(Jm / J - 1) < 1e-11 and abs(dJm / dJ - 1) < 1e-10, (Jm, J, dJm, dJ)


def test_autograd_wrappers_match_the_entry_points():
    import torch

    from heomq import autograd as hag

    theta = torch.tensor([0.6, 0.5, 2.0, -0.7], dtype=torch.float64, requires_grad=True)
    base = dict(ntier=3, nmats=2)
    current = hag.steady_current(theta, "siam", **base)
    current.backward()
    h = 1e-4
    for k in range(4):
        tp, tm = theta.detach().clone(), theta.detach().clone()
        tp[k] += h
        tm[k] -= h
        fd = (hag.steady_current(tp, "siam", **base) - hag.steady_current(tm, "siam", **base)).item() / (2 * h)
        assert abs(theta.grad[k].item() - fd) <= 1e-6 * max(abs(fd), 1e-3 * abs(current.item()))
    m0 = heomq.Model(make_cfg("siam_L2", V=0.0))
    rho_eq, _ = heomq.Context(m0).solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
    m = heomq.Model(make_cfg("siam_L2"))
    amp = torch.tensor(1.3, dtype=torch.float64, requires_grad=True)
    J = hag.chebyshev_current_integral(amp, m, rho_eq, 0.05, 40, 8)
    J.backward()
    h = 1e-5
    jp = hag.chebyshev_current_integral(torch.tensor(1.3 + h, dtype=torch.float64), m, rho_eq, 0.05, 40, 8).item()
    jm = hag.chebyshev_current_integral(torch.tensor(1.3 - h, dtype=torch.float64), m, rho_eq, 0.05, 40, 8).item()
    assert abs(amp.grad.item() - (jp - jm) / (2 * h)) <= 1e-6 * abs((jp - jm) / (2 * h))


def test_full_size_gradients_match_central_differences():
    """The adjoint gradients at the size of the gradient configuration: the serial double dot
    at tier 4 with Pade M = 3 (393 812 entries).  Steady dI_L/d{V, Gamma, U} against central
    differences (h = 1e-4, steady states refined to 1e-12) within 1e-6; the gradient of
    int I_L dt over 1000 Chebyshev steps of 0.05 from the V = 0 steady state under the step
    bias 0.8, with checkpoints every 32 steps (td/chebyshev.f90:160-200 run backwards),
    against central differences of two forward runs (h = 1e-5) within 1e-6."""
    p0 = dict(V=0.8, gamma=0.5, U=2.0, eps=-1.0)

    def cfg(**over):
        p = dict(p0)
        p.update(over)
        return cf.dqd(ntier=5, nmats=3, **p)

    def current(c):
        ctx = heomq.Context(heomq.Model(c), adjoint=False)
        rho, info = ctx.solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
        assert info.converged
        return ctx.current(rho)[0].sum()

    m = heomq.Model(cfg())
    du, de = m.get("dhs_du", m.nrho ** 2, np.complex128), m.get("dhs_deps", m.nrho ** 2, np.complex128)
    ctx = heomq.Context(m, dhs=(du, de))
    rho, info = ctx.solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
    assert info.converged
    deshift = np.array([[0.5, 0.5], [-0.5, -0.5]]).T.reshape(-1) / HB
    dI, _ = ctx.steady_gradient(rho, deshift=deshift, gamma=p0["gamma"], dhs_du=du, dhs_deps=de, which=0xF, crit=1e-12)
    dmx, imx = ctx.steady_gradient(rho, deshift=deshift, gamma=p0["gamma"], dhs_du=du, dhs_deps=de, which=0xF, crit=1e-12,
                                   precision=heomq.PREC_MIXED)
    assert imx.converged
    assert np.max(np.abs(dmx - dI)) <= 1e-8 * np.max(np.abs(dI)), (dmx, dI)
    for k, key in enumerate(("V", "gamma", "U")):
        h = 1e-4 * max(1.0, abs(p0[key]))
        fd = (current(cfg(**{key: p0[key] + h})) - current(cfg(**{key: p0[key] - h}))) / (2 * h)
        assert abs(dI[k] - fd) <= 1e-6 * abs(fd), (key, dI[k], fd)
    ctx.close()

    c0 = heomq.Context(heomq.Model(cfg(V=0.0)), adjoint=False)
    rho_eq, _ = c0.solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
    amps, tchar = m.field()
    ctx = heomq.Context(m)
    J, dJ = ctx.td_gradient(rho_eq, 0.05, 1000, checkpoint_every=32)

    def integral(scale):
        c = heomq.Context(m, adjoint=False, amps=scale * amps, tchar=tchar)
        _, jt = c.propagate(rho_eq, 0.0, 0.05, 1000, method=heomq.PROP_CHEBYSHEV, currents=True)
        return 0.05 * jt[:, 0::m.nalf].sum()

    assert abs(J / integral(1.0) - 1) < 1e-12
    fd = (integral(1 + 1e-5) - integral(1 - 1e-5)) / 2e-5
    assert abs(dJ - fd) <= 1e-6 * abs(fd), (dJ, fd)
    # the same gradient through FP32x2 Chebyshev steps (forward and reverse)
    Jm, dJm = ctx.td_gradient(rho_eq, 0.05, 1000, checkpoint_every=32, method=heomq.PROP_CHEBYSHEV_MIXED)
    assert abs(Jm / J - 1) < 1e-10 and abs(dJm / dJ - 1) < 1e-9, (Jm, J, dJm, dJ)
