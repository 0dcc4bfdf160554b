"""Time propagation on the GPU against the oracle: RK4 (td/intstp.f90) and Chebyshev
(td/chebyshev.f90) steps of the sparse derivative (calcderiv_spa_omp) under a step bias
switched on at t = 0+, with the lead currents of td/calcj.f90 at every step."""
import numpy as np
import pytest

import configs as cf
import heomq
import oracle_ffi as of

pytestmark = pytest.mark.gpu

CASES = {"siam_L2": cf.siam(ntier=3, nmats=2), "dqd_L2": cf.dqd(ntier=3, nmats=2),
         "siam_L2_onset": cf.siam(ntier=3, nmats=2, tchar=0.3)}


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("name", sorted(CASES))
def test_rk4_matches_oracle(name):
    cfg = CASES[name]
    m, ref = heomq.Model(cfg), of.Model(cfg)
    ctx = heomq.Context(m)
    rho0 = m.initial_guess()
    dt, nstep = 0.05, 6
    rho, jt = ctx.propagate(rho0, 0.0, dt, nstep, method=heomq.PROP_RK4, currents=True)
    r = rho0.copy()
    for n in range(nstep):
        np.testing.assert_allclose(jt[n], ref.current(r).T.reshape(-1), rtol=1e-11, atol=1e-9)
        r = ref.rk4_step(n * dt, dt, r)
    assert _rel(rho, r) < 1e-12


@pytest.mark.parametrize("name", sorted(CASES))
def test_chebyshev_matches_oracle(name):
    cfg = CASES[name]
    m, ref = heomq.Model(cfg), of.Model(cfg)
    ctx = heomq.Context(m)
    rho0 = m.initial_guess()
    dt, nstep = 0.05, 4
    delta = ref.cheby_delta()
    nterms = of.cheby_nterms(delta, dt)
    rho, jt = ctx.propagate(rho0, 0.0, dt, nstep, method=heomq.PROP_CHEBYSHEV, currents=True)
    r = rho0.copy()
    for n in range(nstep):
        np.testing.assert_allclose(jt[n], ref.current(r).T.reshape(-1), rtol=1e-11, atol=1e-9)
        r = ref.cheby_step(n * dt, delta, nterms, dt, r)
    assert _rel(rho, r) < 1e-11


def test_long_chebyshev_run_relaxes_to_the_steady_state():
    """After the bias step the current relaxes to the TFQMR steady-state value."""
    cfg = cf.siam(ntier=3, nmats=2, V=0.4)
    m = heomq.Model(cfg)
    ctx = heomq.Context(m)
    rho_ss, _ = ctx.solve_tfqmr(crit=1e-10)
    rho, jt = ctx.propagate(m.initial_guess(), 0.0, 0.05, 800, method=heomq.PROP_CHEBYSHEV, currents=True)
    i_ss = ctx.current(rho_ss)[0].sum()
    i_t = ctx.current(rho)[0].sum()
    assert abs(i_t / i_ss - 1) < 1e-3


@pytest.mark.parametrize("method", [heomq.PROP_RK4, heomq.PROP_CHEBYSHEV], ids=["rk4", "chebyshev"])
def test_full_size_propagation_buffers(method):
    """The double dot at tier 4 (393 812 entries): the device buffers of a propagation with
    current recording are laid out without overlap (the recorded first-step current equals
    the host current of the initial state, and the run completes)."""
    m = heomq.Model(cf.CFG1)
    ctx = heomq.Context(m, adjoint=False)
    rho0 = m.initial_guess()
    rho, jt = ctx.propagate(rho0, 0.0, 0.05, 3, method=method, currents=True)
    np.testing.assert_allclose(jt[0], ctx.current(rho0).T.reshape(-1), rtol=1e-12, atol=1e-9)
    assert np.isfinite(rho).all() and np.isfinite(jt).all()


@pytest.mark.parametrize("name", sorted(CASES))
def test_mixed_chebyshev_follows_the_fp64_one(name):
    """HEOM_PROP_CHEBYSHEV_MIXED (state, recurrence and applies in FP32x2) against the FP64
    Chebyshev run over 400 steps of 0.05: states within 1e-11 relative, currents within 1e-10
    of the largest."""
    m = heomq.Model(CASES[name])
    ctx = heomq.Context(m)
    rho0 = m.initial_guess()
    r64, j64 = ctx.propagate(rho0, 0.0, 0.05, 400, method=heomq.PROP_CHEBYSHEV, currents=True)
    rmx, jmx = ctx.propagate(rho0, 0.0, 0.05, 400, method=heomq.PROP_CHEBYSHEV_MIXED, currents=True)
    assert _rel(rmx, r64) <= 1e-11, _rel(rmx, r64)
    assert _rel(jmx, j64) <= 1e-10, _rel(jmx, j64)


def test_mixed_chebyshev_at_full_size():
    """The gradient configuration's model (double dot, tier 4, M = 3) from the V = 0 steady
    state under the step bias: 1 000 mixed Chebyshev steps of 0.05 against the FP64 ones,
    currents within 1e-9 of the largest and the time integral within 1e-10."""
    cfg = cf.dqd(ntier=5, nmats=3, V=0.8)
    m0 = heomq.Model(cf.dqd(ntier=5, nmats=3, V=0.0))
    c0 = heomq.Context(m0, adjoint=False)
    rho_eq, info = c0.solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
    assert info.converged
    m = heomq.Model(cfg)
    ctx = heomq.Context(m, adjoint=False)
    _, j64 = ctx.propagate(rho_eq, 0.0, 0.05, 1000, method=heomq.PROP_CHEBYSHEV, currents=True)
    _, jmx = ctx.propagate(rho_eq, 0.0, 0.05, 1000, method=heomq.PROP_CHEBYSHEV_MIXED, currents=True)
    assert _rel(jmx, j64) <= 1e-9, _rel(jmx, j64)
    i64, imx = j64[:, 0::m.nalf].sum(), jmx[:, 0::m.nalf].sum()
    assert abs(imx / i64 - 1) <= 1e-10

