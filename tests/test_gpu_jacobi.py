"""GPU parity of the Jacobi steady-state iteration (jacobi/) against the oracle.

The device sweep diagonalises H instead of the Liouvillian; one sweep must still agree with
the oracle's restatement of calc_ax_jacobi_spa_omp (Liouville-space eigenvectors) to rounding,
and the solve must reach the TFQMR steady state.
"""
import numpy as np
import pytest

import configs as cf
import heomq
import oracle_ffi as of

pytestmark = pytest.mark.gpu

CASES = {"siam_L2": cf.siam(ntier=3), "siam_L3": cf.CFG0, "dqd_L2": cf.dqd(ntier=3)}


@pytest.fixture(scope="module", params=list(CASES))
def setup(request):
    cfg = CASES[request.param]
    m = heomq.Model(cfg)
    return request.param, m, heomq.Context(m, adjoint=False), of.Model(cfg)


def test_shift_matches_the_reference_rule(setup):
    name, m, ctx, ref = setup
    assert abs(ctx.jacobi_shift() / of.Jacobi(ref).ejac - 1) < 1e-12, name


def test_one_sweep_matches_oracle(setup):
    """maxit0 = 0 stops after sweep 0; the input RDO is Hermitian, so the solver's
    Hermitisation leaves it unchanged."""
    name, m, ctx, ref = setup
    x = m.initial_guess()
    nz0 = int(m.array("nnz_spa")[0])
    r = np.random.default_rng(11)
    x[nz0:] = 1e-2 * (r.standard_normal(m.lunk - nz0) + 1j * r.standard_normal(m.lunk - nz0))
    J = of.Jacobi(ref)
    for ejac in (J.ejac, 3.0 * J.ejac):
        got, _ = ctx.solve_jacobi(x, crit=0.0, maxit0=0, ejac=ejac, check=False)
        want = of.Jacobi(ref, ejac=ejac).sweep(x)
        assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want), (name, ejac)


@pytest.mark.parametrize("name", ["siam_L3", "dqd_L2"])
def test_jacobi_solve_reaches_the_steady_state(name):
    m = heomq.Model(CASES[name])
    ctx = heomq.Context(m, adjoint=False)
    ejac = 2 * ctx.jacobi_shift()
    rho, info = ctx.solve_jacobi(crit=1e-10, maxit0=40000, ejac=ejac)
    assert info.converged and info.resid <= 1e-10
    ref, _ = ctx.solve_tfqmr(crit=1e-12, maxit0=40000, precision=heomq.PREC_FP64_REFINED, max_refine=16)
    assert abs(ctx.current(rho)[0].sum() / ctx.current(ref)[0].sum() - 1) < 1e-8
    if name != "siam_L3":
        return
    # the oracle's own Jacobi solve from the same start stops within a few sweeps of the device's
    o = of.Model(CASES[name])
    rho_o, info_o = of.Jacobi(o, ejac=ejac).solve(m.initial_guess(), crit=1e-10, maxit0=40000)
    assert abs(info_o.iters - info.iters) <= 50
    assert np.linalg.norm(rho - rho_o) <= 1e-8 * np.linalg.norm(rho_o)
