"""The bench workload at full size, checked through properties that hold at any size.

Serial double dot, tier 4 (393 812 stored entries), 8 bias points in one batch, solved by
the mixed-precision refinement to crit 1e-9, as the benchmark does.  The batch is checked
through size-independent properties (the oracle solves one bias point of this size in
about two seconds on the host cores; that one is compared directly at the end):
- every steady state has unit trace and a Hermitian RDO;
- the current into the dot equals the current out (I_L = -I_R) to solver accuracy;
- the currents agree with the FP64 GPU solver and flow in the direction of the bias;
- the residual of every instance, recomputed by the apply, is at most crit."""
import numpy as np
import pytest

import heomq
import heomq.models as models

pytestmark = pytest.mark.gpu

HB = 0.658211928


def _batch():
    m = heomq.Model(models.dqd(ntier=5, nmats=3, V=0.8))
    ctx = heomq.Context(m, adjoint=False)
    Vs = [0.4 + 0.8 * b / 7 for b in range(8)]
    es = np.array([[V / 2, V / 2, -V / 2, -V / 2] for V in Vs]) / HB
    es = np.ascontiguousarray(es.reshape(8, 2, 2).transpose(0, 2, 1).reshape(8, 4))
    return m, ctx, Vs, es


def _rdo(m, rho):
    nz0 = int(m.array("nnz_spa")[0])
    ir, ic = m.array("irow_spa")[:nz0] - 1, m.array("icol_spa")[:nz0] - 1
    R = np.zeros((m.nrho, m.nrho), complex)
    R[ir, ic] = rho[:nz0]
    return R


def test_bench_batch_properties_at_full_size():
    m, ctx, Vs, es = _batch()
    rhos = np.tile(m.initial_guess(), (8, 1))
    mixed, info = ctx.solve_batch(rhos, eshift_batch=es, crit=1e-9, precision=heomq.PREC_MIXED)
    assert info.converged and info.resid <= 1e-9
    fp64, info64 = ctx.solve_batch(rhos, eshift_batch=es, crit=1e-9, precision=heomq.PREC_FP64)
    assert info64.resid <= 1e-9
    jm = np.array([ctx.current(mixed[b]) for b in range(8)])     # [b, ialf, ispin]
    jf = np.array([ctx.current(fp64[b]) for b in range(8)])
    for b in range(8):
        R = _rdo(m, mixed[b])
        assert abs(np.trace(R) - 1.0) <= 2e-9   # the trace row is part of the residual
        assert np.max(np.abs(R - R.conj().T)) <= 1e-12
    left, right = jm[:, 0, :].sum(axis=1), jm[:, 1, :].sum(axis=1)
    assert np.max(np.abs(left + right) / np.abs(left)) <= 1e-6
    assert np.max(np.abs(left - jf[:, 0, :].sum(axis=1)) / np.abs(left)) <= 1e-7
    assert np.all(left > 0)


def test_bench_batch_residuals_by_the_apply():
    """Each instance's ||e - A x|| recomputed through heom_calc_ax with that instance's lead
    shift (a context per bias point) stays at or below crit."""
    m, _, Vs, es = _batch()
    rhos = np.tile(m.initial_guess(), (8, 1))
    ctx = heomq.Context(m, adjoint=False)
    out, info = ctx.solve_batch(rhos, eshift_batch=es, crit=1e-9, precision=heomq.PREC_MIXED)
    for b in (0, 7):
        mb = heomq.Model(models.dqd(ntier=5, nmats=3, V=Vs[b]))
        cb = heomq.Context(mb, adjoint=False)
        x = np.zeros(mb.lunk + 1, complex)
        x[: mb.lunk] = out[b]
        r = cb.calc_ax_tfqmr_spa(x)
        r[-1] -= 1.0
        assert np.linalg.norm(r) <= 2e-9
        cb.close()


def test_headline_model_matches_the_oracle():
    """The headline model itself (double dot, tier 4, Pade M = 3, V = 0.8) against the oracle's
    FP64 TFQMR on all host cores: the GPU's FP64 solve at crit 1e-9 and its mixed-precision
    solve at crit 1e-10, currents per lead and spin within 1e-8 relative, occupations within
    1e-8 (the oracle's own current error at crit 1e-9 is about 3e-9)."""
    import oracle_ffi as of

    cfg = models.dqd(ntier=5, nmats=3, V=0.8)
    ref = of.Model(cfg)
    rho_ref, info_ref = ref.solve_tfqmr(crit=1e-9, maxit0=40000)
    j_ref, occ_ref = ref.current(rho_ref), ref.occupation(rho_ref)
    m = heomq.Model(cfg)
    ctx = heomq.Context(m, adjoint=False)
    for prec, crit in ((heomq.PREC_FP64, 1e-9), (heomq.PREC_MIXED, 1e-10)):
        rho, info = ctx.solve_tfqmr(crit=crit, precision=prec, maxit0=40000)
        assert info.converged and info.resid <= crit
        j = ctx.current(rho)
        assert np.max(np.abs(j - j_ref)) <= 1e-8 * np.max(np.abs(j_ref)), prec
        assert np.max(np.abs(ctx.occupation(rho) - occ_ref)) <= 1e-8, prec
