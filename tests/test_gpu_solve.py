"""Steady-state solves on the GPU against the oracle's TFQMR.

The FP64 solves run at the reference default crit 1e-8 ($converge, main/main.f90:856) on both
sides and follow the same iterates; the mixed solves run at crit 1e-10 against the oracle at
1e-9 (plain FP64 TFQMR stalls between 1e-9 and 1e-10 on the double dot: the augmented HEOM
system at T = 0.1 is ill-conditioned).  Currents agree to 1e-8 relative, occupations to 1e-8."""
import numpy as np
import pytest

import configs as cf
import heomq
import oracle_ffi as of

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cfg", [cf.siam(ntier=3), cf.CFG0, cf.dqd(ntier=3)], ids=["siam_L2", "siam_L3", "dqd_L2"])
def test_fp64_solve_matches_oracle(cfg):
    m = heomq.Model(cfg)
    ctx = heomq.Context(m)
    ref = of.Model(cfg)
    rho, info = ctx.solve_tfqmr(crit=1e-8)
    rho_ref, info_ref = ref.solve_tfqmr(crit=1e-8)
    assert info.converged and info.resid <= 1e-8
    j, j_ref = ctx.current(rho), ref.current(rho_ref)
    assert np.max(np.abs(j - j_ref)) <= 1e-8 * np.max(np.abs(j_ref))
    occ, occ_ref = ctx.occupation(rho), ref.occupation(rho_ref)
    assert np.max(np.abs(occ - occ_ref)) <= 1e-8


@pytest.mark.parametrize("cfg, prec", [(cf.CFG0, heomq.PREC_MIXED), (cf.dqd(ntier=3), heomq.PREC_MIXED),
                                       (cf.CFG0, heomq.PREC_MIXED_FP32)],
                         ids=["siam_L3-fp32x2", "dqd_L2-fp32x2", "siam_L3-fp32"])
def test_mixed_solve_matches_oracle(cfg, prec):
    """Inner TFQMR in FP32x2 (or plain FP32 where the conditioning allows) on the
    regularised operator, refined with FP64 residuals, reaches the FP64 criterion."""
    m = heomq.Model(cfg)
    ctx = heomq.Context(m)
    ref = of.Model(cfg)
    rho_ref, _ = ref.solve_tfqmr(crit=1e-9)
    rho, info = ctx.solve_tfqmr(crit=1e-10, precision=prec)
    assert info.converged and info.resid <= 1e-10
    j, j_ref = ctx.current(rho), ref.current(rho_ref)
    assert np.max(np.abs(j - j_ref)) <= 1e-8 * np.max(np.abs(j_ref))
    occ, occ_ref = ctx.occupation(rho), ref.occupation(rho_ref)
    assert np.max(np.abs(occ - occ_ref)) <= 1e-8


def test_mixed_batch_converges_on_the_kanamori_model():
    """Three-orbital Kanamori impurity (nd = 64, tier 2, T = 0.05), 4 bias points in one batch.

    Plain FP64 TFQMR stalls near 4e-8 on this batch.  The residual that a first refinement
    round leaves is dominated by slow modes, which a restarted TFQMR resolves only after
    several hundred iterations.  The mixed refinement must still reach crit, and its
    currents must agree with FP64 inner solves refined to 1e-12."""
    hb = 0.658211928
    m = heomq.Model(cf.HUND_L2)
    ctx = heomq.Context(m)
    Vs = [0.4 + 0.8 * b / 3 for b in range(4)]
    es = np.array([[V / 2, V / 2, -V / 2, -V / 2] for V in Vs]) / hb   # (ispin, ialf) column-major per instance
    es = np.ascontiguousarray(es.reshape(4, 2, 2).transpose(0, 2, 1).reshape(4, 4))
    rhos = np.tile(m.initial_guess(), (4, 1))
    out, info = ctx.solve_batch(rhos, eshift_batch=es, crit=1e-9, precision=heomq.PREC_MIXED)
    assert info.converged and info.resid <= 1e-9
    ref, info_ref = ctx.solve_batch(rhos, eshift_batch=es, crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
    assert info_ref.resid <= 1e-11
    j = np.array([ctx.current(out[b])[0].sum() for b in range(4)])
    j_ref = np.array([ctx.current(ref[b])[0].sum() for b in range(4)])
    assert np.max(np.abs(j - j_ref) / np.abs(j_ref)) <= 1e-7


@pytest.mark.parametrize("cfg", [cf.dqd(ntier=4), cf.siam(ntier=5)], ids=["dqd_L3", "siam_L4"])
def test_inner_preconditioner_keeps_the_answer_and_saves_iterations(cfg):
    """Left diagonal scaling of the FP32x2 inner solves (inner_precond 0 = default, -1 = off):
    the same steady state at the FP64 criterion, with fewer operator applies."""
    m = heomq.Model(cfg)
    ctx = heomq.Context(m)
    on, i_on = ctx.solve_tfqmr(crit=1e-9, precision=heomq.PREC_MIXED)
    off, i_off = ctx.solve_tfqmr(crit=1e-9, precision=heomq.PREC_MIXED, inner_precond=-1)
    assert i_on.converged and i_off.converged and i_on.resid <= 1e-9
    j_on, j_off = ctx.current(on)[0].sum(), ctx.current(off)[0].sum()
    assert abs(j_on / j_off - 1) < 1e-8
    assert i_on.iters < i_off.iters
