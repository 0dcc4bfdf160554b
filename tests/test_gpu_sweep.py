"""Batched I-V sweep of single-orbital instances with uneven hierarchies (tiers 2-4).

The instances of one table family form one batch on the deepest member's tables, each
truncated at its own tier (heom_batch_set_tiers).  Checked here:
- a truncated batch against separate solves of the same models at each tier (the truncation
  itself: states entry by entry, zero beyond each instance's tier);
- the 128-instance sweep, one family in one launch sequence, in mixed precision against the
  same sweep refined in FP64 to ||b - A x|| <= 1e-12, and a few instances against their own
  separate FP64 solves."""
import numpy as np
import pytest
import torch

import heomq
from heomq import models, sweep

pytestmark = pytest.mark.gpu


def _family(tiers, Vs, Us):
    cfgs = [models.siam(ntier=nt, nmats=4, V=V, U=U, eps=-U / 2) for nt, V, U in zip(tiers, Vs, Us)]
    deep = heomq.Model(cfgs[int(np.argmax(tiers))])
    nd2 = deep.nrho ** 2
    hs = np.stack([heomq.Model(dict(c, ntier=2)).get("hs", nd2, np.complex128) for c in cfgs])
    es = np.stack([sweep._lead_shift(c, deep.nalf, deep.nspin) for c in cfgs])
    return cfgs, deep, hs, es


# The states agree to about 100 crit (the residual bound times the conditioning of these
# hierarchies: 1.3e-8 was seen at crit 1e-10), so the mixed solve runs at crit 1e-11.
@pytest.mark.parametrize("prec,crit,bar", [(heomq.PREC_FP64_REFINED, 1e-12, 1e-9), (heomq.PREC_MIXED, 1e-11, 1e-8)],
                         ids=["fp64_refined", "mixed"])
def test_truncated_batch_equals_separate_solves_at_each_tier(prec, crit, bar):
    tiers = [2, 3, 4, 5, 3]
    cfgs, deep, hs, es = _family(tiers, [0.6, -0.4, 0.9, 0.3, 0.8], [2.0, 1.0, 3.0, 2.0, 3.0])
    ctx = heomq.Context(deep, adjoint=False)
    batch = heomq.Batch(ctx, hs_batch=hs, eshift_batch=es, nbatch=len(cfgs), ntier=tiers)
    x = torch.zeros((len(cfgs), batch.stride), dtype=torch.complex128, device="cuda")
    # a nonzero start beyond each instance's tier: the solve must clear it
    x[:, : deep.lunk] = torch.from_numpy(deep.initial_guess()).cuda() + 0.25
    torch.cuda.synchronize()
    info = batch.solve_dev(x.data_ptr(), crit=crit, precision=prec, max_refine=16)
    assert info.converged and info.resid <= crit
    xb = x.cpu().numpy()
    jb = batch.currents_static(x.data_ptr())
    for b, cfg in enumerate(cfgs):
        m = heomq.Model(cfg)
        c = heomq.Context(m, adjoint=False)
        rho, inf = c.solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
        assert inf.converged
        # the prefix of the deep layout is the shallower hierarchy's own layout
        err = np.linalg.norm(xb[b, : m.lunk] - rho) / np.linalg.norm(rho)
        assert err <= bar, (b, tiers[b], err)
        assert not np.any(xb[b, m.lunk : deep.lunk]), b
        j = c.current(rho)
        assert np.max(np.abs(jb[b] - j)) <= bar * np.max(np.abs(j)), b
        c.close()
    batch.close()
    ctx.close()


def test_truncated_fp64_solve_follows_the_separate_solves():
    """The reference FP64 TFQMR on a truncated batch: each instance pairs its trace slot with
    the shadow-vector component of its own hierarchy, so its iterates are those of the solve
    on its own tables, and both stop at the same check with the same state (to rounding)."""
    tiers = [2, 4, 3]
    cfgs, deep, hs, es = _family(tiers, [0.7, -0.5, 0.2], [2.0, 3.0, 1.0])
    ctx = heomq.Context(deep, adjoint=False)
    batch = heomq.Batch(ctx, hs_batch=hs, eshift_batch=es, nbatch=len(cfgs), ntier=tiers)
    x = torch.zeros((len(cfgs), batch.stride), dtype=torch.complex128, device="cuda")
    for b, cfg in enumerate(cfgs):
        x[b, : heomq.Model(cfg).lunk] = torch.from_numpy(heomq.Model(cfg).initial_guess()).cuda()
    torch.cuda.synchronize()
    info = batch.solve_dev(x.data_ptr(), crit=1e-8, precision=heomq.PREC_FP64)
    assert info.converged
    xb = x.cpu().numpy()
    iters = []
    for b, cfg in enumerate(cfgs):
        m = heomq.Model(cfg)
        c = heomq.Context(m, adjoint=False)
        rho, inf = c.solve_tfqmr(crit=1e-8, precision=heomq.PREC_FP64)
        iters.append(inf.iters)
        err = np.linalg.norm(xb[b, : m.lunk] - rho) / np.linalg.norm(rho)
        assert err <= 1e-10, (b, tiers[b], err)
        c.close()
    assert info.iters == max(iters)
    batch.close()
    ctx.close()


def test_set_tiers_rejects_tiers_beyond_the_context():
    tiers = [2, 3]
    cfgs, deep, hs, es = _family(tiers, [0.5, 0.5], [2.0, 2.0])
    ctx = heomq.Context(deep, adjoint=False)
    for bad in ([0, 3], [2, 4]):
        with pytest.raises(heomq.HeomError):
            heomq.Batch(ctx, hs_batch=hs, eshift_batch=es, nbatch=2, ntier=bad)
    ctx.close()


def test_sweep_of_128_instances_in_one_family():
    cfgs = models.iv_sweep(n=128, seed=20261203)
    assert len(sweep.group_instances(cfgs)) == 1
    assert {c["ntier"] for c in cfgs} == {3, 4, 5}
    ref, iref = sweep.solve_sweep(cfgs, crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
    assert all(i.converged for i in iref)
    cur, infos = sweep.solve_sweep(cfgs, crit=1e-10)
    assert all(i.converged for i in infos)
    rel = np.abs(cur - ref) / np.abs(ref)
    assert np.max(rel) <= 1e-8, (int(np.argmax(rel)), float(np.max(rel)))
    # one instance of each depth against its own separate solve
    for nt in (3, 4, 5):
        k = next(i for i, c in enumerate(cfgs) if c["ntier"] == nt)
        m = heomq.Model(cfgs[k])
        c = heomq.Context(m, adjoint=False)
        rho, inf = c.solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
        j = c.current(rho)[0].sum()
        assert abs(ref[k] - j) <= 1e-9 * abs(j), (k, nt, ref[k], j)
        c.close()
