"""The instance-interleaved layout of the mixed solver's fused FP32x2 inner kernels.

With interleave G > 1 the batch's vectors hold G instances entry by entry; the lanes of one
entry share the plan's control flow and reads, and a group whose instances have partly
finished runs its remaining ones on fewer lanes.  The per-entry arithmetic is that of the
plain layout, so every interleave must give the same steady states to solver accuracy:
checked here for G = 1, 2, 4, 8 on a biased batch of the double dot, on a batch whose
instances finish at different iterations (lane compaction), and on a truncated batch.
With two instances per lane (lane_instances 2) a thread decodes the plan once for two
adjacent instances of its group; in groups of two its blocks cover the same entries of each
instance as the plain layout and sum them in the same order, so its iterates are the plain
layout's, bit for bit."""
import numpy as np
import pytest
import torch

import heomq
from heomq import models
from test_gpu_sweep import _family

pytestmark = pytest.mark.gpu

HB = 0.658211928


def _bias_batch(m, Vs):
    es = np.array([[V / 2, V / 2, -V / 2, -V / 2] for V in Vs]) / HB
    es = np.ascontiguousarray(es.reshape(len(Vs), 2, 2).transpose(0, 2, 1).reshape(len(Vs), 4))
    ctx = heomq.Context(m, adjoint=False)
    return ctx, heomq.Batch(ctx, eshift_batch=es, nbatch=len(Vs))


def _solve(m, batch, crit, interleave, lanes=0):
    x = torch.zeros((batch.nbatch, batch.stride), dtype=torch.complex128, device="cuda")
    x[:, : m.lunk] = torch.from_numpy(m.initial_guess()).cuda()
    torch.cuda.synchronize()
    info = batch.solve_dev(x.data_ptr(), crit=crit, precision=heomq.PREC_MIXED, interleave=interleave,
                           lane_instances=lanes)
    return x, info


@pytest.mark.parametrize("Vs", [[0.4 + 0.8 * b / 7 for b in range(8)], [-1.5, -0.2, 0.05, 0.3, 0.8, 1.2, 2.0]],
                         ids=["even_bias", "uneven_bias"])
def test_every_interleave_gives_the_same_currents(Vs):
    """The double dot at tier 2, batches of 8 and 7 bias points (the second with instances far
    apart, which finish at different iterations), mixed solves to crit 1e-10 with interleave
    1, 2, 4 and 8: lead currents agree within 1e-8 relative."""
    m = heomq.Model(models.dqd(ntier=3, nmats=3))
    ctx, batch = _bias_batch(m, Vs)
    cur = {}
    for g in (1, 2, 4, 8):
        x, info = _solve(m, batch, 1e-10, g)
        assert info.converged and info.resid <= 1e-10, g
        cur[g] = np.array([ctx.current(x[b, : m.lunk].cpu().numpy()) for b in range(len(Vs))])
    scale = np.abs(cur[1]).max()
    for g in (2, 4, 8):
        assert np.abs(cur[g] - cur[1]).max() <= 1e-8 * scale, g
    batch.close()
    ctx.close()


def test_interleaved_truncated_batch_matches_separate_solves():
    """A truncated batch (instances at tiers 2-5 of one family) with all eight instances in one
    interleaved group, against separate FP64-refined solves at each tier."""
    tiers = [2, 5, 3, 4, 2, 3, 5, 4]
    cfgs, deep, hs, es = _family(tiers, [0.6, -0.4, 0.9, 0.3, -0.8, 0.2, 0.7, -0.1], [2.0, 1.0, 3.0, 2.0, 1.0, 3.0, 2.0, 1.0])
    ctx = heomq.Context(deep, adjoint=False)
    batch = heomq.Batch(ctx, hs_batch=hs, eshift_batch=es, nbatch=len(cfgs), ntier=tiers)
    x = torch.zeros((len(cfgs), batch.stride), dtype=torch.complex128, device="cuda")
    x[:, : deep.lunk] = torch.from_numpy(deep.initial_guess()).cuda()
    torch.cuda.synchronize()
    info = batch.solve_dev(x.data_ptr(), crit=1e-10, precision=heomq.PREC_MIXED, interleave=8)
    assert info.converged
    jb = batch.currents_static(x.data_ptr())
    xb = x.cpu().numpy()
    for b, cfg in enumerate(cfgs):
        mb = heomq.Model(cfg)
        c = heomq.Context(mb, adjoint=False)
        rho, inf = c.solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
        assert inf.converged
        assert np.linalg.norm(xb[b, : mb.lunk] - rho) <= 1e-8 * np.linalg.norm(rho), b
        assert not np.any(xb[b, mb.lunk : deep.lunk]), b
        j = c.current(rho)
        assert np.max(np.abs(jb[b] - j)) <= 1e-8 * np.max(np.abs(j)), b
        c.close()
    batch.close()
    ctx.close()


def test_interleave_must_be_a_power_of_two():
    m = heomq.Model(models.siam(ntier=3, nmats=2))
    ctx, batch = _bias_batch(m, [0.2, 0.4, 0.6])
    x = torch.zeros((3, batch.stride), dtype=torch.complex128, device="cuda")
    x[:, : m.lunk] = torch.from_numpy(m.initial_guess()).cuda()
    torch.cuda.synchronize()
    for bad in (3, 64, -2):
        with pytest.raises(heomq.HeomError):
            batch.solve_dev(x.data_ptr(), crit=1e-9, precision=heomq.PREC_MIXED, interleave=bad)
    batch.close()
    ctx.close()


@pytest.mark.parametrize("Vs", [[0.4 + 0.8 * b / 7 for b in range(8)], [-1.5, -0.2, 0.05, 0.3, 0.8, 1.2, 2.0]],
                         ids=["even_bias", "uneven_bias"])
def test_pairs_give_the_iterates_of_one_instance_per_group(Vs):
    """Interleave 2 with two instances per lane against interleave 1 on the double dot at tier
    4 (Pade M = 3): the same applies and the same steady states, bit for bit, also with an odd
    batch (the last pair half empty) and with instances that finish apart (a pair with one
    running instance goes on with one instance per lane)."""
    m = heomq.Model(models.dqd(ntier=5, nmats=3))
    ctx, batch = _bias_batch(m, Vs)
    x1, i1 = _solve(m, batch, 1e-10, 1)
    x2, i2 = _solve(m, batch, 1e-10, 2, lanes=2)
    assert i1.converged and i2.converged
    assert (i1.iters, i1.refinements) == (i2.iters, i2.refinements)
    assert torch.equal(x1, x2)
    batch.close()
    ctx.close()


def test_two_instances_per_lane_in_wide_groups():
    """Interleave 8 with two instances per lane (four lanes per entry): the currents of interleave
    1 within 1e-8 relative, on a batch of 8 and of 5 bias points."""
    m = heomq.Model(models.dqd(ntier=3, nmats=3))
    for Vs in ([0.4 + 0.8 * b / 7 for b in range(8)], [-0.9, 0.1, 0.5, 1.1, 1.7]):
        ctx, batch = _bias_batch(m, Vs)
        cur = {}
        for g, lanes in ((1, 1), (8, 2)):
            x, info = _solve(m, batch, 1e-10, g, lanes)
            assert info.converged and info.resid <= 1e-10, (g, lanes)
            cur[g] = np.array([ctx.current(x[b, : m.lunk].cpu().numpy()) for b in range(len(Vs))])
        assert np.abs(cur[8] - cur[1]).max() <= 1e-8 * np.abs(cur[1]).max()
        batch.close()
        ctx.close()


def test_two_instances_per_lane_in_groups_of_32():
    """Interleave 32 with two instances per lane (16 lanes per entry) on 20 bias points of the
    single-orbital model, instances finishing apart: currents of interleave 1 within 1e-8."""
    m = heomq.Model(models.siam(ntier=4, nmats=3))
    Vs = [-1.5 + 0.16 * b for b in range(20)]
    ctx, batch = _bias_batch(m, Vs)
    cur = {}
    for g, lanes in ((1, 1), (32, 2)):
        x, info = _solve(m, batch, 1e-10, g, lanes)
        assert info.converged and info.resid <= 1e-10, (g, lanes)
        cur[g] = np.array([ctx.current(x[b, : m.lunk].cpu().numpy()) for b in range(len(Vs))])
    assert np.abs(cur[32] - cur[1]).max() <= 1e-8 * np.abs(cur[1]).max()
    batch.close()
    ctx.close()


def test_automatic_layout_times_every_candidate_then_keeps_one():
    m = heomq.Model(models.siam(ntier=4, nmats=3))
    ctx, batch = _bias_batch(m, [0.1 * b for b in range(1, 7)])
    cand = heomq.layout_candidates(6)
    assert cand == [(1, 1), (2, 2), (8, 1), (8, 2)]
    for k in range(len(cand)):
        assert ctx.tuned_layout(6) == (0, 0), k
        x, info = _solve(m, batch, 1e-9, 0)
        assert info.converged
    assert ctx.tuned_layout(6) in cand
    batch.close()
    ctx.close()


def test_lane_instances_is_checked():
    m = heomq.Model(models.siam(ntier=3, nmats=2))
    ctx, batch = _bias_batch(m, [0.2, 0.4, 0.6])
    for g, lanes in ((1, 2), (2, 3), (4, -1)):
        with pytest.raises(heomq.HeomError):
            _solve(m, batch, 1e-9, g, lanes)
    batch.close()
    # truncated batches keep one instance per lane
    cfgs, deep, hs, es = _family([2, 3], [0.6, -0.4], [2.0, 1.0])
    c2 = heomq.Context(deep, adjoint=False)
    tb = heomq.Batch(c2, hs_batch=hs, eshift_batch=es, nbatch=2, ntier=[2, 3])
    x = torch.zeros((2, tb.stride), dtype=torch.complex128, device="cuda")
    x[:, : deep.lunk] = torch.from_numpy(deep.initial_guess()).cuda()
    torch.cuda.synchronize()
    with pytest.raises(heomq.HeomError):
        tb.solve_dev(x.data_ptr(), crit=1e-9, precision=heomq.PREC_MIXED, interleave=2, lane_instances=2)
    assert heomq.layout_candidates(2, truncated=True) == [(1, 1), (2, 1)]
    tb.close()
    c2.close()
    ctx.close()
