"""The instance-interleaved layout of the mixed solver's fused FP32x2 inner kernels.

With interleave G > 1 the batch's vectors hold G instances entry by entry; the lanes of one
entry share the plan's control flow and reads, and a group whose instances have partly
finished runs its remaining ones on fewer lanes.  The per-entry arithmetic is that of the
plain layout, so every interleave must give the same steady states to solver accuracy:
checked here for G = 1, 2, 4, 8 on a biased batch of the double dot, on a batch whose
instances finish at different iterations (lane compaction), and on a truncated batch."""
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


def _solve(m, batch, crit, interleave):
    x = torch.zeros((batch.nbatch, batch.stride), dtype=torch.complex128, device="cuda")
    x[:, : m.lunk] = torch.from_numpy(m.initial_guess()).cuda()
    torch.cuda.synchronize()
    info = batch.solve_dev(x.data_ptr(), crit=crit, precision=heomq.PREC_MIXED, interleave=interleave)
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
