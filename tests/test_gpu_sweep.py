"""Batched I-V sweep of single-orbital instances with uneven hierarchies (tiers 2-4): each
instance's current from the grouped batch solve against its own FP64 solve."""
import numpy as np
import pytest

import heomq
from heomq import models, sweep

pytestmark = pytest.mark.gpu


def test_uneven_sweep_matches_individual_solves():
    cfgs = models.iv_sweep(n=12, seed=20261203)
    groups = sweep.group_instances(cfgs)
    assert len(groups) >= 2
    cur, infos = sweep.solve_sweep(cfgs, crit=1e-10)
    assert all(i.converged for i in infos)
    for k, cfg in enumerate(cfgs):
        m = heomq.Model(cfg)
        ctx = heomq.Context(m, adjoint=False)
        rho, info = ctx.solve_tfqmr(crit=1e-9, precision=heomq.PREC_FP64)
        ref = ctx.current(rho)[0].sum()
        assert abs(cur[k] - ref) <= 1e-6 * max(abs(ref), 1.0), (k, cur[k], ref)
