"""Batched I-V sweeps over instances with uneven hierarchies.

Instances of one table family (Pade order, orbitals, leads and H sparsity) differ in their H
values, lead shifts and truncation tier.  The reference's tables are tier-major, so the tables
of a shallower hierarchy are a prefix of the deepest one's: a family is one heom_batch built at
its deepest tier, each instance truncated at its own tier (heom_batch_set_tiers), and all its
instances are solved in one launch sequence.  Families are solved one after the other; the
host work of a family (its tables and the per-instance H) runs in worker threads, so that the
next family's tables are built while one solves.
"""

from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import PREC_MIXED, Batch, Context, Model

HBAR = 0.658211928


def _table_key(cfg):
    skip = {"engyshift", "eup", "edown", "uu", "e1up", "e1down", "e2up", "e2down", "uu1", "uu2", "u12", "t12",
            "kan_u", "kan_j", "kan_eps", "ntier"}
    return tuple(sorted((k, repr(v)) for k, v in cfg.items() if k not in skip))


def group_instances(cfgs):
    """Indices of the instances of each table family (equal but for levels, bias and tier)."""
    groups = {}
    for i, cfg in enumerate(cfgs):
        groups.setdefault(_table_key(cfg), []).append(i)
    return list(groups.values())


def _lead_shift(cfg, nalf, nspin):
    es = np.zeros(nalf * nspin)
    for a in range(nalf):
        for s in range(nspin):
            es[a + s * nalf] = cfg["engyshift"][a][s] / HBAR
    return es


def solve_sweep(cfgs, crit=1e-9, precision=PREC_MIXED, device=0, max_refine=8, check=True, interleave=1):
    """Steady states of many instances; returns (lead-1 currents, per-family solve infos).

    The states stay on the device; only the currents (through the allocation-free batch
    current reduction) come back to the host.  check=False returns the infos of families that
    did not reach crit (their `converged` is 0) instead of raising.  interleave: instances
    per entry group of the mixed solver's inner kernels (heom_solve_opts.interleave; every
    family is solved once, on a context of its own, so the automatic choice 0 would always
    take its first candidate)."""
    import torch

    # within a family, instances in order of their tier: the fused kernels run instances in
    # interleaved groups, and a group of one depth skips the blocks beyond its tier together
    groups = [sorted(g, key=lambda i: cfgs[i]["ntier"]) for g in group_instances(cfgs)]
    currents = np.zeros(len(cfgs))
    infos = [None] * len(groups)

    def prepare(idx):
        # host only (the table builder and the tier-1 models release the GIL in their C calls):
        # runs in worker threads while earlier families solve; the family's tables at its
        # deepest tier
        deepest = max(idx, key=lambda i: cfgs[i]["ntier"])
        rep = Model(cfgs[deepest])
        nd2 = rep.nrho ** 2
        # H depends on the level parameters only: a tier-1 model of each instance gives it cheaply
        hs = np.stack([Model(dict(cfgs[i], ntier=2)).get("hs", nd2, np.complex128) for i in idx])
        es = np.stack([_lead_shift(cfgs[i], rep.nalf, rep.nspin) for i in idx])
        return rep, hs, es

    def run(gi, rep, hs, es):
        idx = groups[gi]
        ctx = Context(rep, device=device, adjoint=False)
        tiers = [cfgs[i]["ntier"] for i in idx]
        batch = Batch(ctx, hs_batch=hs, eshift_batch=es, nbatch=len(idx),
                      ntier=None if len(set(tiers)) == 1 else tiers)
        with torch.cuda.device(device):
            x = torch.zeros((len(idx), batch.stride), dtype=torch.complex128, device=f"cuda:{device}")
            x[:, : rep.lunk] = torch.from_numpy(rep.initial_guess()).to(x.device)
            torch.cuda.synchronize(device)
            infos[gi] = batch.solve_dev(x.data_ptr(), crit=crit, precision=precision, max_refine=max_refine,
                                        check=check, interleave=interleave)
            jt = batch.currents_static(x.data_ptr())
        for k, i in enumerate(idx):
            currents[i] = jt[k, 0].sum()
        batch.close()
        ctx.close()

    # families with the smaller tables first, so that the larger tables are built meanwhile
    order = sorted(range(len(groups)), key=lambda g: (max(cfgs[i]["ntier"] for i in groups[g]), len(groups[g])))
    with ThreadPoolExecutor(max_workers=max(1, min(4, len(groups)))) as ex:
        futures = {g: ex.submit(prepare, groups[g]) for g in order}
        for g in order:
            run(g, *futures[g].result())
    return currents, infos
