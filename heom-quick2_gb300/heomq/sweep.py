"""Batched I-V sweeps over instances with uneven hierarchies.

Instances that share one table set (same tier depth, Pade order, orbitals, leads and H
sparsity) differ only in their H values and lead shifts; each such group is one
heom_batch, solved in one launch sequence.  Groups are solved one after the other: each
batch already fills the GPU, and running two contexts' solves from two host threads
overlaps little (about 6 % measured) while their graph captures would have to be kept
apart from each other's synchronisations.  The host work of a group (its tables and the
per-instance H) runs in worker threads, so that the larger tables are built while the
smaller groups solve.
"""

from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import PREC_MIXED, Batch, Context, Model

HBAR = 0.658211928


def _table_key(cfg):
    skip = {"engyshift", "eup", "edown", "uu", "e1up", "e1down", "e2up", "e2down", "uu1", "uu2", "u12", "t12",
            "kan_u", "kan_j", "kan_eps"}
    return tuple(sorted((k, repr(v)) for k, v in cfg.items() if k not in skip))


def group_instances(cfgs):
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


def solve_sweep(cfgs, crit=1e-9, precision=PREC_MIXED, device=0, max_refine=8):
    """Steady states of many instances; returns (lead-1 currents, per-group solve infos).

    The states stay on the device; only the currents (through the allocation-free batch
    current reduction) come back to the host."""
    import torch

    groups = group_instances(cfgs)
    currents = np.zeros(len(cfgs))
    infos = [None] * len(groups)

    def prepare(idx):
        # host only (the table builder and the tier-1 models release the GIL in their C calls):
        # runs in worker threads while earlier groups solve on the device
        rep = Model(cfgs[idx[0]])
        nd2 = rep.nrho ** 2
        # H depends on the level parameters only: a tier-1 model of each instance gives it cheaply
        hs = np.stack([Model(dict(cfgs[i], ntier=2)).get("hs", nd2, np.complex128) for i in idx])
        es = np.stack([_lead_shift(cfgs[i], rep.nalf, rep.nspin) for i in idx])
        return rep, hs, es

    def run(gi, rep, hs, es):
        idx = groups[gi]
        ctx = Context(rep, device=device, adjoint=False)
        batch = Batch(ctx, hs_batch=hs, eshift_batch=es, nbatch=len(idx))
        with torch.cuda.device(device):
            x = torch.zeros((len(idx), batch.stride), dtype=torch.complex128, device=f"cuda:{device}")
            x[:, : rep.lunk] = torch.from_numpy(rep.initial_guess()).to(x.device)
            torch.cuda.synchronize(device)
            infos[gi] = batch.solve_dev(x.data_ptr(), crit=crit, precision=precision, max_refine=max_refine)
            jt = batch.currents_static(x.data_ptr())
        for k, i in enumerate(idx):
            currents[i] = jt[k, 0].sum()
        batch.close()
        ctx.close()

    # groups with the smaller tables first, so that the larger tables are built meanwhile
    order = sorted(range(len(groups)), key=lambda g: (cfgs[groups[g][0]]["ntier"], len(groups[g])))
    with ThreadPoolExecutor(max_workers=max(1, min(4, len(groups)))) as ex:
        futures = {g: ex.submit(prepare, groups[g]) for g in order}
        for g in order:
            run(g, *futures[g].result())
    return currents, infos
