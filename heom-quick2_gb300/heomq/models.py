"""Synthetic impurity models of the benchmark, written as the quantities of the
reference input file (positional lines of main/evaluatepara.f90:71-84 plus the
$para1 / $para4 / $ddots / $jobinfo namelists).  Energies in meV (funits = 1)."""
import numpy as np


def siam(ntier=4, nmats=4, V=0.4, U=2.0, eps=-1.0, gamma=0.5, W=10.0, T=0.1, tchar=0.0):
    """Single-orbital Anderson impurity, nd = 4 ($para1 eup = edown = eps, uu = U)."""
    return dict(norbs=1, nspin=2, nalf=2, nmats=nmats, ntier=ntier, bandwidth=[W, W],
                linewidth=[[gamma], [gamma]], temperature=[T, T],
                engyshift=[[V / 2, V / 2], [-V / 2, -V / 2]], model=1, eup=eps, edown=eps, uu=U, tchar=tchar)


def dqd(ntier=5, nmats=3, V=0.8, U=2.0, eps=-1.0, t=0.5, gamma=0.5, W=10.0, T=0.1, tchar=0.0):
    """Serial double quantum dot, nd = 16 ($para4, $ddots doubledot=T, $jobinfo lscreen=T)."""
    return dict(norbs=2, nspin=2, nalf=2, nmats=nmats, ntier=ntier, bandwidth=[W, W],
                linewidth=[[gamma, gamma], [gamma, gamma]], temperature=[T, T],
                engyshift=[[V / 2, V / 2], [-V / 2, -V / 2]], model=4,
                e1up=eps, e1down=eps, e2up=eps, e2down=eps, uu1=U, uu2=U, u12=0.0, t12=t,
                doubledot=1, lscreen=1, tchar=tchar)


def hund(ntier=3, nmats=6, V=0.2, U=3.0, J=0.3, gamma=0.25, W=10.0, T=0.05):
    """Three-orbital Kanamori impurity, nd = 64 (lreadhs data generated from U, U' = U - 2J, J)."""
    return dict(norbs=3, nspin=2, nalf=2, nmats=nmats, ntier=ntier, bandwidth=[W, W],
                linewidth=[[gamma] * 3, [gamma] * 3], temperature=[T, T],
                engyshift=[[V / 2, V / 2], [-V / 2, -V / 2]], model=5,
                kan_u=U, kan_j=J, kan_eps=-(5 * U - 10 * J) / 2)


SIAM_L3 = siam(ntier=4, nmats=4, V=0.4)      # single-orbital Anderson impurity, truncation tier 3
DQD_L4 = dqd(ntier=5, nmats=3, V=0.8)        # serial double dot, truncation tier 4
HUND_L2 = hund(ntier=3, nmats=6, V=0.2)      # three-orbital Hund impurity, truncation tier 2


def iv_sweep(n=128, seed=20261203):
    """Batched I-V sweep: n SIAM instances, V ~ U[-1, 1], U in {1, 2, 3}, eps = -U/2, L in {2, 3, 4}."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        V = float(rng.uniform(-1.0, 1.0))
        U = float(rng.choice([1.0, 2.0, 3.0]))
        L = int(rng.choice([2, 3, 4]))
        out.append(siam(ntier=L + 1, nmats=4, V=V, U=U, eps=-U / 2))
    return out
