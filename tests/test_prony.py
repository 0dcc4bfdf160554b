"""The Prony scheme (psfjob, main/zpout_psf.f90; main/evaluatepara.f90:1993-2000): fitted
exponentials in place of the Drude pole and the Pade terms, with the fitted table supplied by
the caller.  No GPU needed.

  * A table that restates the Pade decomposition of a Lorentzian band in the Prony form gives
    the coefficient tables of the Pade build to rounding and the same index tables.
  * The library's builder and the oracle agree on a table that is not a Pade restatement
    (integer tables bit for bit, coefficients exactly).
  * The oracle's steady state under such a table matches the dense hierarchy of the
    published equations (tests/dense_heom.py) fed with the same exponentials.
"""
import numpy as np
import pytest

import configs as cf
import dense_heom as dh
import heomq
import oracle_ffi as of
from test_independent_heom import mode_index, observables_dense, observables_oracle

INT_TABLES = ["nfirst", "nlast", "indextable", "index_coef_ref", "indexcoef", "itypecoef", "ifactfcoef",
              "ifactrcoef", "nnz_spa", "ind_spa", "irow_spa", "icol_spa"]


def other_table():
    return cf.prony_table()


@pytest.mark.parametrize("cfg", [cf.siam(ntier=3, nmats=2, T=0.1), cf.dqd(ntier=3, nmats=2, T=0.1)], ids=["siam", "dqd"])
def test_pade_restated_as_prony_gives_the_pade_tables(cfg):
    tab = heomq.psf_table_from_pade(cfg["nmats"], cfg["bandwidth"][0], cfg["temperature"][0], tpsf=0.7)
    a, b = heomq.Model(cfg), heomq.Model(dict(cfg, psf=tab))
    for k in ("cb", "cd", "cgamma"):
        x, y = a.array(k), b.array(k)
        assert np.abs(x - y).max() <= 1e-13 * np.abs(x).max(), k
    for k in INT_TABLES:
        np.testing.assert_array_equal(a.array(k), b.array(k), err_msg=k)


@pytest.mark.parametrize("cfg", [cf.siam(ntier=4, nmats=1, T=0.3), cf.dqd(ntier=3, nmats=1, T=0.3)], ids=["siam", "dqd"])
def test_builder_and_oracle_agree_on_a_prony_table(cfg):
    c = dict(cfg, psf=other_table())
    p, o = heomq.Model(c), of.Model(c)
    assert (p.lunk, p.nunk, p.lall) == (o.lunk, o.nunk, o.lall)
    for k in INT_TABLES:
        np.testing.assert_array_equal(p.array(k).astype(np.int64), o.get(k)[: p.array(k).size].astype(np.int64), err_msg=k)
    for k in ("cb", "cd", "cgamma"):
        np.testing.assert_array_equal(p.array(k), o.get(k)[: p.array(k).size], err_msg=k)


@pytest.mark.parametrize("norbs", [1, 2], ids=["siam", "dqd"])
def test_oracle_prony_steady_state_matches_dense_hierarchy(norbs):
    tab = other_table()
    T, V, U, eps, t, g = 0.3, 0.6, 2.0, -0.8, 0.5, 0.5
    cfg = (cf.siam(ntier=3, nmats=1, V=V, U=U, eps=eps, T=T) if norbs == 1
           else cf.dqd(ntier=3, nmats=1, V=V, U=U, eps=eps, t=t, T=T))
    m = of.Model(dict(cfg, psf=tab))
    rho, _ = m.solve_tfqmr(crit=1e-12, maxit0=40000)
    o_occ, o_cur, o_dbl, o_coh, o_spec = observables_oracle(m, rho, norbs)
    # the same exponentials in the dense hierarchy: eta = T / tpsf coef (per unit linewidth),
    # gamma = -T / tpsf pole (the reference's cgama is minus the decay rate)
    s = T / tab["tpsf"]
    terms = [(s * c, -s * p) for c, p in zip(tab["coef"], tab["pole"])]
    nm = 2 * norbs
    a = dh.annihilators(nm)
    n = [x.T @ x for x in a]
    idx = mode_index(norbs)
    H = np.zeros((1 << nm, 1 << nm))
    for o in range(norbs):
        H += eps * (n[idx[(o, 0)]] + n[idx[(o, 1)]]) + U * n[idx[(o, 0)]] @ n[idx[(o, 1)]]
    if norbs == 2:
        for sp in range(2):
            H += t * (a[idx[(0, sp)]].T @ a[idx[(1, sp)]] + a[idx[(1, sp)]].T @ a[idx[(0, sp)]])
    leads = [[0], [0]] if norbs == 1 else [[0], [1]]
    coup = {(al, idx[(o, sp)]): g for al, orbs in enumerate(leads) for o in orbs for sp in range(2)}
    h = dh.Hierarchy(H / dh.HBAR, a, dh.exponential_bath(coup, [V / 2, -V / 2], terms), 2)
    d_occ, d_cur, d_dbl, d_coh, d_spec = observables_dense(h, h.steady(), a, idx, norbs)
    np.testing.assert_allclose(o_occ, d_occ, atol=1e-9)
    np.testing.assert_allclose(o_cur, d_cur, atol=1e-8 * np.abs(d_cur).max())
    np.testing.assert_allclose(o_spec, d_spec, atol=1e-9)
    assert np.abs(d_cur).max() > 1e2


def test_prony_table_is_validated():
    bad = dict(heomq.psf_table_from_pade(1, 10.0, 0.1), tpsf=0.0)
    with pytest.raises(heomq.HeomError):
        heomq.Model(dict(cf.siam(ntier=3, nmats=1), psf=bad))
