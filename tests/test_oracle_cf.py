"""Known answers that pin the oracle's correlation-function system (no GPU needed).

corrfunc/corrfunc.f90:146-192 turns two solves of the frequency-domain system
(corrfunc/solve_cf_tfqmr_spa.f90) into the spectral function of a_{iorbs,ispin}:
A(w) = Re Tr[a^dag X(isgnb=2, isgnw=2)] / pi / hbar + Re Tr[a X(isgnb=1, isgnw=1)] / pi / hbar.
For U = 0 the hierarchy closes at tier 2 and A(w) = -Im G^r(w) / pi with
G^r = [w - h - Sigma(w)]^-1, Sigma_alpha = Gamma_alpha W / (2 (w - mu_alpha + i W)) on the
orbitals the lead couples to; the first part is A(w) f_eff(w), the occupied spectrum, with
f_eff the Gamma-weighted lead Fermi functions.
"""
import numpy as np
import pytest

import configs as cf
import oracle_ffi as of

T, V, W, GAMMA = 0.2, 0.4, 5.0, 0.5
MUS = (V / 2, -V / 2)


def _sigma(w, mu):
    return GAMMA * W / (2 * (w - mu + 1j * W))


def _fermi(w, mu):
    return 0.5 * (1 - np.tanh((w - mu) / (2 * T)))


def _steady(cfg):
    m = of.Model(cfg)
    rho, _ = m.solve_tfqmr(crit=1e-12, maxit0=40000)
    return m, rho


@pytest.fixture(scope="module")
def level():
    return _steady(cf.siam(ntier=3, nmats=10, V=V, U=0.0, eps=0.3, T=T, W=W))


@pytest.mark.parametrize("ispin", [1, 2])
@pytest.mark.parametrize("w", [-1.0, 0.3, 0.8])
def test_resonant_level_spectral_function(level, ispin, w):
    m, rho = level
    c = of.CF(m, 1, ispin)
    A, d1, d2 = c.dos(rho, w)
    g = 1.0 / (w - 0.3 - sum(_sigma(w, mu) for mu in MUS))
    assert abs(A / (-g.imag / np.pi) - 1) < 1e-10
    gam = [GAMMA * W * W / ((w - mu) ** 2 + W * W) for mu in MUS]
    feff = sum(G * _fermi(w, mu) for G, mu in zip(gam, MUS)) / sum(gam)
    assert abs(d1 / (A * feff) - 1) < 1e-8
    assert abs(d2 / (A * (1 - feff)) - 1) < 1e-8


@pytest.mark.parametrize("iorbs", [1, 2])
def test_double_dot_spectral_function(iorbs):
    """Serial double dot at U = 0: dot 1 on the left lead, dot 2 on the right, hopping t."""
    m, rho = _steady(cf.dqd(ntier=3, nmats=1, V=V, U=0.0, eps=0.3, t=0.5, T=T, W=W))
    c = of.CF(m, iorbs, 1)
    w = 0.3
    A, _, _ = c.dos(rho, w)
    g = np.linalg.inv(np.array([[w - 0.3 - _sigma(w, MUS[0]), -0.5], [-0.5, w - 0.3 - _sigma(w, MUS[1])]]))
    assert abs(A / (-g[iorbs - 1, iorbs - 1].imag / np.pi) - 1) < 1e-10


def test_cf_pattern_tables(level):
    m, _ = level
    c = of.CF(m, 1, 1)
    nnz, ind = c.get("nnzcf_spa"), c.get("indcf_spa")
    assert ind[0] == 1 and np.all(ind[1:] == ind[:-1] + nnz[:-1])
    assert ind[-1] + nnz[-1] - 1 == c.lunkcf
    ir, ic = c.get("irowcf_spa"), c.get("icolcf_spa")
    assert ir.min() >= 1 and ir.max() <= m.nrho and ic.min() >= 1 and ic.max() <= m.nrho
    # entries of one block are distinct and in column-major order
    for n in range(m.nunk):
        s = slice(ind[n] - 1, ind[n] - 1 + nnz[n])
        key = (ic[s] - 1) * m.nrho + (ir[s] - 1)
        assert np.all(np.diff(key) > 0)


def test_cf_apply_is_real_linear(level):
    m, _ = level
    c = of.CF(m, 1, 1)
    rng = np.random.default_rng(5)
    n = c.lunkcf
    x1 = [rng.standard_normal(n) + 1j * rng.standard_normal(n) for _ in range(2)]
    x2 = [rng.standard_normal(n) + 1j * rng.standard_normal(n) for _ in range(2)]
    y1, y2 = c.apply(0.7, 1, *x1), c.apply(0.7, 1, *x2)
    y3 = c.apply(0.7, 1, *(2.5 * a - 1.5 * b for a, b in zip(x1, x2)))
    for k in range(2):
        assert np.allclose(y3[k], 2.5 * y1[k] - 1.5 * y2[k], rtol=1e-12, atol=1e-12)
    # the omega terms only couple h and a: the difference between two frequencies is
    # (dfacta (w1 - w0) xa, dfactb (w1 - w0) xh), dfacta = -1, dfactb = +1 for isgnw = 1
    y0 = c.apply(0.0, 1, *x1)
    assert np.allclose(y1[0] - y0[0], -0.7 * x1[1], atol=1e-12)
    assert np.allclose(y1[1] - y0[1], 0.7 * x1[0], atol=1e-12)
    z0, z1 = c.apply(0.0, 2, *x1), c.apply(0.7, 2, *x1)
    assert np.allclose(z1[0] - z0[0], 0.7 * x1[1], atol=1e-12)
    assert np.allclose(z0[0], y0[0]) and np.allclose(z0[1], y0[1])


@pytest.mark.parametrize("isgnb, isgnw", [(1, 1), (2, 2)])
def test_reference_tfqmr_agrees_with_gmres(level, isgnb, isgnw):
    """The C restatement of solve_cf_tfqmr_spa (TFQMR from x = 0) against an independent GMRES.
    On this small hierarchy the Krylov space closes and TFQMR stops on an exact zero of
    rho or sigma (ierr 8) a little above crit, which the reference accepts as its result."""
    m, rho = level
    c = of.CF(m, 1, 1)
    w = 0.4 / of.HBAR
    xh, xa, info = c.tfqmr(rho, w, isgnb, isgnw, crit=1e-11, maxit0=40000, nthreads=1)
    assert info.resid <= 1e-9
    gh, ga, _ = c.solve(rho, w, isgnb, isgnw, tol=1e-13)
    assert np.linalg.norm(xh - gh) <= 1e-8 * np.linalg.norm(gh)
    assert np.linalg.norm(xa - ga) <= 1e-8 * np.linalg.norm(ga)
