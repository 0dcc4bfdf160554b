"""The oracle's restatement of the Jacobi steady-state iteration (jacobi/), pinned against
independent answers (no GPU needed): its fixed point is the TFQMR steady state, the Hermitian
eigen-solver it uses reproduces its input, and the shift follows prelude_jacobi's rule."""
import numpy as np
import pytest

import configs as cf
import oracle_ffi as of


@pytest.mark.parametrize("n", [1, 4, 16, 33])
def test_hermitian_eigen_decomposition(n):
    r = np.random.default_rng(n)
    a = r.standard_normal((n, n)) + 1j * r.standard_normal((n, n))
    a = a + a.conj().T
    w, v = of.herm_eig(a)
    assert np.linalg.norm(v @ np.diag(w) @ v.conj().T - a) <= 1e-12 * np.linalg.norm(a)
    assert np.linalg.norm(v.conj().T @ v - np.eye(n)) <= 1e-12 * n
    np.testing.assert_allclose(np.sort(w), np.linalg.eigvalsh(a), atol=1e-12 * np.abs(w).max())


@pytest.mark.parametrize("cfg", [cf.siam(ntier=3), cf.CFG0], ids=["siam_L2", "siam_L3"])
def test_jacobi_fixed_point_is_the_steady_state(cfg):
    """With twice the shift of prelude_jacobi's rule (the $jacobi e_jacobi input); at the rule's
    own shift the SIAM L2 iteration does not contract (its residual hovers near 1)."""
    m = of.Model(cfg)
    J = of.Jacobi(m, ejac=2 * of.Jacobi(m).ejac)
    rho, info = J.solve(m.initial_guess(), crit=1e-10, maxit0=20000)
    assert info.resid <= 1e-10
    ref, _ = m.solve_tfqmr(crit=1e-12, maxit0=40000)
    assert np.linalg.norm(rho - ref) <= 1e-8 * np.linalg.norm(ref)
    assert abs(m.current(rho)[0].sum() / m.current(ref)[0].sum() - 1) < 1e-8


def test_shift_rule():
    """ejac = max(span of the nonzero eigenvalues of [H, .], sqrt((ntier - 1) max|cb|))."""
    cfg = cf.CFG0
    m = of.Model(cfg)
    e = np.linalg.eigvalsh(m.get("hs").reshape(m.nrho, m.nrho, order="F"))
    cb = np.abs(m.get("cb")).max()
    want = max(2 * (e.max() - e.min()), np.sqrt((m.ntier - 1) * cb))
    assert abs(of.Jacobi(m).ejac / want - 1) < 1e-12


def test_sweep_keeps_the_trace():
    m = of.Model(cf.siam(ntier=3))
    J = of.Jacobi(m)
    x = m.initial_guess()
    r = np.random.default_rng(3)
    nz0 = int(m.get("nnz_spa")[0])
    x[nz0:] = 1e-2 * (r.standard_normal(m.lunk - nz0) + 1j * r.standard_normal(m.lunk - nz0))
    rows, cols = m.get("irow_spa")[:nz0], m.get("icol_spa")[:nz0]
    diag = rows == cols
    xn = J.sweep(x)
    assert abs(xn[:nz0][diag].sum() - x[:nz0][diag].sum()) < 1e-13
