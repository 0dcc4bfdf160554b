"""Known answers that pin the oracle (no GPU needed).

The reference ships no tests and no golden outputs, so the oracle is pinned by
physics with closed-form or independently computed answers:
  * U = 0: the fermionic hierarchy closes at tier 2 and the steady current equals the
    Landauer integral for the same Lorentzian bands, shifted with their bias
    (engyshift moves the whole lead, main/evaluatepara.f90:2428-2433);
  * particle-hole symmetric Anderson model: n_up + n_down = 1, I_L = -I_R, I(-V) = -I(V);
  * V = 0: no current, Tr rho = 1, rho Hermitian;
  * the TFQMR shadow-vector generator (tfqmr_double/drandn.f90) and the Chebyshev
    Bessel coefficients (td/chebyshev.f90 bessj) against independent code.
"""
import numpy as np
import pytest

import configs as cf
import oracle_ffi as of

HBAR = 0.658211928      # meV ps
JCONST = 1.602177e5     # current unit: e / ps in pA


def landauer_current(eps, V, gamma, W, T):
    """Spin-summed current into lead L of a resonant level between two Lorentzian leads
    (full width gamma at the band centre, half-width W, band centred on mu_alpha)."""
    from scipy.integrate import quad

    mus = (V / 2, -V / 2)

    def fermi(w, mu):
        return 0.5 * (1.0 - np.tanh((w - mu) / (2 * T)))

    def trans(w):
        g = [gamma * W * W / ((w - mu) ** 2 + W * W) for mu in mus]
        sig = sum(gamma * W / (2 * (w - mu + 1j * W)) for mu in mus)
        return g[0] * g[1] * abs(1.0 / (w - eps - sig)) ** 2

    val, _ = quad(lambda w: trans(w) * (fermi(w, mus[0]) - fermi(w, mus[1])), -V / 2 - 60 * T, V / 2 + 60 * T,
                  limit=400, epsabs=1e-14, epsrel=1e-12)
    return 2 * val * JCONST / (2 * np.pi * HBAR)


@pytest.mark.parametrize("V, T, W, nmats, tol", [(1.0, 0.2, 5.0, 10, 1e-7), (0.4, 0.5, 10.0, 10, 1e-7),
                                                 (0.4, 0.1, 10.0, 20, 1e-7)])
def test_noninteracting_current_is_landauer(V, T, W, nmats, tol):
    cfg = cf.siam(ntier=3, nmats=nmats, V=V, U=0.0, eps=0.3, T=T, W=W)
    m = of.Model(cfg)
    rho, _ = m.solve_tfqmr(crit=1e-12, maxit0=40000)
    jt = m.current(rho)
    ref = landauer_current(0.3, V, 0.5, W, T)
    assert abs(jt[0].sum() / ref - 1) < tol
    assert abs(jt[0].sum() + jt[1].sum()) < 1e-7 * abs(ref)


def test_noninteracting_hierarchy_closes_at_tier_two():
    cfgs = [cf.siam(ntier=n, nmats=4, V=0.4, U=0.0, eps=0.3, T=0.5) for n in (3, 4)]
    cur = []
    for cfg in cfgs:
        m = of.Model(cfg)
        rho, _ = m.solve_tfqmr(crit=1e-12, maxit0=40000)
        cur.append(m.current(rho)[0].sum())
    assert abs(cur[1] / cur[0] - 1) < 1e-9


def _solve(cfg):
    m = of.Model(cfg)
    rho, _ = m.solve_tfqmr(crit=1e-12, maxit0=40000)
    return m, rho


def test_particle_hole_symmetry():
    U = 2.0
    m, rho = _solve(cf.siam(ntier=3, nmats=4, V=0.6, U=U, eps=-U / 2))
    occ = m.occupation(rho)
    assert abs(occ.sum() - 1.0) < 1e-8
    jt = m.current(rho)
    assert abs(jt[0].sum() + jt[1].sum()) < 1e-8 * abs(jt[0].sum())
    m2, rho2 = _solve(cf.siam(ntier=3, nmats=4, V=-0.6, U=U, eps=-U / 2))
    j2 = m2.current(rho2)
    assert abs(j2[0].sum() + jt[0].sum()) < 1e-7 * abs(jt[0].sum())


def test_equilibrium():
    m, rho = _solve(cf.siam(ntier=3, nmats=4, V=0.0))
    jt = m.current(rho)
    assert np.max(np.abs(jt)) < 1e-6          # pA; the biased current is ~1e4
    nd = m.nrho
    r0 = np.zeros((nd, nd), dtype=complex)
    ir, ic = m.get("irow_spa"), m.get("icol_spa")
    nnz0 = m.get("nnz_spa")[0]
    r0[ir[:nnz0] - 1, ic[:nnz0] - 1] = rho[:nnz0]
    assert abs(np.trace(r0) - 1.0) < 1e-10
    assert np.max(np.abs(r0 - r0.conj().T)) < 1e-10


def test_drandn_is_the_published_lcg():
    """drandn.f90 with SEED = 1: the multiplier is 2^29 + 5 (found by doubling up to the
    32-bit limit), the modulus 2^31 - 1; each step emits seed / modulus, then
    seed <- |(multiplier * seed, wrapped to 32 bits) rem modulus|."""
    n = 1000
    a = of.drandn(n, seed=1)
    im, imax = 2 ** 29 + 5, 2 ** 31 - 1
    seed = 1
    ref = np.empty(n)
    for k in range(n):
        ref[k] = seed / imax
        prod = (im * seed) & 0xFFFFFFFF
        if prod >= 2 ** 31:
            prod -= 2 ** 32
        seed = abs(prod) % imax
    np.testing.assert_array_equal(a, ref)


@pytest.mark.parametrize("x", [0.5, 3.0, 17.0, 60.0])
def test_bessel_coefficients(x):
    from scipy.special import jv

    for n in (0, 1, 2, 5, 10, 30):
        ref = jv(n, x)
        got = of.besselj(n, x)
        assert abs(got - ref) <= 1e-12 * max(1.0, abs(ref))


def test_chebyshev_term_count_grows_with_the_spectral_width():
    n1 = of.cheby_nterms(10.0, 0.05)
    n2 = of.cheby_nterms(100.0, 0.05)
    assert 0 < n1 < n2


def test_augmented_system_null_space():
    """The reference's augmented steady-state system [L; Tr] x = e is singular but
    consistent: its real null space holds the free trace unknown x[lunk] (2 real
    directions) and nd - 1 anti-Hermitian stationary RDO directions, which change the
    current.  The mixed-precision solver regularises exactly these directions."""
    m = of.Model(cf.siam(ntier=3, nmats=2, V=0.4))
    n = m.lunk + 1
    M = np.zeros((2 * n, 2 * n))
    for k in range(n):
        for part in (0, 1):
            x = np.zeros(n, complex)
            x[k] = 1.0 if part == 0 else 1j
            y = m.calc_ax(x, nthreads=1)
            M[:n, part * n + k] = y.real
            M[n:, part * n + k] = y.imag
    u, s, vt = np.linalg.svd(M)
    null = np.where(s < 1e-11 * s[0])[0]
    assert len(null) == 2 + (m.nrho - 1)
    assert s[null[0] - 1] > 1e-4 * s[0]                       # a clear gap above the null space
    b = np.zeros(2 * n)
    b[n - 1] = 1.0
    assert np.sqrt(sum((u[:, j] @ b) ** 2 for j in null)) < 1e-13   # consistent
    currents = [np.abs(m.current(vt[j][: n - 1] + 1j * vt[j][n: 2 * n - 1])).max() for j in null]
    assert max(currents) > 1.0                                 # the null space moves the current
