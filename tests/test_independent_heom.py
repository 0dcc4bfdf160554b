"""Parity pinned independently of the oracle: a dense hierarchy assembled in numpy from the
published fermionic HEOM (tests/dense_heom.py, which reads neither oracle/ nor the library's
tables) is itself pinned by exact answers, then compared with the oracle on interacting
single-orbital and double-dot models.

  1. The hierarchy against the exact reduced dynamics of a system (one spinless level; a
     spinful level with U and hopping) coupled to a few discrete bath modes: the bath
     correlation functions are exact finite sums of exponentials and the hierarchy
     terminates by Pauli exclusion, so the two must agree to rounding.
  2. Its Pade decomposition of the Fermi function against the Fermi function, and against
     the poles and residues of the oracle and of the library's model builder.
  3. U = 0: its steady current against the Landauer formula (the Fermi functions replaced by
     the same Pade approximant, for which the hierarchy is exact at tier 2), for the
     resonant level and for the serial double dot; the oracle's double-dot current
     (tfqmr_double/calc_ax_tfqmr_spa_omp.f90 with the multi-orbital Jordan-Wigner signs of
     :316-318, :369-370) against the same formula.
  4. U != 0: the oracle's steady state (occupations, lead currents per spin, double
     occupancy, inter-dot coherence, the RDO spectrum) and its RK4 transients
     (td/calcderiv_spa_omp.f90, td/intstp.f90) against the dense hierarchy.
"""
import numpy as np
import pytest
import scipy.linalg as sl

import configs as cf
import dense_heom as dh
import heomq
import oracle_ffi as of


# ----------------------------------------------------------------------------- helpers
def exact_rdo(hs_fn, ns, modes, rho_s0, times):
    """Reduced density matrix of ns system modes coupled to discrete bath modes
    [(mu, t, eps, f)], from rho_s0 times the thermal bath state, by exact evolution in the
    full Fock space (system modes first, so the system operators are O_S x 1_B)."""
    nb = len(modes)
    a = dh.annihilators(ns + nb)
    H = hs_fn(a[:ns])
    for k, (mu, t, eps, f) in enumerate(modes):
        d = a[ns + k]
        H = H + eps * d.T @ d + t * a[mu].T @ d + np.conj(t) * d.T @ a[mu]
    pb = np.array([np.prod([f if (b >> k) & 1 else 1 - f for k, (_, _, _, f) in enumerate(modes)])
                   for b in range(1 << nb)])
    ds = 1 << ns
    W0 = np.kron(np.diag(pb), rho_s0)
    out = []
    for t in times:
        U = sl.expm(-1j * H * t)
        W = U @ W0 @ U.conj().T
        out.append(sum(W[b * ds:(b + 1) * ds, b * ds:(b + 1) * ds] for b in range(1 << nb)))
    return out


def mode_index(norbs):
    """This module's spin-orbital numbering: mu = orbital + norbs * spin."""
    return {(o, s): o + norbs * s for s in range(2) for o in range(norbs)}


def dense_model(norbs, eps, U, t, V, gamma, W, T, npade, ntier):
    """The single-orbital model (norbs = 1, both leads on the level) or the serial double dot
    (norbs = 2, lead 0 on dot 0, lead 1 on dot 1), H in energy / hbar."""
    nm = 2 * norbs
    a = dh.annihilators(nm)
    n = [x.T @ x for x in a]
    idx = mode_index(norbs)
    H = np.zeros((1 << nm, 1 << nm))
    for o in range(norbs):
        H += eps * (n[idx[(o, 0)]] + n[idx[(o, 1)]]) + U * n[idx[(o, 0)]] @ n[idx[(o, 1)]]
    if norbs == 2:
        for s in range(2):
            c1, c2 = a[idx[(0, s)]], a[idx[(1, s)]]
            H += t * (c1.T @ c2 + c2.T @ c1)
    leads = [[0], [0]] if norbs == 1 else [[0], [1]]
    coup = {(al, idx[(o, s)]): gamma for al, orbs in enumerate(leads) for o in orbs for s in range(2)}
    bath = dh.lorentz_psd_bath(coup, W, T, [V / 2, -V / 2], npade)
    return dh.Hierarchy(H / dh.HBAR, a, bath, ntier), a, n, idx, H


def landauer_psd(norbs, eps, t, V, gamma, W, T, npade):
    """Spin-summed Landauer current into the system from lead 0 (pA), with the Fermi functions
    replaced by their [npade-1/npade] Pade approximant: T(w) = G0 G1 |G_{01}(w)|^2."""
    from scipy.integrate import quad

    xi, kap = dh.psd_fermi(npade)
    mus = (V / 2, -V / 2)

    def f(w, mu):
        return dh.fermi_psd((w - mu) / T, xi, kap).real

    def trans(w):
        g = [gamma * W * W / ((w - mu) ** 2 + W * W) for mu in mus]
        s = [gamma * W / (2 * (w - mu + 1j * W)) for mu in mus]
        if norbs == 1:
            return g[0] * g[1] * abs(1.0 / (w - eps - s[0] - s[1])) ** 2
        G = np.linalg.inv(np.array([[w - eps - s[0], -t], [-t, w - eps - s[1]]]))
        return g[0] * g[1] * abs(G[0, 1]) ** 2

    val, _ = quad(lambda w: trans(w) * (f(w, mus[0]) - f(w, mus[1])), -400, 400, points=[-V / 2, V / 2, eps],
                  limit=2000, epsabs=1e-15, epsrel=1e-13)
    return 2 * val * dh.JCONST / (2 * np.pi * dh.HBAR)


def oracle_rdo(m, rho):
    nz = m.get("nnz_spa")[0]
    ir, ic = m.get("irow_spa")[:nz] - 1, m.get("icol_spa")[:nz] - 1
    r = np.zeros((m.nrho, m.nrho), dtype=complex)
    r[ir, ic] = rho[:nz]
    return r


def observables_dense(h, x, a, idx, norbs):
    """Occupations [orb, spin], currents [lead, spin] (pA), double occupancies per orbital,
    Re <c^+_{0s} c_{1s}> per spin (double dot) and the RDO spectrum."""
    r = h.rdo(x)
    occ = np.array([[np.trace(a[idx[(o, s)]].T @ a[idx[(o, s)]] @ r).real for s in range(2)] for o in range(norbs)])
    nspin = [sum(a[idx[(o, s)]].T @ a[idx[(o, s)]] for o in range(norbs)) for s in range(2)]
    cur = np.array([[h.lead_rate(x, al, nspin[s]) * dh.JCONST for s in range(2)] for al in range(2)])
    dbl = np.array([np.trace(a[idx[(o, 0)]].T @ a[idx[(o, 0)]] @ a[idx[(o, 1)]].T @ a[idx[(o, 1)]] @ r).real
                    for o in range(norbs)])
    coh = (np.array([np.trace(a[idx[(0, s)]].T @ a[idx[(1, s)]] @ r).real for s in range(2)]) if norbs == 2 else None)
    return occ, cur, dbl, coh, np.sort(np.linalg.eigvalsh(0.5 * (r + r.conj().T)))


def observables_oracle(m, rho, norbs):
    r = oracle_rdo(m, rho)
    ops = {(o, s): m.dense_op(o + 1, s + 1) for o in range(norbs) for s in range(2)}
    occ = m.occupation(rho)
    cur = m.current(rho)
    dbl = np.array([np.trace(ops[(o, 0)].T @ ops[(o, 0)] @ ops[(o, 1)].T @ ops[(o, 1)] @ r).real for o in range(norbs)])
    coh = (np.array([np.trace(ops[(0, s)].T @ ops[(1, s)] @ r).real for s in range(2)]) if norbs == 2 else None)
    return occ, cur, dbl, coh, np.sort(np.linalg.eigvalsh(0.5 * (r + r.conj().T)))


# ----------------------------------------------------------------------------- 1. exact
def test_hierarchy_reproduces_exact_discrete_bath_dynamics():
    times = [0.5, 1.3, 3.0]
    # a spinless level and two bath modes
    a1 = dh.annihilators(1)
    modes = [(0, 0.4, 0.7, 0.3), (0, 0.25, -0.5, 0.8)]
    rho0 = np.diag([0.35, 0.65]).astype(complex)
    ex = exact_rdo(lambda o: 0.3 * o[0].T @ o[0], 1, modes, rho0, times)
    h = dh.Hierarchy(0.3 * a1[0].T @ a1[0], a1, dh.discrete_bath(modes), ntier=4)
    for r, x in zip(ex, h.evolve(rho0, times)):
        assert np.abs(h.rdo(x) - r).max() < 1e-13

    # two modes with interaction and hopping, two bath modes each (hierarchy complete at tier 8)
    def hs(o):
        n0, n1 = o[0].T @ o[0], o[1].T @ o[1]
        return -0.4 * (n0 + n1) + 1.1 * n0 @ n1 + 0.2 * (o[0].T @ o[1] + o[1].T @ o[0])

    a2 = dh.annihilators(2)
    modes = [(0, 0.3, 0.5, 0.2), (1, 0.35, -0.6, 0.7), (0, 0.2, -0.2, 0.6), (1, 0.15, 0.9, 0.1)]
    rho0 = np.diag([0.1, 0.3, 0.4, 0.2]).astype(complex)
    ex = exact_rdo(hs, 2, modes, rho0, times)
    h = dh.Hierarchy(hs(a2), a2, dh.discrete_bath(modes), ntier=8)
    for r, x in zip(ex, h.evolve(rho0, times)):
        assert np.abs(h.rdo(x) - r).max() < 1e-13
        assert np.abs(r - rho0).max() > 1e-2            # the state has moved


# ----------------------------------------------------------------------------- 2. Pade
@pytest.mark.parametrize("npade", [2, 4, 6])
def test_pade_decomposition_matches_the_oracle_and_the_builder(npade):
    xi, kappa = dh.psd_fermi(npade)
    m = of.Model(cf.siam(ntier=2, nmats=npade))
    # the reference writes f(x) = 1/2 + sum_p cpcoef_p (1/(x + pole_p) + 1/(x - pole_p)) with the
    # poles +-i xi_p (cppole(2, nmats)), i.e. cpcoef = -kappa
    pole = m.get("cppole")
    np.testing.assert_allclose(pole[0::2], 1j * xi, rtol=1e-12)
    np.testing.assert_allclose(pole[1::2], -1j * xi, rtol=1e-12)
    np.testing.assert_allclose(m.get("cpcoef"), -kappa, rtol=1e-11)
    x = np.linspace(-15, 15, 301)
    ref = 0.5 + sum(c * (1 / (x + p) + 1 / (x - p)) for c, p in zip(m.get("cpcoef"), pole[0::2]))
    np.testing.assert_allclose(ref.real, dh.fermi_psd(x, xi, kappa).real, atol=1e-12)
    b = heomq.Model(cf.siam(ntier=2, nmats=npade))
    np.testing.assert_allclose(b.get("cpcoef", npade, np.float64), m.get("cpcoef"), rtol=1e-11)


def test_pade_approximant_converges_to_the_fermi_function():
    x = np.linspace(-30, 30, 2001)
    for npade, tol in ((10, 1e-10), (20, 1e-13)):
        xi, kappa = dh.psd_fermi(npade)
        assert np.abs(dh.fermi_psd(x, xi, kappa).real - 1 / (1 + np.exp(x))).max() < tol


# ----------------------------------------------------------------------------- 3. U = 0
@pytest.mark.parametrize("norbs, npade", [(1, 2), (2, 1)], ids=["resonant_level", "double_dot"])
def test_dense_hierarchy_noninteracting_current_is_landauer(norbs, npade):
    h, a, n, idx, _ = dense_model(norbs, eps=0.3, U=0.0, t=0.5, V=0.8, gamma=0.5, W=10.0, T=0.5, npade=npade, ntier=2)
    x = h.steady()
    N = sum(n)
    IL, IR = h.lead_rate(x, 0, N) * dh.JCONST, h.lead_rate(x, 1, N) * dh.JCONST
    ref = landauer_psd(norbs, 0.3, 0.5, 0.8, 0.5, 10.0, 0.5, npade)
    assert abs(IL / ref - 1) < 1e-10
    assert abs(IL + IR) < 1e-10 * abs(ref)


@pytest.mark.parametrize("T, npade", [(0.5, 3), (0.2, 4)])
def test_oracle_double_dot_noninteracting_current_is_landauer(T, npade):
    """The oracle's serial double dot at U = 0 (tier 2 is exact there): its lead currents
    against T(w) = G_L G_R |G_12(w)|^2 with the same Pade Fermi functions; this pins the
    inter-orbital Jordan-Wigner signs of the couplings, which the single-level test cannot."""
    cfg = cf.dqd(ntier=3, nmats=npade, V=0.8, U=0.0, eps=0.3, t=0.5, T=T)
    m = of.Model(cfg)
    rho, _ = m.solve_tfqmr(crit=1e-12, maxit0=40000)
    jt = m.current(rho)
    ref = landauer_psd(2, 0.3, 0.5, 0.8, 0.5, 10.0, T, npade)
    assert abs(jt[0].sum() / ref - 1) < 1e-8
    assert abs(jt[0].sum() + jt[1].sum()) < 1e-8 * abs(ref)
    np.testing.assert_allclose(jt[0, 0], jt[0, 1], rtol=1e-8)     # spin degenerate


# ----------------------------------------------------------------------------- 4. U != 0
INTERACTING = {
    "siam_U2": (1, dict(eps=-0.7, U=2.0, t=0.0, V=0.6, gamma=0.5, W=10.0, T=0.3, npade=1)),
    "dqd_U2": (2, dict(eps=-1.0, U=2.0, t=0.5, V=0.8, gamma=0.5, W=10.0, T=0.3, npade=1)),
}


def oracle_cfg(norbs, p, ntier):
    if norbs == 1:
        return cf.siam(ntier=ntier + 1, nmats=p["npade"], V=p["V"], U=p["U"], eps=p["eps"], gamma=p["gamma"], W=p["W"],
                       T=p["T"])
    return cf.dqd(ntier=ntier + 1, nmats=p["npade"], V=p["V"], U=p["U"], eps=p["eps"], t=p["t"], gamma=p["gamma"],
                  W=p["W"], T=p["T"])


@pytest.fixture(scope="module", params=list(INTERACTING))
def interacting(request):
    norbs, p = INTERACTING[request.param]
    h, a, n, idx, H = dense_model(norbs, ntier=2, **p)
    return request.param, norbs, p, h, a, idx, H


def test_oracle_steady_state_matches_dense_hierarchy(interacting):
    name, norbs, p, h, a, idx, H = interacting
    x = h.steady()
    d_occ, d_cur, d_dbl, d_coh, d_spec = observables_dense(h, x, a, idx, norbs)
    m = of.Model(oracle_cfg(norbs, p, 2))
    rho, info = m.solve_tfqmr(crit=1e-12, maxit0=40000)
    o_occ, o_cur, o_dbl, o_coh, o_spec = observables_oracle(m, rho, norbs)
    scale = np.abs(d_cur).max()
    np.testing.assert_allclose(o_occ, d_occ, atol=1e-9, err_msg=name)
    np.testing.assert_allclose(o_cur, d_cur, atol=1e-8 * scale, err_msg=name)
    np.testing.assert_allclose(o_dbl, d_dbl, atol=1e-9, err_msg=name)
    np.testing.assert_allclose(o_spec, d_spec, atol=1e-9, err_msg=name)
    if norbs == 2:
        np.testing.assert_allclose(o_coh, d_coh, atol=1e-9, err_msg=name)
    assert scale > 1e3 and np.abs(d_dbl).max() > 1e-3       # a biased, interacting state


def test_oracle_initial_guess_is_the_boltzmann_state(interacting):
    """analyze_hs + initialize1_spa: the RDO guess is exp(-H/T) / Z at the lead-1 temperature
    (its spectrum and occupations against the dense Boltzmann state), all ADOs zero."""
    name, norbs, p, h, a, idx, H = interacting
    w, v = np.linalg.eigh(H)
    b = v @ np.diag(np.exp(-(w - w.min()) / p["T"])) @ v.conj().T
    b /= np.trace(b)
    m = of.Model(oracle_cfg(norbs, p, 2))
    g = m.initial_guess()
    nz = m.get("nnz_spa")[0]
    assert np.abs(g[nz:]).max() == 0.0
    r = oracle_rdo(m, g)
    np.testing.assert_allclose(np.sort(np.linalg.eigvalsh(r)), np.sort(np.linalg.eigvalsh(b)), atol=1e-12)
    np.testing.assert_allclose(m.occupation(g).sum(), sum(np.trace(a[k].T @ a[k] @ b).real for k in range(len(a))),
                               atol=1e-12)


def test_oracle_rk4_transient_matches_dense_hierarchy(interacting):
    """From the Boltzmann state with the bias switched on (all ADOs zero): the oracle's RK4
    steps of calcderiv (dt = 2.5e-4 ps) against the exponential of the dense generator, at
    t = 0.1 and 0.25 ps (occupations, lead currents, RDO spectrum)."""
    name, norbs, p, h, a, idx, H = interacting
    w, v = np.linalg.eigh(H)
    b = v @ np.diag(np.exp(-(w - w.min()) / p["T"])) @ v.conj().T
    b /= np.trace(b)
    times = [0.1, 0.25]
    xs = h.evolve(b, times)
    m = of.Model(oracle_cfg(norbs, p, 2))
    rho = m.initial_guess()
    dt, t = 2.5e-4, 1e-9        # t > 0 at every stage: the step bias is on throughout
    for target, x in zip(times, xs):
        while t < target - 1e-12:
            rho = m.rk4_step(t, dt, rho)
            t += dt
        d_occ, d_cur, _, _, d_spec = observables_dense(h, x, a, idx, norbs)
        o_occ, o_cur, _, _, o_spec = observables_oracle(m, rho, norbs)
        scale = np.abs(d_cur).max()
        np.testing.assert_allclose(o_occ, d_occ, atol=1e-9, err_msg=f"{name} t={target}")
        np.testing.assert_allclose(o_cur, d_cur, atol=1e-7 * scale, err_msg=f"{name} t={target}")
        np.testing.assert_allclose(o_spec, d_spec, atol=1e-9, err_msg=f"{name} t={target}")
        assert scale > 1e2
