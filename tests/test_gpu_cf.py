"""GPU parity of the correlation-function path (corrfunc/) against the oracle.

The operator (calc_ax_cf_spa_omp), the solves (solve_cf_tfqmr_spa) and the spectral
function (corrfunc.f90:146-217) run through the C ABI on the device and are compared with
the oracle's restatement on the same inputs; for U = 0 the spectral function is also checked
against the closed-form Green's function of the resonant level and of the serial double dot.
"""
import numpy as np
import pytest

import configs as cf
import heomq
import oracle_ffi as of

pytestmark = pytest.mark.gpu

T, V, W, GAMMA = 0.2, 0.4, 5.0, 0.5
MUS = (V / 2, -V / 2)

CASES = {
    "level_L2": cf.siam(ntier=3, nmats=4, V=V, U=0.0, eps=0.3, T=T, W=W),
    "siam_L3": cf.CFG0,
    "dqd_L2": cf.dqd(ntier=3),
    "hund_L1": cf.hund(ntier=2, nmats=2),
}


def rvec(n, seed):
    r = np.random.default_rng(seed)
    return r.standard_normal(n) + 1j * r.standard_normal(n)


@pytest.fixture(scope="module", params=list(CASES))
def setup(request):
    cfg = CASES[request.param]
    m = heomq.Model(cfg)
    return request.param, m, heomq.Context(m, adjoint=False), of.Model(cfg)


def _sigma(w, mu):
    return GAMMA * W / (2 * (w - mu + 1j * W))


def test_cf_apply_matches_oracle(setup):
    name, m, ctx, ref = setup
    for io in range(1, m.norbs + 1):
        for sp in (1, 2):
            c, r = heomq.CorrFunc(ctx, io, sp), of.CF(ref, io, sp)
            assert c.lunkcf == r.lunkcf
            xh, xa = rvec(c.lunkcf, 10 * io + sp), rvec(c.lunkcf, 100 + 10 * io + sp)
            for w, isgnw in ((0.0, 1), (0.7, 1), (1.3, 2)):
                yh, ya = c.calc_ax_cf_spa(w, isgnw, xh, xa)
                rh, ra = r.apply(w, isgnw, xh, xa)
                scale = np.linalg.norm(np.concatenate([rh, ra]))
                err = np.linalg.norm(np.concatenate([yh - rh, ya - ra]))
                assert err <= 1e-13 * scale, (name, io, sp, w, isgnw, err / scale)


def test_cf_pattern_passed_in_gives_the_same_operator(setup):
    """A caller's own nnzcf_spa etc. (the Fortran drop-in path) against the model's pattern."""
    name, m, ctx, ref = setup
    r = of.CF(ref, 1, 1)
    pat = {k: r.get(k) for k in ("nnzcf_spa", "indcf_spa", "irowcf_spa", "icolcf_spa")}
    c = heomq.CorrFunc(ctx, 1, 1, pattern=pat)
    xh, xa = rvec(c.lunkcf, 7), rvec(c.lunkcf, 8)
    yh, ya = c.calc_ax_cf_spa(0.4, 2, xh, xa)
    rh, ra = r.apply(0.4, 2, xh, xa)
    assert np.linalg.norm(np.concatenate([yh - rh, ya - ra])) <= 1e-13 * np.linalg.norm(np.concatenate([rh, ra]))


@pytest.mark.parametrize("isgnb, isgnw, checked", [(1, 1, 2), (2, 2, 1), (1, 2, 1)])
def test_cf_solve_matches_oracle(isgnb, isgnw, checked):
    cfg = CASES["siam_L3"]
    m = heomq.Model(cfg)
    ctx = heomq.Context(m, adjoint=False)
    ref = of.Model(cfg)
    rho, _ = ctx.solve_tfqmr(crit=1e-11, maxit0=40000)
    c, r = heomq.CorrFunc(ctx, 1, 1), of.CF(ref, 1, 1)
    w = np.array([-0.8, 0.3]) / of.HBAR
    zh, za, info = c.solve_cf_tfqmr_spa(rho, isgnb, isgnw, w, crit=1e-11, maxit0=40000)
    assert info.converged and info.resid <= 1e-11
    for k in range(checked):
        xh, xa, res = r.solve(rho, w[k], isgnb, isgnw, tol=1e-13)
        for got, want in ((zh[k], r.rdo(xh)), (za[k], r.rdo(xa))):
            assert np.linalg.norm(got - want) <= 1e-8 * np.linalg.norm(want)


def test_resonant_level_spectral_function():
    m = heomq.Model(CASES["level_L2"])
    ctx = heomq.Context(m, adjoint=False)
    rho, _ = ctx.solve_tfqmr(crit=1e-11, maxit0=40000)
    freqs = np.linspace(-2.0, 2.5, 19)
    for sp in (1, 2):
        out, info = heomq.CorrFunc(ctx, 1, sp).dos(rho, freqs, crit=1e-11, maxit0=40000)
        assert info.converged
        g = 1.0 / (freqs - 0.3 - sum(_sigma(freqs, mu) for mu in MUS))
        np.testing.assert_allclose(out[:, 0], -g.imag / np.pi, rtol=1e-8)
        np.testing.assert_allclose(out[:, 3] + 1j * out[:, 4], g, rtol=1e-8)
        np.testing.assert_allclose(out[:, 0], out[:, 1] + out[:, 2], rtol=1e-14)


@pytest.mark.parametrize("iorbs", [1, 2])
def test_double_dot_spectral_function(iorbs):
    m = heomq.Model(cf.dqd(ntier=3, nmats=2, V=V, U=0.0, eps=0.3, t=0.5, T=T, W=W))
    ctx = heomq.Context(m, adjoint=False)
    rho, _ = ctx.solve_tfqmr(crit=1e-11, maxit0=40000)
    freqs = np.linspace(-1.5, 2.0, 8)
    out, info = heomq.CorrFunc(ctx, iorbs, 1).dos(rho, freqs, crit=1e-11, maxit0=40000)
    assert info.converged
    for k, w in enumerate(freqs):
        g = np.linalg.inv(np.array([[w - 0.3 - _sigma(w, MUS[0]), -0.5], [-0.5, w - 0.3 - _sigma(w, MUS[1])]]))
        assert abs(out[k, 0] / (-g[iorbs - 1, iorbs - 1].imag / np.pi) - 1) < 1e-8


def test_interacting_spectral_function_matches_oracle():
    cfg = CASES["siam_L3"]
    m = heomq.Model(cfg)
    ctx = heomq.Context(m, adjoint=False)
    ref = of.Model(cfg)
    rho, _ = ctx.solve_tfqmr(crit=1e-11, maxit0=40000)
    rho_ref, _ = ref.solve_tfqmr(crit=1e-11, maxit0=40000)
    freqs = np.array([-1.2, 0.9])
    out, info = heomq.CorrFunc(ctx, 1, 1).dos(rho, freqs, crit=1e-11, maxit0=40000)
    assert info.converged
    r = of.CF(ref, 1, 1)
    for k, w in enumerate(freqs):
        A, d1, d2 = r.dos(rho_ref, w, tol=1e-13)
        np.testing.assert_allclose(out[k, :3], [A, d1, d2], rtol=1e-8, atol=1e-12)


def test_batched_frequencies_match_single_solves():
    cfg = CASES["siam_L3"]
    m = heomq.Model(cfg)
    ctx = heomq.Context(m, adjoint=False)
    rho, _ = ctx.solve_tfqmr(crit=1e-11, maxit0=40000)
    c = heomq.CorrFunc(ctx, 1, 2)
    freqs = np.linspace(-3, 3, 12)
    out, _ = c.dos(rho, freqs, crit=1e-11, maxit0=40000)
    for k in (0, 5, 11):
        one, _ = c.dos(rho, freqs[k:k + 1], crit=1e-11, maxit0=40000)
        np.testing.assert_allclose(one[0], out[k], rtol=1e-9, atol=1e-13)


@pytest.mark.parametrize("name, crit", [("siam_L3", 1e-11), ("dqd_L2", 1e-10)])
def test_mixed_precision_spectral_function_matches_fp64(name, crit):
    """FP32x2 inner solves with FP64 refinement reach the same spectra as the FP64 TFQMR."""
    m = heomq.Model(CASES[name])
    ctx = heomq.Context(m, adjoint=False)
    rho, _ = ctx.solve_tfqmr(crit=1e-11, maxit0=40000, precision=heomq.PREC_MIXED)
    c = heomq.CorrFunc(ctx, 1, 1)
    freqs = np.linspace(-2.5, 2.5, 9)
    ref, i64 = c.dos(rho, freqs, crit=crit, maxit0=40000)
    got, imx = c.dos(rho, freqs, crit=crit, maxit0=40000, precision=heomq.PREC_MIXED)
    assert i64.converged and imx.converged and imx.resid <= crit
    np.testing.assert_allclose(got, ref, rtol=100 * crit, atol=1e-12)


def test_time_domain_matches_oracle_rk4():
    """corrfunc's time-domain branch: RK4 of X(0) = B rho under the cf operator (no frequency
    terms) against the same RK4 on the oracle's operator, and C(t) = Tr[a (X_h + i X_a)/2]."""
    cfg = CASES["siam_L3"]
    m = heomq.Model(cfg)
    ctx = heomq.Context(m, adjoint=False)
    ref = of.Model(cfg)
    rho, _ = ctx.solve_tfqmr(crit=1e-11, maxit0=40000, precision=heomq.PREC_MIXED)
    c, r = heomq.CorrFunc(ctx, 1, 1), of.CF(ref, 1, 1)
    dt, nstep = 0.02, 12
    corr = c.propagate(rho, dt, nstep, ljw=True)
    # t = 0: <a^dag a> = n_up and <a a^dag> = 1 - n_up
    n_up = ctx.occupation(rho)[0, 0]
    assert abs(corr[0, 0] - n_up) < 1e-12 and abs(corr[0, 1] - (1 - n_up)) < 1e-12
    a = ref.dense_op(1, 1)
    for isgnb, col in ((2, 0), (1, 1)):
        xh, xa = r.rhs(rho, isgnb)
        for k in range(nstep + 1):
            z = 0.5 * r.rdo(xh) + 0.5j * r.rdo(xa)
            want = np.trace(a.conj().T @ z) if col == 0 else np.conj(np.trace(a @ z))
            assert abs(corr[k, col] - want) <= 1e-11 * max(1.0, abs(want)), (isgnb, k)
            k1 = r.apply(0.0, 1, xh, xa)
            k2 = r.apply(0.0, 1, xh + dt / 2 * k1[0], xa + dt / 2 * k1[1])
            k3 = r.apply(0.0, 1, xh + dt / 2 * k2[0], xa + dt / 2 * k2[1])
            k4 = r.apply(0.0, 1, xh + dt * k3[0], xa + dt * k3[1])
            xh = xh + dt / 6 * (k1[0] + 2 * k2[0] + 2 * k3[0] + k4[0])
            xa = xa + dt / 6 * (k1[1] + 2 * k2[1] + 2 * k3[1] + k4[1])


def test_time_and_frequency_domains_agree():
    """The frequency-domain solution is the Laplace transform of the time-domain one: with
    L_w = L + w J for isgnw = 2 (J (h, a) = (a, -h), which commutes with L),
    X_h(w) = int cos(wt) X_h(t) + sin(wt) X_a(t) dt and X_a(w) = int cos(wt) X_a(t) - sin(wt) X_h(t) dt."""
    m = heomq.Model(CASES["level_L2"])
    ctx = heomq.Context(m, adjoint=False)
    rho, _ = ctx.solve_tfqmr(crit=1e-11, maxit0=40000, precision=heomq.PREC_MIXED)
    c = heomq.CorrFunc(ctx, 1, 1)
    dt, nstep = 0.01, 4000
    _, xh_t, xa_t = c.propagate(rho, dt, nstep, ljw=False, rdo=True)
    t = dt * np.arange(nstep + 1)
    w_simp = np.ones(nstep + 1)
    w_simp[1:-1:2], w_simp[2:-1:2] = 4, 2
    w_simp *= dt / 3
    for w in (0.4, 1.3):
        cw, sw = np.cos(w * t)[:, None, None], np.sin(w * t)[:, None, None]
        lap_h = np.tensordot(w_simp, cw * xh_t + sw * xa_t, axes=1)
        lap_a = np.tensordot(w_simp, cw * xa_t - sw * xh_t, axes=1)
        zh, za, info = c.solve_cf_tfqmr_spa(rho, 2, 2, [w], crit=1e-12, maxit0=40000)
        scale = np.linalg.norm(zh[0]) + np.linalg.norm(za[0])
        assert np.linalg.norm(lap_h - zh[0]) + np.linalg.norm(lap_a - za[0]) <= 1e-6 * scale, w
