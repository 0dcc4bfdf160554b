"""Dense fermionic HEOM assembled in numpy from the published equations: test infrastructure,
independent of oracle/ and of the library's table builder.

The hierarchy is the one of Jin, Zheng and Yan, J. Chem. Phys. 128, 234703 (2008), written
here for a system whose spin-orbitals mu couple diagonally to non-interacting leads alpha:

    d/dt rho_J = -(i L + sum_{j in J} gamma_j) rho_J
                 - i sum_{j not in J} A_jbar rho_{J + j}
                 - i sum_{r = 1..n} (-1)^(n - r) C_{j_r} rho_{J - j_r}

with J = (j_1 < ... < j_n) an ordered tuple of distinct "drawers" j = (sigma, alpha, mu, m),
rho_{J + j} the tuple with j appended (re-sorted with the sign of the permutation),
    A_jbar X = a^{sigma bar}_mu X + (-1)^{|X|} X a^{sigma bar}_mu,
    C_j X    = eta_j a^sigma_mu X - (-1)^{|X|} conj(eta_{jbar}) X a^sigma_mu,
|X| the tier of X, a^+ = a^dagger, a^- = a, and the bath correlation functions
    C^sigma_{alpha mu}(t) = sum_m eta_{sigma alpha mu m} exp(-gamma_{sigma alpha mu m} t),
    C^+(t) = <F^dagger(t) F(0)>_B,  C^-(t) = <F(t) F^dagger(0)>_B,  F = sum_k t_k d_k.
The sign conventions of A and C are those that reproduce the exact reduced dynamics of a
system coupled to a few discrete bath modes (where the decomposition of C(t) is exact and the
hierarchy terminates by Pauli exclusion); tests/test_independent_heom.py checks exactly that.

Vectorisation: each ADO is an nd x nd matrix stacked column-major; the generator is a sparse
matrix on the stacked vector.  The Fock basis is this module's own: bit i of a basis index is
the occupation of mode i, with Jordan-Wigner strings over the lower modes.
"""
import itertools

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

HBAR = 0.658211928      # meV ps
JCONST = 1.602177e5     # e / ps in pA


# ----------------------------------------------------------------------------- Fock space
def annihilators(nmodes):
    """Dense Jordan-Wigner annihilation operators of nmodes fermionic modes."""
    dim = 1 << nmodes
    ops = []
    for i in range(nmodes):
        a = np.zeros((dim, dim))
        for s in range(dim):
            if s >> i & 1:
                sign = (-1) ** bin(s & ((1 << i) - 1)).count("1")
                a[s ^ (1 << i), s] = sign
        ops.append(a)
    return ops


# ----------------------------------------------------------------------------- Pade (PSD)
def psd_fermi(n):
    """[n-1/n] Pade spectrum decomposition of the Fermi function (Hu, Xu and Yan, J. Chem.
    Phys. 133, 101106 (2010)): 1/(1 + e^x) ~ 1/2 - sum_j 2 kappa_j x / (x^2 + xi_j^2).
    xi: 2 / (positive eigenvalues) of the 2n x 2n tridiagonal matrix 1/sqrt(b_m b_{m+1}),
    b_m = 2m - 1; the residues from the interlacing zeros zeta (the (2n-1) x (2n-1) matrix
    with b shifted by one)."""
    b = np.array([2.0 * m - 1.0 for m in range(1, 2 * n + 2)])

    def poles(k, shift):
        lam = np.zeros((k, k))
        for i in range(k - 1):
            lam[i, i + 1] = lam[i + 1, i] = 1.0 / np.sqrt(b[i + shift] * b[i + 1 + shift])
        ev = np.sort(np.linalg.eigvalsh(lam))[::-1][: k // 2]   # the positive half (odd k: one zero)
        return np.sort(2.0 / ev)

    xi = poles(2 * n, 0)
    zeta = poles(2 * n - 1, 1)
    kappa = np.empty(n)
    for j in range(n):
        num = np.prod(zeta ** 2 - xi[j] ** 2)
        den = np.prod([xi[k] ** 2 - xi[j] ** 2 for k in range(n) if k != j])
        kappa[j] = 0.5 * n * b[n] * num / den
    return xi, kappa


def fermi_psd(x, xi, kappa):
    x = np.asarray(x, dtype=complex)
    return 0.5 - sum(2 * k * x / (x * x + s * s) for s, k in zip(xi, kappa))


# ----------------------------------------------------------------------------- baths
class Drawer:
    __slots__ = ("sigma", "alpha", "mu", "m", "gamma", "eta")

    def __init__(self, sigma, alpha, mu, m, gamma, eta):
        self.sigma, self.alpha, self.mu, self.m, self.gamma, self.eta = sigma, alpha, mu, m, gamma, eta

    def key(self):
        return (self.sigma, self.alpha, self.mu, self.m)


def lorentz_psd_bath(couplings, W, T, mus, npade):
    """Drawers of Lorentzian leads, Gamma_{alpha mu}(w) = g W^2 / ((w - mu_alpha)^2 + W^2)
    (couplings[(alpha, mu)] = g, the full width at the band centre; the band moves with the
    lead's chemical potential), Fermi functions at temperature T replaced by their [n-1/n]
    Pade decomposition.  Contour integration of C^sigma(t) = 1/(2 pi) int dw e^{sigma i w t}
    Gamma(w) f^sigma(w - mu) (f^+ = f, f^- = 1 - f) over the half plane where the exponential
    decays gives the Lorentzian pole (m = 0) and the Pade poles (m = 1..n).  Energies in
    meV, rates in 1/ps (divided by hbar)."""
    xi, kappa = psd_fermi(npade)
    out = []
    for (alpha, mu), g in sorted(couplings.items()):
        ma = mus[alpha]
        for sigma in (1, -1):
            # Lorentzian pole w = mu_a + sigma i W
            fz = fermi_psd(sigma * 1j * W / T, xi, kappa)
            fs = fz if sigma == 1 else 1.0 - fz
            out.append(Drawer(sigma, alpha, mu, 0, (W - sigma * 1j * ma) / HBAR, 0.5 * g * W * fs / HBAR ** 2))
            for p in range(npade):
                z = xi[p] * T
                eta = -1j * kappa[p] * T * g * W * W / (W * W - z * z)
                out.append(Drawer(sigma, alpha, mu, p + 1, (z - sigma * 1j * ma) / HBAR, eta / HBAR ** 2))
    return out


def exponential_bath(couplings, mus, terms):
    """Drawers of leads whose correlation functions are given as sums of exponentials in the
    lead's own frame, C^sigma(t) = g sum_m eta_m exp(-gamma_m t) for both signs (a Prony fit of
    a band centred at the lead's chemical potential; terms = [(eta_m, gamma_m)] per unit
    coupling g, rates in 1/ps): the bias moves each exponent by -sigma i mu_alpha / hbar."""
    out = []
    for (alpha, mu), g in sorted(couplings.items()):
        ma = mus[alpha]
        for sigma in (1, -1):
            for k, (eta, gam) in enumerate(terms):
                out.append(Drawer(sigma, alpha, mu, k, gam - sigma * 1j * ma / HBAR, g * eta))
    return out


def discrete_bath(modes):
    """Drawers of discrete bath modes: modes = [(mu, t_k, eps_k, occupation f_k)].  Then
    C^+(t) = sum |t|^2 f e^{i eps t}, C^-(t) = sum |t|^2 (1 - f) e^{-i eps t}: one drawer per
    (sigma, mode), exact."""
    out = []
    for k, (mu, t, eps, f) in enumerate(modes):
        out.append(Drawer(1, k, mu, 0, -1j * eps, abs(t) ** 2 * f))
        out.append(Drawer(-1, k, mu, 0, 1j * eps, abs(t) ** 2 * (1 - f)))
    return out


# ----------------------------------------------------------------------------- hierarchy
class Hierarchy:
    """The generator of the hierarchy truncated at tier ntier, on stacked column-major ADOs."""

    def __init__(self, H, a_ops, drawers, ntier):
        self.nd = H.shape[0]
        self.H = H
        self.a = a_ops
        self.dr = drawers
        K = len(drawers)
        key_index = {d.key(): i for i, d in enumerate(drawers)}
        self.bar = [key_index[(-d.sigma, d.alpha, d.mu, d.m)] for d in drawers]
        self.ados = [()]
        for n in range(1, ntier + 1):
            self.ados += list(itertools.combinations(range(K), n))
        self.index = {J: i for i, J in enumerate(self.ados)}
        self.L = self._assemble()

    def op(self, sigma, mu):
        return self.a[mu].T.conj() if sigma == 1 else self.a[mu]

    def _assemble(self):
        nd = self.nd
        nn = nd * nd
        I = sp.identity(nd, format="csr")

        def left(A):
            return sp.kron(I, sp.csr_matrix(A)).tocoo()

        def right(B):
            return sp.kron(sp.csr_matrix(B).T, I).tocoo()

        liou = (-1j * (left(self.H) - right(self.H))).tocoo()
        # per drawer and parity of the ADO acted on: A_jbar (from above) and C_j (from below)
        up, down = {}, {}
        for j, d in enumerate(self.dr):
            ab = self.op(-d.sigma, d.mu)
            a = self.op(d.sigma, d.mu)
            eb = np.conj(self.dr[self.bar[j]].eta)
            for par in (1, -1):
                up[j, par] = (left(ab) + par * right(ab)).tocoo()
                down[j, par] = (d.eta * left(a) - par * eb * right(a)).tocoo()
        rows, cols, vals = [], [], []

        def put(r, c, M, scale):
            rows.append(M.row + r * nn)
            cols.append(M.col + c * nn)
            vals.append(scale * M.data)

        maxn = len(self.ados[-1])
        for J in self.ados:
            r = self.index[J]
            n = len(J)
            put(r, r, liou, 1.0)
            g = sum(self.dr[j].gamma for j in J)
            if g != 0:
                put(r, r, sp.identity(nn, format="coo"), -g)
            # higher tier: rho_{J + j} (sign of re-sorting j from the end to its place)
            if n < maxn:
                for j in range(len(self.dr)):
                    if j in J:
                        continue
                    sgn = (-1) ** sum(1 for x in J if x > j)
                    put(r, self.index[tuple(sorted(J + (j,)))], up[j, (-1) ** (n + 1)], -1j * sgn)
            # lower tier: rho_{J - j_r}
            for pos, j in enumerate(J):
                put(r, self.index[J[:pos] + J[pos + 1:]], down[j, (-1) ** (n - 1)], -1j * (-1) ** (n - (pos + 1)))
        N = len(self.ados) * nn
        return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))

    # --- states
    def size(self):
        return len(self.ados) * self.nd * self.nd

    def rdo(self, x):
        return x[: self.nd * self.nd].reshape(self.nd, self.nd, order="F")

    def ado(self, x, J):
        i = self.index[J] * self.nd * self.nd
        return x[i: i + self.nd * self.nd].reshape(self.nd, self.nd, order="F")

    def vector(self, rho0):
        x = np.zeros(self.size(), dtype=complex)
        x[: self.nd * self.nd] = np.asarray(rho0, dtype=complex).reshape(-1, order="F")
        return x

    def evolve(self, rho0, times):
        """The hierarchy's state at the given times from rho0 with all ADOs zero."""
        x = self.vector(rho0)
        return [spla.expm_multiply(self.L * t, x) if t > 0 else x.copy() for t in times]

    def steady(self):
        """Null vector of the generator with Tr rho = 1: the first row of L (whose RDO rows sum
        to zero under the trace) is replaced by the trace functional."""
        nd = self.nd
        A = self.L.tolil(copy=True)
        tr = np.zeros(self.size(), dtype=complex)
        tr[[i * nd + i for i in range(nd)]] = 1.0
        A[0, :] = tr
        b = np.zeros(self.size(), dtype=complex)
        b[0] = 1.0
        return spla.spsolve(A.tocsc(), b)

    def lead_rate(self, x, alpha, N):
        """d<N>/dt of the system from lead alpha: tr(N (-i sum_{j in alpha} A_jbar rho_j))."""
        acc = 0.0
        for j, d in enumerate(self.dr):
            if d.alpha != alpha:
                continue
            a = self.op(-d.sigma, d.mu)
            X = self.ado(x, (j,))
            acc += np.trace(N @ (-1j * (a @ X - X @ a)))
        return acc.real
