"""ctypes binding of the C oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py.  The GB300 product path never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "liboracle.so")
MAXALF, MAXORB = 2, 3


class Params(C.Structure):
    _fields_ = [
        ("norbs", C.c_int), ("nspin", C.c_int), ("nalf", C.c_int), ("nmats", C.c_int), ("ntier", C.c_int),
        ("bandwidth", C.c_double * MAXALF), ("linewidth", (C.c_double * MAXORB) * MAXALF),
        ("temperature", C.c_double * MAXALF), ("engyshift", (C.c_double * 2) * MAXALF),
        ("lscreen", C.c_int), ("doubledot", C.c_int), ("model", C.c_int),
        ("eup", C.c_double), ("edown", C.c_double), ("uu", C.c_double),
        ("e1up", C.c_double), ("e1down", C.c_double), ("e2up", C.c_double), ("e2down", C.c_double),
        ("uu1", C.c_double), ("uu2", C.c_double), ("u12", C.c_double), ("t12", C.c_double),
        ("kan_u", C.c_double), ("kan_j", C.c_double), ("kan_eps", C.c_double),
        ("hs_in", C.c_void_p), ("tchar", (C.c_double * 2) * MAXALF), ("pattern_seed", C.c_ulonglong),
        ("npsf", C.c_int), ("tpsf", C.c_double), ("rpsf", C.c_double), ("psf_coef", C.c_void_p), ("psf_pole", C.c_void_p),
    ]


class SolveInfo(C.Structure):
    _fields_ = [("iters", C.c_int), ("axb", C.c_int), ("ierr", C.c_int), ("exit_reason", C.c_int), ("resid", C.c_double)]


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        L = C.CDLL(_LIB)
        L.orc_build.argtypes = [C.POINTER(Params), C.POINTER(C.c_void_p)]
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_last_error.restype = C.c_char_p
        L.orc_info.restype = C.c_int64
        L.orc_info.argtypes = [C.c_void_p, C.c_char_p]
        L.orc_copy.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p]
        for f in ("orc_calc_ax",):
            getattr(L, f).argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_calcderiv.argtypes = [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_apply_shift.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        L.orc_current.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_occupation.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_initial_guess.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_solve_tfqmr.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_void_p, C.POINTER(SolveInfo), C.c_int]
        L.orc_rk4_step.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_void_p, C.c_int]
        L.orc_cheby_delta.restype = C.c_double
        L.orc_cheby_delta.argtypes = [C.c_void_p]
        L.orc_cheby_nterms.argtypes = [C.c_double, C.c_double, C.c_double]
        L.orc_cheby_step.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_double, C.c_void_p, C.c_int]
        L.orc_drandn.argtypes = [C.c_int64, C.c_void_p, C.c_int]
        L.orc_besselj_ext.restype = C.c_double
        L.orc_besselj_ext.argtypes = [C.c_int, C.c_double]
        L.orc_cf_build.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_ulonglong, C.POINTER(C.c_void_p)]
        L.orc_cf_free.argtypes = [C.c_void_p]
        L.orc_cf_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int] + [C.c_void_p] * 4 + [C.c_int]
        L.orc_cf_solve.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                   C.c_void_p, C.c_void_p, C.POINTER(SolveInfo), C.c_int]
        L.orc_cf_rhs.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.orc_jacobi_build.argtypes = [C.c_void_p, C.c_double, C.POINTER(C.c_void_p)]
        L.orc_jacobi_free.argtypes = [C.c_void_p]
        L.orc_jacobi_ejac.restype = C.c_double
        L.orc_jacobi_ejac.argtypes = [C.c_void_p]
        L.orc_jacobi_sweep.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_solve_jacobi.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_void_p, C.POINTER(SolveInfo)]
        L.orc_herm_eig.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_cf_info.restype = C.c_int64
        L.orc_cf_info.argtypes = [C.c_void_p, C.c_char_p]
        L.orc_cf_copy.argtypes = [C.c_void_p, C.c_int64, C.c_char_p, C.c_void_p]
        _lib = L
    return _lib


def make_params(cfg):
    """cfg: dict with the reference input-file quantities (see tests/configs.py)."""
    p = Params()
    p.norbs, p.nspin, p.nalf, p.nmats, p.ntier = cfg["norbs"], cfg["nspin"], cfg["nalf"], cfg["nmats"], cfg["ntier"]
    for a in range(cfg["nalf"]):
        p.bandwidth[a] = cfg["bandwidth"][a]
        p.temperature[a] = cfg["temperature"][a]
        for o in range(cfg["norbs"]):
            p.linewidth[a][o] = cfg["linewidth"][a][o]
        for s in range(cfg["nspin"]):
            p.engyshift[a][s] = cfg["engyshift"][a][s]
            p.tchar[a][s] = cfg.get("tchar", 0.0)
    p.lscreen = int(cfg.get("lscreen", 0))
    p.doubledot = int(cfg.get("doubledot", 0))
    p.model = cfg["model"]
    for k in ("eup", "edown", "uu", "e1up", "e1down", "e2up", "e2down", "uu1", "uu2", "u12", "t12", "kan_u", "kan_j", "kan_eps"):
        setattr(p, k, float(cfg.get(k, 0.0)))
    p.pattern_seed = int(cfg.get("pattern_seed", 20261203))
    psf = cfg.get("psf")
    if psf:
        # Prony scheme: the fitted table (coefficients, poles) the caller supplies
        p._psf = (np.ascontiguousarray(psf["coef"], dtype=np.complex128), np.ascontiguousarray(psf["pole"], dtype=np.complex128))
        p.npsf = len(p._psf[0])
        p.tpsf, p.rpsf = float(psf["tpsf"]), float(psf["rpsf"])
        p.psf_coef, p.psf_pole = p._psf[0].ctypes.data, p._psf[1].ctypes.data
    return p


class Model:
    def __init__(self, cfg, hs=None):
        self.cfg = cfg
        p = make_params(cfg)
        self._hs = None
        if hs is not None:
            self._hs = np.ascontiguousarray(np.asarray(hs, dtype=np.complex128).reshape(-1, order="F"))
            p.hs_in = self._hs.ctypes.data
        self._params = p
        h = C.c_void_p()
        if lib().orc_build(C.byref(p), C.byref(h)) != 0:
            raise RuntimeError("oracle build failed: " + lib().orc_last_error().decode())
        self.h = h
        for k in ("norbs", "nspin", "nalf", "nmats", "ntier", "ncor", "nopr", "nvar", "nrho", "nams", "nunk", "ntable", "lall", "lunk", "lscreen"):
            setattr(self, k, int(lib().orc_info(h, k.encode())))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_free(self.h)
            self.h = None

    _dtypes = {
        "cb": np.complex128, "cd": np.complex128, "cgama": np.complex128, "cgamma": np.complex128, "dipm": np.float64,
        "hs": np.complex128, "amsori": np.float64, "cpcoef": np.float64, "cppole": np.complex128,
        "ifirst": np.int64, "ilast": np.int64, "nfirst": np.int64, "nlast": np.int64, "index_coef_ref": np.int64,
        "indexcoef": np.int64, "itypecoef": np.int8, "ifactfcoef": np.int8, "ifactrcoef": np.int8,
        "ind_spa": np.int64, "eleadinfty": np.float64, "zxip": np.float64,
    }

    def get(self, name):
        n = {
            "cb": self.norbs * self.nspin * self.ncor * self.nalf * 2, "cd": None, "cgama": None,
            "cgamma": self.nvar, "dipm": self.nvar, "mpm": self.nvar, "morbs": self.nvar, "mspin": self.nvar,
            "ilead": self.nvar, "mcor": self.nvar, "mopr": self.nvar, "iredex": self.nvar, "indexdraw": self.nvar,
            "jredex": self.nopr, "jomit": self.nopr, "amsori": self.nrho ** 2 * self.norbs * self.nspin,
            "rowams": self.nams * self.norbs * self.nspin, "colams": None, "sgnams": None, "hs": self.nrho ** 2,
            "cpcoef": self.nmats, "cppole": self.nmats * 2, "ifirst": self.ntier, "ilast": self.ntier,
            "nfirst": self.ntier, "nlast": self.ntier, "indextable": self.ntable, "index_coef_ref": self.nunk,
            "indexcoef": self.lall, "itypecoef": self.lall, "ifactfcoef": self.lall, "ifactrcoef": self.lall,
            "nnz_spa": self.nunk, "ind_spa": self.nunk, "irow_spa": self.lunk, "icol_spa": self.lunk,
            "eleadinfty": MAXALF * 2, "zxip": MAXALF * MAXORB,
        }
        alias = {"cd": "cb", "cgama": "cb", "colams": "rowams", "sgnams": "rowams"}
        cnt = n[name] if n.get(name) is not None else n[alias[name]]
        a = np.zeros(cnt, dtype=self._dtypes.get(name, np.int32))
        if lib().orc_copy(self.h, name.encode(), a.ctypes.data) != 0:
            raise KeyError(name)
        return a

    def dense_op(self, iorbs, ispin):
        """a_{iorbs,ispin} as a dense nrho x nrho matrix."""
        nr, na = self.nrho, self.nams
        k = na * ((iorbs - 1) + (ispin - 1) * self.norbs)
        r, c, sg = (self.get(x)[k:k + na] for x in ("rowams", "colams", "sgnams"))
        a = np.zeros((nr, nr))
        a[r - 1, c - 1] = np.where(sg != 0, -1.0, 1.0)
        return a

    # ---- applies ----
    def calc_ax(self, x, nthreads=0):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        assert x.size == self.lunk + 1
        y = np.zeros(self.lunk + 1, dtype=np.complex128)
        lib().orc_calc_ax(self.h, x.ctypes.data, y.ctypes.data, nthreads)
        return y

    def calcderiv(self, t, x, nthreads=0):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.zeros(self.lunk, dtype=np.complex128)
        lib().orc_calcderiv(self.h, t, x.ctypes.data, y.ctypes.data, nthreads)
        return y

    def apply_shift(self, eshift, x, with_trace, nthreads=0):
        es = np.zeros((MAXALF, 2))
        es[: np.asarray(eshift).shape[0], : np.asarray(eshift).shape[1]] = eshift
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.zeros(self.lunk + 1, dtype=np.complex128)
        lib().orc_apply_shift(self.h, es.ctypes.data, x.ctypes.data, y.ctypes.data, int(with_trace), nthreads)
        return y if with_trace else y[: self.lunk]

    def current(self, rho):
        rho = np.ascontiguousarray(rho, dtype=np.complex128)
        jt = np.zeros(self.nalf * self.nspin)
        lib().orc_current(self.h, rho.ctypes.data, jt.ctypes.data)
        return jt.reshape(self.nspin, self.nalf).T  # jt[ialf, ispin]

    def occupation(self, rho):
        rho = np.ascontiguousarray(rho, dtype=np.complex128)
        occ = np.zeros(self.norbs * self.nspin)
        lib().orc_occupation(self.h, rho.ctypes.data, occ.ctypes.data)
        return occ.reshape(self.nspin, self.norbs).T

    def initial_guess(self):
        r = np.zeros(self.lunk, dtype=np.complex128)
        lib().orc_initial_guess(self.h, r.ctypes.data)
        return r

    def solve_tfqmr(self, crit=1e-10, maxit0=20000, rho=None, nthreads=0):
        if rho is None:
            rho = self.initial_guess()
        rho = np.ascontiguousarray(rho, dtype=np.complex128).copy()
        info = SolveInfo()
        lib().orc_solve_tfqmr(self.h, crit, maxit0, rho.ctypes.data, C.byref(info), nthreads)
        return rho, info

    def rk4_step(self, t, dt, rho, nthreads=0):
        rho = np.ascontiguousarray(rho, dtype=np.complex128).copy()
        lib().orc_rk4_step(self.h, t, dt, rho.ctypes.data, nthreads)
        return rho

    def cheby_delta(self):
        return lib().orc_cheby_delta(self.h)

    def cheby_step(self, t, delta, nterms, dt, rho, nthreads=0):
        rho = np.ascontiguousarray(rho, dtype=np.complex128).copy()
        lib().orc_cheby_step(self.h, t, delta, nterms, dt, rho.ctypes.data, nthreads)
        return rho


def drandn(n, seed=1):
    a = np.zeros(n)
    lib().orc_drandn(n, a.ctypes.data, seed)
    return a


def besselj(n, x):
    return lib().orc_besselj_ext(n, x)


def cheby_nterms(delta, dt, dpre=1e-21):
    return lib().orc_cheby_nterms(delta, dt, dpre)


HBAR = 0.658211928


class CF:
    """Correlation-function system of B = a_{iorbs,ispin} on an oracle model
    (corrfunc/prelude_cf_spa.f90, calc_ax_cf_spa_omp.f90, solve_cf_tfqmr_spa.f90).

    The unknown has two components (h, a), each lunkcf complex entries.  The operator is
    real-linear only (its RDO row adds conjugate transposes), so solves work on the real
    vector [Re h, Im h, Re a, Im a]."""

    def __init__(self, model, iorbs=1, ispin=1, seed=20261203):
        self.model = model
        h = C.c_void_p()
        if lib().orc_cf_build(model.h, iorbs, ispin, seed, C.byref(h)) != 0:
            raise RuntimeError("oracle cf build failed: " + lib().orc_last_error().decode())
        self.h = h
        self.iorbs, self.ispin = iorbs, ispin
        self.lunkcf = int(lib().orc_cf_info(h, b"lunkcf"))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_cf_free(self.h)
            self.h = None

    def get(self, name):
        n = {"nnzcf_spa": self.model.nunk, "indcf_spa": self.model.nunk,
             "irowcf_spa": self.lunkcf, "icolcf_spa": self.lunkcf}[name]
        a = np.zeros(n, dtype=np.int64 if name == "indcf_spa" else np.int32)
        if lib().orc_cf_copy(self.h, self.model.nunk, name.encode(), a.ctypes.data) != 0:
            raise KeyError(name)
        return a

    def apply(self, omega, isgnw, xh, xa, nthreads=0):
        """(yh, ya) = L_cf (xh, xa); omega in internal units (energy / hbar)."""
        xh = np.ascontiguousarray(xh, dtype=np.complex128)
        xa = np.ascontiguousarray(xa, dtype=np.complex128)
        yh = np.zeros(self.lunkcf, dtype=np.complex128)
        ya = np.zeros(self.lunkcf, dtype=np.complex128)
        lib().orc_cf_apply(self.model.h, self.h, omega, isgnw, xh.ctypes.data, xa.ctypes.data,
                           yh.ctypes.data, ya.ctypes.data, nthreads)
        return yh, ya

    def tfqmr(self, rho, omega, isgnb, isgnw, crit=1e-10, maxit0=20000, nthreads=0):
        """The reference algorithm (solve_cf_tfqmr_spa): TFQMR from x = 0 in C."""
        rho = np.ascontiguousarray(rho, dtype=np.complex128)
        xh = np.zeros(self.lunkcf, dtype=np.complex128)
        xa = np.zeros(self.lunkcf, dtype=np.complex128)
        info = SolveInfo()
        lib().orc_cf_solve(self.model.h, self.h, rho.ctypes.data, isgnb, isgnw, omega, crit, maxit0, xh.ctypes.data,
                           xa.ctypes.data, C.byref(info), nthreads)
        return xh, xa, info

    def rhs(self, rho, isgnb):
        rho = np.ascontiguousarray(rho, dtype=np.complex128)
        bh = np.zeros(self.lunkcf, dtype=np.complex128)
        ba = np.zeros(self.lunkcf, dtype=np.complex128)
        lib().orc_cf_rhs(self.model.h, self.h, rho.ctypes.data, isgnb, bh.ctypes.data, ba.ctypes.data)
        return bh, ba

    def _split(self, z):
        n = self.lunkcf
        return z[:n] + 1j * z[n:2 * n], z[2 * n:3 * n] + 1j * z[3 * n:]

    def solve(self, rho, omega, isgnb, isgnw, tol=1e-12):
        """Solve L_cf x = -(brhoh, brhoa) (solve_cf_tfqmr_spa.f90:185-197) with restarted GMRES."""
        from scipy.sparse.linalg import LinearOperator, gmres
        n = self.lunkcf

        def mv(z):
            # one thread: OpenMP workers spinning between calls would compete with the BLAS
            # threads of GMRES's orthogonalisation
            yh, ya = self.apply(omega, isgnw, *self._split(np.asarray(z).ravel()), nthreads=1)
            return np.concatenate([yh.real, yh.imag, ya.real, ya.imag])

        bh, ba = self.rhs(rho, isgnb)
        b = -np.concatenate([bh.real, bh.imag, ba.real, ba.imag])
        op = LinearOperator((4 * n, 4 * n), matvec=mv, dtype=np.float64)
        z, info = gmres(op, b, rtol=tol, atol=0.0, restart=200, maxiter=200)
        resid = np.linalg.norm(mv(z) - b) / max(np.linalg.norm(b), 1e-300)
        xh, xa = self._split(z)
        return xh, xa, resid

    def rdo(self, x):
        """Dense nrho x nrho matrix of the first (RDO) block of a cf component."""
        nr = self.model.nrho
        nz = int(self.get("nnzcf_spa")[0])
        ir, ic = self.get("irowcf_spa")[:nz], self.get("icolcf_spa")[:nz]
        out = np.zeros((nr, nr), dtype=np.complex128)
        out[ir - 1, ic - 1] = x[:nz]
        return out

    def dos(self, rho, omega_ev, tol=1e-12):
        """Spectral function A(omega) of a_{iorbs,ispin} in 1/eV (corrfunc/corrfunc.f90:146-192):
        (total, part from C_{B^dag B}, part from C_{B B^dag})."""
        a = self.model.dense_op(self.iorbs, self.ispin)
        w = omega_ev / HBAR
        xh, xa, _ = self.solve(rho, w, 2, 2, tol)
        c5 = 0.5 * self.rdo(xh) + 0.5j * self.rdo(xa)
        d1 = np.trace(a.conj().T @ c5).real / np.pi / HBAR
        xh, xa, _ = self.solve(rho, w, 1, 1, tol)
        c5 = 0.5 * self.rdo(xh) + 0.5j * self.rdo(xa)
        d2 = np.trace(a @ c5).real / np.pi / HBAR
        return d1 + d2, d1, d2


class Jacobi:
    """The Jacobi steady-state iteration of the reference (jacobi/) on an oracle model.
    ejac: the shift in energy / hbar; <= 0 selects prelude_jacobi's rule."""

    def __init__(self, model, ejac=0.0):
        self.model = model
        h = C.c_void_p()
        lib().orc_jacobi_build(model.h, ejac, C.byref(h))
        self.h = h
        self.ejac = lib().orc_jacobi_ejac(h)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_jacobi_free(self.h)
            self.h = None

    def sweep(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        xn = np.zeros(self.model.lunk, dtype=np.complex128)
        lib().orc_jacobi_sweep(self.model.h, self.h, x.ctypes.data, xn.ctypes.data)
        return xn

    def solve(self, rho, crit=1e-10, maxit0=20000):
        rho = np.ascontiguousarray(rho, dtype=np.complex128).copy()
        info = SolveInfo()
        lib().orc_solve_jacobi(self.model.h, self.h, crit, maxit0, rho.ctypes.data, C.byref(info))
        return rho, info


def herm_eig(a):
    a = np.array(a, dtype=np.complex128, order="F", copy=True)
    n = a.shape[0]
    w = np.zeros(n)
    v = np.zeros((n, n), dtype=np.complex128, order="F")
    lib().orc_herm_eig(n, a.ctypes.data, w.ctypes.data, v.ctypes.data)
    return w, v
