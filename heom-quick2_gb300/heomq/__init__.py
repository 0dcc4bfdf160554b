"""heomq -- Python host interface of the GB300 HEOM library (ctypes over the C ABI).

Mirrors the reference's sparse-path routines:
  Context.calc_ax_tfqmr_spa(x)   <- calc_ax_tfqmr_spa_omp(ldim, rcgtmp, rcgrhs)
  Context.calcderiv_spa(t, x)    <- calcderiv_spa_omp(tt)
  Context.calc_atrx(x)           <- calc_atrx_bicg_omp (adjoint, here on the sparse layout)
  Context.solve_tfqmr(rho, ...)  <- solve_tfqmr
  Context.current / occupation   <- calcj / calcocc
  Context.propagate(...)         <- intstp (RK4) / chebyshev
and raises HeomError carrying the library's message where the reference would stop.
The compute path is the CUDA library; there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

from . import models  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libheom_gb300.so")

PREC_FP64, PREC_MIXED, PREC_MIXED_FP32, PREC_FP64_REFINED = 0, 1, 2, 3
# instances per call of heom_batch_current_static (the size of its static device scratch)
STATIC_CURRENT_MAX = 4096


def static_current_chunks(n, limit=STATIC_CURRENT_MAX):
    """(first instance, count) of the consecutive calls that cover n instances."""
    return [(b0, min(limit, n - b0)) for b0 in range(0, n, limit)]
PROP_RK4, PROP_CHEBYSHEV, PROP_CHEBYSHEV_MIXED = 0, 1, 2
ERRORS = {-1: "invalid argument", -2: "CUDA failure", -3: "out of memory", -4: "unsupported",
          -5: "TFQMR breakdown", -6: "not converged", -7: "device wait timed out"}


class HeomError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


_p = C.POINTER


class Tables(C.Structure):
    _fields_ = [
        ("norbs", C.c_int32), ("nspin", C.c_int32), ("nalf", C.c_int32), ("ncor", C.c_int32), ("ntier", C.c_int32),
        ("nrho", C.c_int32), ("nams", C.c_int32), ("lscreen", C.c_int32),
        ("nunk", C.c_int64), ("lall", C.c_int64), ("lunk_spa", C.c_int64),
        ("cgamma", C.c_void_p), ("dipm", C.c_void_p),
        ("mpm", C.c_void_p), ("morbs", C.c_void_p), ("mspin", C.c_void_p), ("ilead", C.c_void_p), ("mcor", C.c_void_p),
        ("indexdraw", C.c_void_p), ("cb", C.c_void_p), ("cd", C.c_void_p), ("eleadinfty", C.c_void_p),
        ("nfirst", C.c_void_p), ("nlast", C.c_void_p), ("ifirst", C.c_void_p), ("indextable", C.c_void_p),
        ("index_coef_ref", C.c_void_p), ("indexcoef", C.c_void_p), ("itypecoef", C.c_void_p),
        ("ifactfcoef", C.c_void_p), ("ifactrcoef", C.c_void_p),
        ("rowams", C.c_void_p), ("colams", C.c_void_p), ("sgnams", C.c_void_p), ("hs", C.c_void_p),
        ("nnz_spa", C.c_void_p), ("ind_spa", C.c_void_p), ("irow_spa", C.c_void_p), ("icol_spa", C.c_void_p),
    ]


class Params(C.Structure):
    _fields_ = [
        ("norbs", C.c_int32), ("nspin", C.c_int32), ("nalf", C.c_int32), ("nmats", C.c_int32), ("ntier", C.c_int32),
        ("bandwidth", C.c_double * 2), ("linewidth", (C.c_double * 3) * 2), ("temperature", C.c_double * 2),
        ("engyshift", (C.c_double * 2) * 2), ("lscreen", C.c_int32), ("doubledot", C.c_int32), ("model", C.c_int32),
        ("eup", C.c_double), ("edown", C.c_double), ("uu", C.c_double),
        ("e1up", C.c_double), ("e1down", C.c_double), ("e2up", C.c_double), ("e2down", C.c_double),
        ("uu1", C.c_double), ("uu2", C.c_double), ("u12", C.c_double), ("t12", C.c_double),
        ("kan_u", C.c_double), ("kan_j", C.c_double), ("kan_eps", C.c_double),
        ("hs_in", C.c_void_p), ("tchar", (C.c_double * 2) * 2),
        ("npsf", C.c_int32), ("tpsf", C.c_double), ("rpsf", C.c_double), ("psf_coef", C.c_void_p),
        ("psf_pole", C.c_void_p),
    ]


class CtxOpts(C.Structure):
    _fields_ = [("device", C.c_int32), ("build_adjoint", C.c_int32), ("amps", C.c_void_p), ("tchar", C.c_void_p),
                ("dhs", C.c_void_p * 4)]


class SolveOpts(C.Structure):
    _fields_ = [("crit", C.c_double), ("maxit0", C.c_int32), ("precision", C.c_int32), ("inner_tol", C.c_double),
                ("max_refine", C.c_int32), ("stag_window", C.c_int32), ("inner_precond", C.c_int32),
                ("interleave", C.c_int32), ("lane_instances", C.c_int32)]


def layout_candidates(nbatch, truncated=False):
    """The (interleave, lane_instances) layouts of the FP32x2 inner kernels that the automatic
    choice of the mixed batch solves times, in its order (the library's rule, restated here
    for reports): one instance per group; interleave 2 with two instances per lane (not for
    truncated batches); the smallest power of two g >= nbatch (at most 32) with one and with
    two instances per lane."""
    g = 1
    while g < nbatch and g < 32:
        g *= 2
    c = [(1, 1)]
    if g == 1:
        return c
    if not truncated:
        c.append((2, 2))
    if g > 2 or truncated:
        c.append((g, 1))
    if g > 2 and not truncated:
        c.append((g, 2))
    return c


class SolveInfo(C.Structure):
    _fields_ = [("iters", C.c_int32), ("ierr", C.c_int32), ("refinements", C.c_int32), ("converged", C.c_int32),
                ("resid", C.c_double), ("seconds", C.c_double), ("launches", C.c_int64)]


class CfTables(C.Structure):
    _fields_ = [("iorbs", C.c_int32), ("ispin", C.c_int32), ("lunkcf_spa", C.c_int64), ("nnzcf_spa", C.c_void_p),
                ("indcf_spa", C.c_void_p), ("irowcf_spa", C.c_void_p), ("icolcf_spa", C.c_void_p)]


class GradOpts(C.Structure):
    _fields_ = [("deshift", C.c_void_p), ("gamma", C.c_double), ("dhs_du", C.c_void_p), ("dhs_deps", C.c_void_p),
                ("crit", C.c_double), ("maxit0", C.c_int32), ("precision", C.c_int32)]


# symbol -> (restype, argtypes); also the list of entry points of include/heom_gb300.h
SIGNATURES = {
    "heom_model_build": (C.c_int, [_p(Params), _p(C.c_void_p)]),
    "heom_model_destroy": (None, [C.c_void_p]),
    "heom_model_tables": (_p(Tables), [C.c_void_p]),
    "heom_model_initial_guess": (C.c_int, [C.c_void_p, C.c_void_p]),
    "heom_model_field": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "heom_model_get": (C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p]),
    "heom_ctx_create": (C.c_int, [_p(Tables), _p(CtxOpts), _p(C.c_void_p)]),
    "heom_ctx_destroy": (None, [C.c_void_p]),
    "heom_ctx_lunk": (C.c_int64, [C.c_void_p]),
    "heom_last_error": (C.c_char_p, []),
    "heom_calc_ax": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "heom_calcderiv": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]),
    "heom_calc_atrx": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "heom_calc_ax_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "heom_calc_atrx_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "heom_calc_ax_fp32_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "heom_calc_ax_fp32x2_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "heom_calc_ax_inner_dev": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "heom_solve_tfqmr": (C.c_int, [C.c_void_p, _p(SolveOpts), C.c_void_p, _p(SolveInfo)]),
    "heom_current": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "heom_occupation": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "heom_propagate": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_int32, C.c_void_p, C.c_void_p]),
    "heom_steady_gradient": (C.c_int, [C.c_void_p, _p(GradOpts), C.c_void_p, C.c_int32, C.c_void_p, _p(SolveInfo)]),
    "heom_td_gradient": (C.c_int, [C.c_void_p, C.c_double, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "heom_td_gradient_ex": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                      C.c_void_p]),
    "heom_solve_batch": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, _p(SolveOpts), C.c_void_p, _p(SolveInfo)]),
    "heom_bench_apply": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "heom_bench_inner": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "heom_bench_inner_layout": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                          C.c_void_p]),
    "heom_tuned_layout": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "heom_ctx_stats": (C.c_int, [C.c_void_p, C.c_void_p]),
    "heom_batch_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, _p(C.c_void_p)]),
    "heom_batch_stride": (C.c_int64, [C.c_void_p]),
    "heom_batch_solve_dev": (C.c_int, [C.c_void_p, _p(SolveOpts), C.c_void_p, _p(SolveInfo)]),
    "heom_batch_destroy": (None, [C.c_void_p]),
    "heom_batch_set_tiers": (C.c_int, [C.c_void_p, C.c_void_p]),
    "heom_batch_current_static": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int64, C.c_void_p]),
    "heom_solve_jacobi": (C.c_int, [C.c_void_p, _p(SolveOpts), C.c_double, C.c_void_p, _p(SolveInfo)]),
    "heom_jacobi_shift": (C.c_int, [C.c_void_p, C.c_void_p]),
    "heom_bench_jacobi": (C.c_int, [C.c_void_p, C.c_double, C.c_int32, C.c_void_p]),
    "heom_model_cf_pattern": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, _p(CfTables)]),
    "heom_cf_create": (C.c_int, [C.c_void_p, _p(Tables), _p(CfTables), _p(C.c_void_p)]),
    "heom_cf_destroy": (None, [C.c_void_p]),
    "heom_cf_lunk": (C.c_int64, [C.c_void_p]),
    "heom_cf_calc_ax": (C.c_int, [C.c_void_p, C.c_double, C.c_int32, C.c_int64] + [C.c_void_p] * 4),
    "heom_cf_solve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, _p(SolveOpts),
                                C.c_void_p, C.c_void_p, _p(SolveInfo)]),
    "heom_cf_bench_apply": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "heom_cf_bench_inner": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]),
    "heom_cf_propagate": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                    C.c_void_p]),
    "heom_cf_dos": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, _p(SolveOpts), C.c_void_p,
                              _p(SolveInfo)]),
}

_lib = None


def lib():
    """Load the in-tree CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise HeomError(-4, f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise HeomError(rc, lib().heom_last_error().decode())


def _c128(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} complex entries, got {a.size}")
    return a


def make_params(cfg):
    p = Params()
    p.norbs, p.nspin, p.nalf, p.nmats, p.ntier = cfg["norbs"], cfg["nspin"], cfg["nalf"], cfg["nmats"], cfg["ntier"]
    for a in range(cfg["nalf"]):
        p.bandwidth[a] = cfg["bandwidth"][a]
        p.temperature[a] = cfg["temperature"][a]
        for o in range(cfg["norbs"]):
            p.linewidth[a][o] = cfg["linewidth"][a][o]
        for s in range(cfg["nspin"]):
            p.engyshift[a][s] = cfg["engyshift"][a][s]
            tc = cfg.get("tchar", 0.0)
            p.tchar[a][s] = tc[a][s] if isinstance(tc, (list, tuple)) else tc
    p.lscreen = int(cfg.get("lscreen", 0))
    p.doubledot = int(cfg.get("doubledot", 0))
    p.model = cfg["model"]
    for k in ("eup", "edown", "uu", "e1up", "e1down", "e2up", "e2down", "uu1", "uu2", "u12", "t12", "kan_u", "kan_j", "kan_eps"):
        setattr(p, k, float(cfg.get(k, 0.0)))
    psf = cfg.get("psf")
    if psf:
        # Prony scheme (psfjob): the fitted table the caller supplies (coefficients, poles, the
        # fit's reference temperature tpsf and band ratio rpsf)
        p._psf = (_c128(psf["coef"]), _c128(psf["pole"]))
        p.npsf = len(p._psf[0])
        p.tpsf, p.rpsf = float(psf["tpsf"]), float(psf["rpsf"])
        p.psf_coef, p.psf_pole = p._psf[0].ctypes.data, p._psf[1].ctypes.data
    return p


def psf_table_from_pade(nmats, W, T, tpsf=1.0):
    """The Drude pole and the [nmats-1/nmats] Pade terms of a Lorentzian band of half-width W at
    temperature T written as a Prony table (coefficients, poles) for the same band: the
    exponentials of the Pade scheme in the form the Prony scheme takes them (one set of poles
    for both signs, cb = T / tpsf coef linewidth, cgama = T / tpsf pole).  A table in the
    reference's itype_psf form is used the same way."""
    m = Model(dict(norbs=1, nspin=2, nalf=1, nmats=nmats, ntier=2, bandwidth=[W, W], linewidth=[[1.0], [1.0]],
                   temperature=[T, T], engyshift=[[0.0, 0.0], [0.0, 0.0]], model=1))
    ncor = nmats + 1
    cb = m.array("cb").reshape(1, 2, ncor, 1, 2, order="F")          # cb(norbs, nspin, ncor, nalf, nsgn)
    cgamma = m.array("cgamma")[:ncor]                                 # sign +, spin 1: the ncor drawers
    s = T / tpsf
    return {"coef": cb[0, 0, :, 0, 0] / s, "pole": cgamma / s, "tpsf": tpsf, "rpsf": W / T}   # linewidth 1


class Model:
    """Host-side set-up of one job (evaluatepara, buildoperator, calchs, ball2drawer,
    buildcoefindex, prelude_spa): the tables the sparse path consumes."""

    def __init__(self, cfg, hs=None):
        self.cfg = dict(cfg)
        p = make_params(cfg)
        self._hs = None
        if hs is not None:
            self._hs = _c128(np.asarray(hs).reshape(-1, order="F"))
            p.hs_in = self._hs.ctypes.data
            p.model = 9
        h = C.c_void_p()
        _check(lib().heom_model_build(C.byref(p), C.byref(h)))
        self.h = h
        self.tables = lib().heom_model_tables(h).contents
        t = self.tables
        self.nrho, self.lunk, self.nunk, self.lall = t.nrho, t.lunk_spa, t.nunk, t.lall
        self.norbs, self.nspin, self.nalf, self.ncor, self.ntier = t.norbs, t.nspin, t.nalf, t.ncor, t.ntier

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.heom_model_destroy(self.h)
            self.h = None

    def array(self, name):
        """numpy copy of one table of the heom_tables view."""
        t = self.tables
        nvar = 2 * t.norbs * t.nspin * t.nalf * t.ncor
        ncb = t.norbs * t.nspin * t.ncor * t.nalf * 2
        spec = {
            "cgamma": (nvar, np.complex128), "dipm": (nvar, np.float64), "mpm": (nvar, np.int32), "morbs": (nvar, np.int32),
            "mspin": (nvar, np.int32), "ilead": (nvar, np.int32), "mcor": (nvar, np.int32), "indexdraw": (nvar, np.int32),
            "cb": (ncb, np.complex128), "cd": (ncb, np.complex128), "eleadinfty": (t.nalf * t.nspin, np.float64),
            "nfirst": (t.ntier, np.int64), "nlast": (t.ntier, np.int64), "ifirst": (t.ntier, np.int64),
            "index_coef_ref": (t.nunk, np.int64), "indexcoef": (t.lall, np.int64), "itypecoef": (t.lall, np.int8),
            "ifactfcoef": (t.lall, np.int8), "ifactrcoef": (t.lall, np.int8),
            "rowams": (t.nams * t.norbs * t.nspin, np.int32), "colams": (t.nams * t.norbs * t.nspin, np.int32),
            "sgnams": (t.nams * t.norbs * t.nspin, np.int32), "hs": (t.nrho ** 2, np.complex128),
            "nnz_spa": (t.nunk, np.int32), "ind_spa": (t.nunk, np.int64), "irow_spa": (t.lunk_spa, np.int32),
            "icol_spa": (t.lunk_spa, np.int32),
        }
        if name == "indextable":
            nlast = self.array("nlast")
            nfirst = self.array("nfirst")
            n = 1 + sum(int(nlast[k] - nfirst[k] + 1) * k for k in range(1, t.ntier))
            spec[name] = (n, np.int32)
        cnt, dt = spec[name]
        ptr = getattr(t, name)
        buf = (C.c_char * (cnt * np.dtype(dt).itemsize)).from_address(ptr)
        return np.frombuffer(bytes(buf), dtype=dt).copy()

    def get(self, name, count, dtype):
        out = np.zeros(count, dtype=dtype)
        _check(lib().heom_model_get(self.h, name.encode(), out.ctypes.data))
        return out

    def initial_guess(self):
        r = np.zeros(self.lunk, dtype=np.complex128)
        _check(lib().heom_model_initial_guess(self.h, r.ctypes.data))
        return r

    def cf_pattern(self, iorbs=1, ispin=1):
        """Correlation-function pattern of a_{iorbs,ispin} (prelude_cf_spa) as numpy arrays."""
        t = CfTables()
        _check(lib().heom_model_cf_pattern(self.h, iorbs, ispin, C.byref(t)))

        def arr(ptr, cnt, dt):
            buf = (C.c_char * (cnt * np.dtype(dt).itemsize)).from_address(ptr)
            return np.frombuffer(bytes(buf), dtype=dt).copy()

        L = t.lunkcf_spa
        return {"iorbs": iorbs, "ispin": ispin, "lunkcf_spa": L,
                "nnzcf_spa": arr(t.nnzcf_spa, self.nunk, np.int32), "indcf_spa": arr(t.indcf_spa, self.nunk, np.int64),
                "irowcf_spa": arr(t.irowcf_spa, L, np.int32), "icolcf_spa": arr(t.icolcf_spa, L, np.int32)}

    def field(self):
        a = np.zeros(self.nalf * self.nspin)
        tc = np.zeros(self.nalf * self.nspin)
        _check(lib().heom_model_field(self.h, a.ctypes.data, tc.ctypes.data))
        return a, tc


class Context:
    """Device-resident plan of one model (opaque heom_ctx)."""

    def __init__(self, model, device=0, adjoint=True, amps=None, tchar=None, dhs=()):
        self.model = model
        o = CtxOpts()
        o.device = device
        o.build_adjoint = int(adjoint)
        self._keep = []
        if amps is None and tchar is None:   # the model's own pulse (getengyshift, fieldtype 0)
            amps, tchar = model.field()
        if amps is not None:
            a = np.ascontiguousarray(amps, dtype=np.float64)
            self._keep.append(a)
            o.amps = a.ctypes.data
        if tchar is not None:
            tc = np.ascontiguousarray(tchar, dtype=np.float64)
            self._keep.append(tc)
            o.tchar = tc.ctypes.data
        for k, d in enumerate(dhs):
            if d is not None:
                dd = _c128(d)
                self._keep.append(dd)
                o.dhs[k] = dd.ctypes.data
        h = C.c_void_p()
        _check(lib().heom_ctx_create(C.byref(model.tables), C.byref(o), C.byref(h)))
        self.h = h
        self.lunk = model.lunk
        self.device = device

    def close(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.heom_ctx_destroy(self.h)
            self.h = None

    __del__ = close

    # -- reference-named entry points --
    def calc_ax_tfqmr_spa(self, x):
        x = _c128(x, self.lunk + 1)
        y = np.zeros(self.lunk + 1, dtype=np.complex128)
        _check(lib().heom_calc_ax(self.h, self.lunk, x.ctypes.data, y.ctypes.data))
        return y

    def calcderiv_spa(self, t, x):
        x = _c128(x, self.lunk)
        y = np.zeros(self.lunk, dtype=np.complex128)
        _check(lib().heom_calcderiv(self.h, float(t), x.ctypes.data, y.ctypes.data))
        return y

    def _device_apply(self, fn, x, precision):
        """Run a device-vector apply fn(dx, dy) on x (lunk + 1 complex values) in the number
        type of `precision`: FP32x2 splits x into FP32 high and low parts (float4 per value)."""
        import torch

        x = _c128(x, self.lunk + 1)
        if precision == PREC_MIXED:
            parts = []
            for comp in (x.real, x.imag):
                hi = comp.astype(np.float32)
                parts.append((hi, (comp - hi.astype(np.float64)).astype(np.float32)))
            v = np.stack([parts[0][0], parts[1][0], parts[0][1], parts[1][1]], axis=1)
        elif precision == PREC_MIXED_FP32:
            v = np.stack([x.real, x.imag], axis=1).astype(np.float32)
        else:
            v = np.stack([x.real, x.imag], axis=1)
        with torch.cuda.device(self.device):
            xd = torch.from_numpy(np.ascontiguousarray(v)).to(f"cuda:{self.device}")
            yd = torch.zeros_like(xd)
            torch.cuda.synchronize(self.device)
            _check(fn(C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr())))
            y = yd.cpu().numpy().astype(np.float64)
        if precision == PREC_MIXED:
            return (y[:, 0] + y[:, 2]) + 1j * (y[:, 1] + y[:, 3])
        return y[:, 0] + 1j * y[:, 1]

    def calc_ax_fp32x2(self, x):
        """y = A x in the FP32x2 arithmetic of the mixed-precision inner solves (the unregularised
        operator): x is split into FP32 high and low parts, y returned as hi + lo in FP64."""
        return self._device_apply(lambda dx, dy: lib().heom_calc_ax_fp32x2_dev(self.h, dx, dy), x, PREC_MIXED)

    def calc_ax_inner(self, x, precision=PREC_MIXED, precond=True):
        """The operator of the mixed-precision inner solves (regularised, rows scaled by the inner
        preconditioner when precond) in the arithmetic of `precision`, on a host vector."""
        return self._device_apply(lambda dx, dy: lib().heom_calc_ax_inner_dev(self.h, precision, int(precond), dx, dy),
                                  x, precision)

    def calc_atrx(self, x):
        x = _c128(x, self.lunk + 1)
        y = np.zeros(self.lunk + 1, dtype=np.complex128)
        _check(lib().heom_calc_atrx(self.h, self.lunk, x.ctypes.data, y.ctypes.data))
        return y

    def solve_tfqmr(self, rho=None, crit=1e-10, maxit0=20000, precision=PREC_FP64, inner_tol=0.0, max_refine=8,
                    check=True, inner_precond=0):
        if rho is None:
            rho = self.model.initial_guess()
        rho = _c128(rho, self.lunk).copy()
        o = SolveOpts(crit=crit, maxit0=maxit0, precision=precision, inner_tol=inner_tol, max_refine=max_refine,
                      inner_precond=inner_precond)
        info = SolveInfo()
        rc = lib().heom_solve_tfqmr(self.h, C.byref(o), rho.ctypes.data, C.byref(info))
        if check:
            _check(rc)
        return rho, info

    def solve_jacobi(self, rho=None, crit=1e-10, maxit0=20000, ejac=0.0, check=True):
        """Steady state by the reference's Jacobi sweeps (methodss = 4); ejac in energy / hbar,
        <= 0 for prelude_jacobi's rule."""
        if rho is None:
            rho = self.model.initial_guess()
        rho = _c128(rho, self.lunk).copy()
        o = SolveOpts(crit=crit, maxit0=maxit0, precision=PREC_FP64)
        info = SolveInfo()
        rc = lib().heom_solve_jacobi(self.h, C.byref(o), float(ejac), rho.ctypes.data, C.byref(info))
        if check:
            _check(rc)
        return rho, info

    def bench_jacobi(self, ejac=0.0, reps=10):
        """(transform s, apply s, transform bytes, transform complex multiply-adds) per launch."""
        out = np.zeros(4)
        _check(lib().heom_bench_jacobi(self.h, float(ejac), reps, out.ctypes.data))
        return tuple(out.tolist())

    def jacobi_shift(self):
        e = C.c_double()
        _check(lib().heom_jacobi_shift(self.h, C.byref(e)))
        return e.value

    def solve_batch(self, rhos, hs_batch=None, eshift_batch=None, crit=1e-10, maxit0=20000, precision=PREC_FP64,
                    inner_tol=0.0, max_refine=8, inplace=False):
        """Steady states of a batch; rhos (nbatch, lunk) holds the initial guesses.  With
        inplace=True a C-contiguous complex128 rhos (e.g. a view of pinned memory) is solved
        in place."""
        if inplace:
            if rhos.dtype != np.complex128 or not rhos.flags.c_contiguous:
                raise ValueError("inplace needs a C-contiguous complex128 array")
        else:
            rhos = np.ascontiguousarray(rhos, dtype=np.complex128).copy()
        nb = rhos.shape[0]
        hs = None if hs_batch is None else _c128(hs_batch)
        es = None if eshift_batch is None else np.ascontiguousarray(eshift_batch, dtype=np.float64)
        o = SolveOpts(crit=crit, maxit0=maxit0, precision=precision, inner_tol=inner_tol, max_refine=max_refine)
        info = SolveInfo()
        _check(lib().heom_solve_batch(self.h, nb, None if hs is None else hs.ctypes.data,
                                      None if es is None else es.ctypes.data, C.byref(o), rhos.ctypes.data, C.byref(info)))
        return rhos, info

    def current(self, rho):
        rho = _c128(rho, self.lunk)
        jt = np.zeros(self.model.nalf * self.model.nspin)
        _check(lib().heom_current(self.h, rho.ctypes.data, jt.ctypes.data))
        return jt.reshape(self.model.nspin, self.model.nalf).T   # jt[ialf, ispin]

    def occupation(self, rho):
        rho = _c128(rho, self.lunk)
        occ = np.zeros(self.model.norbs * self.model.nspin)
        _check(lib().heom_occupation(self.h, rho.ctypes.data, occ.ctypes.data))
        return occ.reshape(self.model.nspin, self.model.norbs).T

    def propagate(self, rho, t0, dt, nstep, method=PROP_RK4, currents=False):
        rho = _c128(rho, self.lunk).copy()
        jt = np.zeros((nstep, self.model.nalf * self.model.nspin)) if currents else None
        _check(lib().heom_propagate(self.h, method, t0, dt, nstep, rho.ctypes.data, None if jt is None else jt.ctypes.data))
        return (rho, jt) if currents else rho

    def steady_gradient(self, rho, deshift=None, gamma=None, dhs_du=None, dhs_deps=None, which=0xF, crit=1e-10, maxit0=20000,
                        precision=PREC_FP64):
        rho = _c128(rho, self.lunk)
        o = GradOpts(crit=crit, maxit0=maxit0, gamma=gamma or 0.0, precision=precision)
        keep = []
        if deshift is not None:
            d = np.ascontiguousarray(deshift, dtype=np.float64); keep.append(d); o.deshift = d.ctypes.data
        if dhs_du is not None:
            d = _c128(dhs_du); keep.append(d); o.dhs_du = d.ctypes.data
        if dhs_deps is not None:
            d = _c128(dhs_deps); keep.append(d); o.dhs_deps = d.ctypes.data
        dI = np.zeros(4)
        info = SolveInfo()
        _check(lib().heom_steady_gradient(self.h, C.byref(o), rho.ctypes.data, which, dI.ctypes.data, C.byref(info)))
        return dI, info

    def td_gradient(self, rho0, dt, nstep, checkpoint_every=32, method=PROP_CHEBYSHEV):
        """(J, dJ/dA) of J = dt sum_n I_1(rho_n) through the Chebyshev steps of `method`
        (PROP_CHEBYSHEV or PROP_CHEBYSHEV_MIXED)."""
        rho0 = _c128(rho0, self.lunk)
        val = C.c_double()
        grad = C.c_double()
        _check(lib().heom_td_gradient_ex(self.h, method, dt, nstep, checkpoint_every, rho0.ctypes.data, C.byref(val),
                                         C.byref(grad)))
        return val.value, grad.value

    def bench_apply(self, precision=PREC_FP64, reps=20, nbatch=1):
        """Average device time of one apply launch over nbatch instances, and its algorithmic bytes."""
        s = C.c_double()
        b = C.c_double()
        _check(lib().heom_bench_apply(self.h, precision, nbatch, reps, C.byref(s), C.byref(b)))
        return s.value, b.value

    def bench_inner(self, precision=PREC_MIXED, reps=20, nbatch=1):
        """Average device times of the two fused kernels of an inner TFQMR iteration over nbatch
        instances, and their algorithmic bytes per launch: ((s_b, s_a), (bytes_b, bytes_a))."""
        s = (C.c_double * 2)()
        b = (C.c_double * 2)()
        _check(lib().heom_bench_inner(self.h, precision, nbatch, reps, s, b))
        return (s[0], s[1]), (b[0], b[1])

    def bench_inner_layout(self, interleave, lane_instances=1, reps=20, nbatch=1):
        """bench_inner in FP32x2 with a given instance layout (SolveOpts.interleave and
        lane_instances) instead of the one the batch solves use."""
        s = (C.c_double * 2)()
        b = (C.c_double * 2)()
        _check(lib().heom_bench_inner_layout(self.h, nbatch, reps, interleave, lane_instances, s, b))
        return (s[0], s[1]), (b[0], b[1])

    def tuned_layout(self, nbatch, truncated=False):
        """(interleave, lane_instances) the automatic choice keeps for mixed batch solves of
        nbatch instances, or (0, 0) while it is still timing the candidates."""
        g = C.c_int32()
        l = C.c_int32()
        _check(lib().heom_tuned_layout(self.h, nbatch, 1 if truncated else 0, C.byref(g), C.byref(l)))
        return g.value, l.value

    def stats(self):
        """Plan statistics (see heom_ctx_stats in include/heom_gb300.h)."""
        out = np.zeros(9)
        _check(lib().heom_ctx_stats(self.h, out.ctypes.data))
        keys = ("entries", "ados", "classes", "couplings", "maps", "gathers", "same_tier_terms", "lower_gathers", "plan_bytes")
        return dict(zip(keys, out.tolist()))


class CorrFunc:
    """Frequency-domain correlation functions of B = a_{iorbs,ispin} (corrfunc/): the operator
    calc_ax_cf_spa_omp, the solve solve_cf_tfqmr_spa batched over frequencies, and the
    spectral function of corrfunc.f90.  pattern: dict of nnzcf_spa, indcf_spa, irowcf_spa,
    icolcf_spa (1-based, as prelude_cf_spa makes them); default: the model's own."""

    def __init__(self, ctx, iorbs=1, ispin=1, pattern=None):
        self.ctx = ctx
        pat = pattern if pattern is not None else ctx.model.cf_pattern(iorbs, ispin)
        self.pattern = {
            "nnzcf_spa": np.ascontiguousarray(pat["nnzcf_spa"], dtype=np.int32),
            "indcf_spa": np.ascontiguousarray(pat["indcf_spa"], dtype=np.int64),
            "irowcf_spa": np.ascontiguousarray(pat["irowcf_spa"], dtype=np.int32),
            "icolcf_spa": np.ascontiguousarray(pat["icolcf_spa"], dtype=np.int32),
        }
        t = CfTables(iorbs=iorbs, ispin=ispin, lunkcf_spa=int(self.pattern["irowcf_spa"].size))
        for k, v in self.pattern.items():
            setattr(t, k, v.ctypes.data)
        h = C.c_void_p()
        _check(lib().heom_cf_create(ctx.h, C.byref(ctx.model.tables), C.byref(t), C.byref(h)))
        self.h = h
        self.iorbs, self.ispin = iorbs, ispin
        self.lunkcf = int(lib().heom_cf_lunk(h))
        self.nrho = ctx.model.nrho

    def close(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.heom_cf_destroy(self.h)
            self.h = None

    __del__ = close

    def calc_ax_cf_spa(self, dfreq, isgnw, rcga, rcgb):
        """(rhsa, rhsb) = L_cf (rcga, rcgb); dfreq in energy / hbar."""
        xa, xb = _c128(rcga, self.lunkcf), _c128(rcgb, self.lunkcf)
        ya = np.zeros(self.lunkcf, dtype=np.complex128)
        yb = np.zeros(self.lunkcf, dtype=np.complex128)
        _check(lib().heom_cf_calc_ax(self.h, float(dfreq), int(isgnw), self.lunkcf, xa.ctypes.data, xb.ctypes.data,
                                     ya.ctypes.data, yb.ctypes.data))
        return ya, yb

    def solve_cf_tfqmr_spa(self, rho, isgnb, isgnw, dfreq, crit=1e-10, maxit0=20000, precision=PREC_FP64):
        """RDO blocks (zouth, zouta), each (nfreq, nrho, nrho), of the solves at every dfreq."""
        w = np.ascontiguousarray(np.atleast_1d(dfreq), dtype=np.float64)
        rho = _c128(rho, self.ctx.lunk)
        n = self.nrho
        zh = np.zeros(w.size * n * n, dtype=np.complex128)
        za = np.zeros(w.size * n * n, dtype=np.complex128)
        o = SolveOpts(crit=crit, maxit0=maxit0, precision=precision)
        info = SolveInfo()
        _check(lib().heom_cf_solve(self.h, rho.ctypes.data, int(isgnb), int(isgnw), w.size, w.ctypes.data, C.byref(o),
                                   zh.ctypes.data, za.ctypes.data, C.byref(info)))
        # column-major nrho x nrho blocks
        return zh.reshape(w.size, n, n).transpose(0, 2, 1), za.reshape(w.size, n, n).transpose(0, 2, 1), info

    def dos(self, rho, freq_ev, crit=1e-10, maxit0=20000, precision=PREC_FP64):
        """Columns A(w), occupied part, empty part, Re G^r, Im G^r at every frequency (eV)."""
        f = np.ascontiguousarray(np.atleast_1d(freq_ev), dtype=np.float64)
        rho = _c128(rho, self.ctx.lunk)
        out = np.zeros(5 * f.size)
        o = SolveOpts(crit=crit, maxit0=maxit0, precision=precision)
        info = SolveInfo()
        _check(lib().heom_cf_dos(self.h, rho.ctypes.data, f.size, f.ctypes.data, C.byref(o), out.ctypes.data,
                                 C.byref(info)))
        return out.reshape(f.size, 5), info

    def propagate(self, rho, dt, nstep, ljw=True, rdo=False):
        """Time-domain correlation functions (corrfunc lfreq_dos = F): corr (nstep+1, 2) and, with
        rdo, the RDO blocks of X_h and X_a at every step (nstep+1, nrho, nrho).  dt in 1/(energy/hbar)."""
        rho = _c128(rho, self.ctx.lunk)
        corr = np.zeros(2 * (nstep + 1), dtype=np.complex128)
        n = self.nrho
        rh = np.zeros((nstep + 1) * n * n, dtype=np.complex128) if rdo else None
        ra = np.zeros((nstep + 1) * n * n, dtype=np.complex128) if rdo else None
        _check(lib().heom_cf_propagate(self.h, rho.ctypes.data, float(dt), int(nstep), int(bool(ljw)), corr.ctypes.data,
                                       None if rh is None else rh.ctypes.data, None if ra is None else ra.ctypes.data))
        corr = corr.reshape(nstep + 1, 2)
        if not rdo:
            return corr
        return corr, rh.reshape(nstep + 1, n, n).transpose(0, 2, 1), ra.reshape(nstep + 1, n, n).transpose(0, 2, 1)

    def bench_inner(self, nbatch=2, reps=20):
        """((B s, A s), (B bytes, A bytes)) per launch of the fused FP32x2 inner kernels."""
        out = np.zeros(4)
        _check(lib().heom_cf_bench_inner(self.h, nbatch, reps, out.ctypes.data))
        return (out[0], out[1]), (out[2], out[3])

    def bench_apply(self, nbatch=1, reps=20):
        """(seconds per launch, algorithmic bytes per launch) of the FP64 cf apply."""
        s = C.c_double()
        b = C.c_double()
        _check(lib().heom_cf_bench_apply(self.h, nbatch, reps, C.byref(s), C.byref(b)))
        return s.value, b.value


class Batch:
    """Instances of one table set (bias / level sweeps) solved together; parameters stay on
    the device.  x_dev: device pointer (int) to nbatch FP64 complex vectors of stride `stride`.

    ntier: optional tier count per instance (1 .. the context's ntier): instance b is solved
    on the hierarchy truncated at ntier[b] tiers, in the context's layout (heom_batch_set_tiers)."""

    def __init__(self, ctx, hs_batch=None, eshift_batch=None, nbatch=None, ntier=None):
        self.ctx = ctx
        if nbatch is None:
            nbatch = len(hs_batch) if hs_batch is not None else len(eshift_batch)
        self.nbatch = nbatch
        self._hs = None if hs_batch is None else _c128(hs_batch)
        self._es = None if eshift_batch is None else np.ascontiguousarray(eshift_batch, dtype=np.float64)
        h = C.c_void_p()
        _check(lib().heom_batch_create(ctx.h, nbatch, None if self._hs is None else self._hs.ctypes.data,
                                       None if self._es is None else self._es.ctypes.data, C.byref(h)))
        self.h = h
        self.stride = lib().heom_batch_stride(h)
        self._tiers = None
        if ntier is not None:
            self._tiers = np.ascontiguousarray(ntier, dtype=np.int32)
            if self._tiers.shape != (nbatch,):
                self.close()
                raise HeomError(-1, f"ntier needs one tier count per instance ({nbatch})")
            rc = lib().heom_batch_set_tiers(h, self._tiers.ctypes.data)
            if rc:
                msg = lib().heom_last_error().decode()
                self.close()
                raise HeomError(rc, msg)

    def solve_dev(self, x_dev, crit=1e-8, maxit0=20000, precision=PREC_MIXED, inner_tol=0.0, max_refine=8, check=True,
                  stag_window=0, inner_precond=0, interleave=0, lane_instances=0):
        o = SolveOpts(crit=crit, maxit0=maxit0, precision=precision, inner_tol=inner_tol, max_refine=max_refine,
                      stag_window=stag_window, inner_precond=inner_precond, interleave=interleave,
                      lane_instances=lane_instances)
        info = SolveInfo()
        rc = lib().heom_batch_solve_dev(self.h, C.byref(o), C.c_void_p(x_dev), C.byref(info))
        if check:
            _check(rc)
        return info

    def currents_static(self, x_dev, nbatch=None, vstride=None):
        """Lead currents jt[b, ialf, ispin] of device states, without device allocation.

        The C entry point takes at most STATIC_CURRENT_MAX instances per call; larger batches
        go through it in consecutive chunks of the same device array."""
        n = self.nbatch if nbatch is None else nbatch
        vs = self.stride if vstride is None else vstride
        if n < 1 or n > self.nbatch:
            raise HeomError(-1, f"nbatch {n} outside 1..{self.nbatch} (the vectors of this batch)")
        ns = self.ctx.model.nalf * self.ctx.model.nspin
        jt = np.zeros(n * ns)
        for b0, cnt in static_current_chunks(n):
            _check(lib().heom_batch_current_static(self.ctx.h, C.c_void_p(x_dev + b0 * vs * 16), cnt, vs,
                                                    jt[b0 * ns:].ctypes.data))
        return jt.reshape(n, self.ctx.model.nspin, self.ctx.model.nalf).transpose(0, 2, 1)

    def close(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.heom_batch_destroy(self.h)
            self.h = None

    __del__ = close
