"""ctypes loader for the CPU oracle (test infrastructure only: tests, smoke() and bench.py's
cpu_baseline leg use it as the checker; the product never imports it)."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None

I64P = ctypes.POINTER(ctypes.c_int64)
I32P = ctypes.POINTER(ctypes.c_int32)
F64P = ctypes.POINTER(ctypes.c_double)


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.oracle_hypot.restype = ctypes.c_double
        L.oracle_hypot.argtypes = [ctypes.c_double, ctypes.c_double]
        L.oracle_hypotf.restype = ctypes.c_float
        L.oracle_hypotf.argtypes = [ctypes.c_float, ctypes.c_float]
        L.oracle_score.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, F64P]
        L.oracle_spai.restype = ctypes.c_void_p
        L.oracle_spai.argtypes = [ctypes.c_int, ctypes.c_int64, I64P, I64P, F64P, ctypes.c_double,
                                  ctypes.c_int64, ctypes.c_int64, ctypes.c_int]
        L.oracle_spai_info.argtypes = [ctypes.c_void_p, I64P]
        L.oracle_spai_p.argtypes = [ctypes.c_void_p, I64P, I64P, F64P]
        L.oracle_spai_columns.argtypes = [ctypes.c_void_p, I32P, I32P, I32P, I32P, I32P, F64P, F64P]
        L.oracle_spai_column.restype = ctypes.c_int64
        L.oracle_spai_column.argtypes = [ctypes.c_void_p, ctypes.c_int64, I64P, F64P]
        L.oracle_spai_fit.restype = ctypes.c_int
        L.oracle_spai_fit.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, I64P, I64P, I64P,
                                      I64P, I64P, F64P, F64P, F64P]
        L.oracle_spai_free.argtypes = [ctypes.c_void_p]
        L.oracle_gmres.argtypes = [ctypes.c_int, ctypes.c_int64, I64P, I64P, F64P, I64P, I64P, F64P,
                                   F64P, ctypes.c_double, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, F64P, F64P]
        L.oracle_ir.restype = ctypes.c_int
        L.oracle_ir.argtypes = [ctypes.c_int, ctypes.c_int64, I64P, I64P, F64P, F64P, F64P, F64P, F64P, F64P]
        L.oracle_spai_sample.restype = ctypes.c_double
        L.oracle_spai_sample.argtypes = [ctypes.c_int, ctypes.c_int64, I64P, I64P, F64P, ctypes.c_double,
                                         ctypes.c_int64, ctypes.c_int64, I64P, ctypes.c_int64, ctypes.c_int,
                                         I64P]
        L.oracle_spai_columns_sample.restype = ctypes.c_int64
        L.oracle_spai_columns_sample.argtypes = [ctypes.c_int, ctypes.c_int64, I64P, I64P, F64P, ctypes.c_double,
                                                 ctypes.c_int64, ctypes.c_int64, I64P, ctypes.c_int64,
                                                 ctypes.c_int, I32P, I32P, I32P, I32P, F64P, I32P, I64P,
                                                 I64P, F64P, ctypes.c_int64]
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_refine.restype = ctypes.c_int
        L.oracle_refine.argtypes = [ctypes.c_int64, I64P, I64P, F64P, I64P, I64P, F64P, F64P, F64P,
                                    F64P, F64P, F64P]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def _csr(system):
    n, ptr, idx, val = system
    return (int(n), np.ascontiguousarray(ptr, np.int64), np.ascontiguousarray(idx, np.int64),
            np.ascontiguousarray(val, np.float64))


PRECISION = {"f64": 0, "f32": 1, "mixed": 2}


class Spai:
    """Oracle SPAI result: status, P (CSR), per-column metadata."""

    def __init__(self, system, epsilon=0.3, alpha=5, beta=8, precision="f64", history=False):
        n, ptr, idx, val = _csr(system)
        L = lib()
        self.n = n
        self._h = L.oracle_spai(1 if precision == "f32" else 0, n, _p(ptr, I64P), _p(idx, I64P),
                                _p(val, F64P), epsilon, alpha, beta, 1 if history else 0)
        info = np.zeros(3, np.int64)
        L.oracle_spai_info(self._h, _p(info, I64P))
        self.status, self.first_failed, nnz = int(info[0]), int(info[1]), int(info[2])
        self.p_ptr = np.zeros(n + 1, np.int64)
        self.p_idx = np.zeros(nnz, np.int64)
        self.p_val = np.zeros(nnz, np.float64)
        L.oracle_spai_p(self._h, _p(self.p_ptr, I64P), _p(self.p_idx, I64P), _p(self.p_val, F64P))
        if self.status == 2 and nnz == 0 and not np.any(self.p_ptr):
            pass
        self.col_status = np.zeros(n, np.int32)
        self.fits = np.zeros(n, np.int32)
        self.growths = np.zeros(n, np.int32)
        self.clamps = np.zeros(n, np.int32)
        self.qsize = np.zeros(n, np.int32)
        self.residual = np.zeros(n)
        self.scaling = np.zeros(n)
        L.oracle_spai_columns(self._h, _p(self.col_status, I32P), _p(self.fits, I32P),
                              _p(self.growths, I32P), _p(self.clamps, I32P), _p(self.qsize, I32P),
                              _p(self.residual, F64P), _p(self.scaling, F64P))

    @property
    def p(self):
        return (self.n, self.p_ptr, self.p_idx, self.p_val)

    def column(self, k):
        q = int(self.qsize[k])
        pat = np.zeros(q, np.int64)
        coef = np.zeros(q)
        lib().oracle_spai_column(self._h, k, _p(pat, I64P), _p(coef, F64P))
        return pat, coef

    def fit(self, k, f):
        L = lib()
        sizes = np.zeros(5, np.int64)
        if L.oracle_spai_fit(self._h, k, f, _p(sizes, I64P), None, None, None, None, None, None, None) != 0:
            return None
        q, m, c, s, ns = (int(x) for x in sizes)
        pat, sh, cand, sel = (np.zeros(x, np.int64) for x in (q, m, c, s))
        scores, coef, scal = np.zeros(ns), np.zeros(q), np.zeros(3)
        L.oracle_spai_fit(self._h, k, f, _p(sizes, I64P), _p(pat, I64P), _p(sh, I64P), _p(cand, I64P),
                          _p(sel, I64P), _p(scores, F64P), _p(coef, F64P), _p(scal, F64P))
        return dict(pattern=pat, shadow=sh, candidates=cand, selected=sel, scores=scores,
                    coefficients=coef, residual=scal[0], mean_score=scal[1], pivot_ratio=scal[2])

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_spai_free(self._h)
            self._h = None


def score(rsq, dot, den, precision="f64"):
    out = np.zeros(3)
    lib().oracle_score(1 if precision == "f32" else 0, rsq, dot, den, _p(out, F64P))
    return int(out[0]), float(out[1]), bool(out[2])


IR_KEYS = ("status", "converged", "outer_steps", "inner_attempts", "inner_iterations", "nbe", "cbe",
           "residual_inf", "forward", "spai_status", "nnz_p", "last_inner_status", "spai_seconds",
           "refine_seconds")


def _ir_report(rep):
    d = dict(zip(IR_KEYS, rep.tolist()))
    for k in ("status", "converged", "outer_steps", "inner_attempts", "inner_iterations",
              "spai_status", "nnz_p", "last_inner_status"):
        d[k] = int(d[k])
    d["converged"] = bool(d["converged"])
    return d


def ir(system, b, precision="f64", epsilon=0.3, alpha=None, beta=8, tau=None, innercap=0,
       outercap=20, be_tolerance=0.0, reference=None, lazy=True, wide=None):
    """Full SPAI-GMRES-IR pipeline; returns (x, report dict). wide: binary32 GMRES dots and
    norms accumulated in binary64 (None = by precision: on for mixed, off for f32)."""
    n, ptr, idx, val = _csr(system)
    if alpha is None:
        alpha = (n + 7) // 8
    if tau is None:
        tau = 1e-8 if precision == "f64" else 1e-4
    b = np.ascontiguousarray(b, np.float64)
    x = np.zeros(n)
    opts = np.array([epsilon, alpha, beta, tau, innercap, outercap, be_tolerance, 1 if lazy else 0,
                     -1 if wide is None else int(bool(wide))], np.float64)
    rep = np.zeros(14)
    ref = None if reference is None else np.ascontiguousarray(reference, np.float64)
    lib().oracle_ir(PRECISION[precision], n, _p(ptr, I64P), _p(idx, I64P), _p(val, F64P), _p(b, F64P),
                    None if ref is None else _p(ref, F64P), _p(opts, F64P), _p(x, F64P), _p(rep, F64P))
    return x, _ir_report(rep)


def refine(system, p_system, b, tau=1e-8, innercap=0, outercap=20, be_tolerance=0.0, reference=None,
           lazy=True):
    """refine_with_preconditioner (binary64) with an explicit P."""
    n, ptr, idx, val = _csr(system)
    _, pptr, pidx, pval = _csr(p_system)
    b = np.ascontiguousarray(b, np.float64)
    x = np.zeros(n)
    opts = np.array([0.3, 1, 8, tau, innercap, outercap, be_tolerance, 1 if lazy else 0], np.float64)
    rep = np.zeros(12)
    ref = None if reference is None else np.ascontiguousarray(reference, np.float64)
    lib().oracle_refine(n, _p(ptr, I64P), _p(idx, I64P), _p(val, F64P), _p(pptr, I64P), _p(pidx, I64P),
                        _p(pval, F64P), _p(b, F64P), None if ref is None else _p(ref, F64P), _p(opts, F64P),
                        _p(x, F64P), _p(rep, F64P))
    return x, _ir_report(rep)


GMRES_KEYS = ("status", "converged", "iterations", "final_original", "final_relative")


def gmres(system, p_system, rhs, tol=1e-8, cap=0, precision="f64", accept_every=False, lazy=True, wide=False):
    n, ptr, idx, val = _csr(system)
    _, pptr, pidx, pval = _csr(p_system)
    rhs = np.ascontiguousarray(rhs, np.float64)
    x = np.zeros(n)
    rep = np.zeros(5)
    lib().oracle_gmres(1 if precision == "f32" else 0, n, _p(ptr, I64P), _p(idx, I64P), _p(val, F64P),
                       _p(pptr, I64P), _p(pidx, I64P), _p(pval, F64P), _p(rhs, F64P), tol, cap,
                       1 if accept_every else 0, 1 if lazy else 0, 1 if wide else 0, _p(x, F64P),
                       _p(rep, F64P))
    d = dict(zip(GMRES_KEYS, rep.tolist()))
    d["status"], d["converged"], d["iterations"] = int(d["status"]), bool(d["converged"]), int(d["iterations"])
    return x, d


def spai_sample_seconds(system, cols, epsilon=0.3, alpha=5, beta=8, precision="f64", threads=1):
    """Wall seconds of the oracle's adaptive fits for the given columns (threads in parallel)."""
    n, ptr, idx, val = _csr(system)
    cols = np.ascontiguousarray(cols, np.int64)
    fits = ctypes.c_int64()
    sec = lib().oracle_spai_sample(1 if precision in ("f32", "mixed") else 0, n, _p(ptr, I64P), _p(idx, I64P),
                                   _p(val, F64P), epsilon, alpha, beta, _p(cols, I64P), len(cols), threads,
                                   ctypes.byref(fits))
    return sec, fits.value


def set_threads(threads):
    """Threads for the SPAI construction's column fits (the result does not depend on it)."""
    lib().oracle_set_threads(int(threads))


def spai_columns(system, cols, epsilon=0.3, alpha=5, beta=8, precision="f64", threads=1):
    """Adaptive fits of the listed columns only (no full construction): per-column status, fits,
    growths, clamps, residual, assembly flag, and their rows of P (ptr over the list, idx, val)."""
    n, ptr, idx, val = _csr(system)
    cols = np.ascontiguousarray(cols, np.int64)
    m = len(cols)
    st, fi, gr, cl, bad = (np.zeros(m, np.int32) for _ in range(5))
    res = np.zeros(m)
    pp = np.zeros(m + 1, np.int64)
    cap = max(64 * m, 1)
    for _ in range(2):
        pi = np.zeros(cap, np.int64)
        pv = np.zeros(cap)
        total = lib().oracle_spai_columns_sample(1 if precision in ("f32", "mixed") else 0, n, _p(ptr, I64P),
                                                 _p(idx, I64P), _p(val, F64P), epsilon, alpha, beta,
                                                 _p(cols, I64P), m, threads, _p(st, I32P), _p(fi, I32P),
                                                 _p(gr, I32P), _p(cl, I32P), _p(res, F64P), _p(bad, I32P),
                                                 _p(pp, I64P), _p(pi, I64P), _p(pv, F64P), cap)
        if total <= cap:
            return dict(status=st, fits=fi, growths=gr, clamps=cl, residual=res, assembly_bad=bad,
                        p_ptr=pp, p_idx=pi[:total], p_val=pv[:total])
        cap = int(total)
    raise RuntimeError("oracle_spai_columns_sample: capacity")


def hypot(a, b):
    return lib().oracle_hypot(a, b)


def hypotf(a, b):
    return lib().oracle_hypotf(a, b)
