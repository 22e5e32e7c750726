"""Python mirror of the libspai_ir C ABI (include/spai_ir.h).

Names and semantics follow the reference's solver API (include/bspai/*.hpp): the status enums
and their names, SpaiOptions/GmresOptions/IrOptions defaults, cuda_gpu_spai_gmres_ir as
ir_solve(), CudaGmresContext as Handle.gmres(), CudaCsrSpmv as Handle.spmv(). There is no CPU
fallback: loading fails loudly when the CUDA library has not been built.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "_build", "libspai_ir.so")
CLI_DIR = os.path.join(PKG, "_build")

PRECISION = {"f64": 0, "f32": 1, "mixed": 2}
FLAG_NO_GRAPH = 1
FLAG_FAST_SPAI = 2
FLAG_HISTORY = 4
FLAG_RESTART_AT_CAP = 8
FLAG_RIGHT_PRECONDITIONING = 16
FLAG_EXACT_SPAI = 0  # sequential, bit-reproducing SPAI (the default)

SPAI_STATUS = ["success", "not_attempted", "invalid_input", "rank_deficient", "numerical_failure",
               "empty_candidates", "zero_denominator", "invalid_score", "no_growth", "iteration_limit"]
GMRES_STATUS = ["success", "zero_rhs", "exact_initial_solution", "invalid_input",
                "zero_preconditioned_rhs", "breakdown", "iteration_limit", "nonconvergence",
                "numerical_failure"]
IR_STATUS = ["success", "invalid_input", "construction_failure", "inner_failure", "stagnation",
             "iteration_limit", "numerical_failure"]

(IR_SUCCESS, IR_INVALID_INPUT, IR_CONSTRUCTION_FAILURE, IR_INNER_FAILURE, IR_STAGNATION, IR_ITERATION_LIMIT,
 IR_NUMERICAL_FAILURE) = range(7)

OK, ERR_ARGUMENT, ERR_CUDA, ERR_WORKSPACE, ERR_TIMEOUT, ERR_NOT_BUILT, ERR_UNSUPPORTED = 0, -1, -2, -3, -4, -5, -6
ERR_FORMAT = -7


class SpaiError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"libspai_ir error {code}: {message}")
        self.code = code


class Csr(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("nnz", ctypes.c_int64),
                ("row_offsets", ctypes.POINTER(ctypes.c_int64)),
                ("col_indices", ctypes.POINTER(ctypes.c_int64)),
                ("values", ctypes.POINTER(ctypes.c_double))]


class Options(ctypes.Structure):
    _fields_ = [("epsilon", ctypes.c_double), ("alpha", ctypes.c_int64), ("beta", ctypes.c_int64),
                ("tau", ctypes.c_double), ("innercap", ctypes.c_int64), ("outercap", ctypes.c_int64),
                ("be_tolerance", ctypes.c_double), ("precision", ctypes.c_int32),
                ("flags", ctypes.c_int32)]


class OuterRecord(ctypes.Structure):
    _fields_ = [("step", ctypes.c_int64), ("residual_inf", ctypes.c_double), ("residual_2", ctypes.c_double),
                ("normwise_backward_error", ctypes.c_double), ("componentwise_backward_error", ctypes.c_double)]


class InnerRecord(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("update_applied", ctypes.c_int32), ("iterations", ctypes.c_int64),
                ("final_relative", ctypes.c_double)]


class IterationRecord(ctypes.Structure):
    _fields_ = [("inner", ctypes.c_int64), ("iteration", ctypes.c_int64), ("estimated_relative", ctypes.c_double),
                ("recomputed_relative", ctypes.c_double), ("accepted", ctypes.c_int32), ("triggered", ctypes.c_int32)]


def _records(arr, count):
    return [{f: getattr(arr[i], f) for f, _ in arr[i]._fields_ } for i in range(count)]


class Report(ctypes.Structure):
    _fields_ = [("ir_status", ctypes.c_int32), ("spai_status", ctypes.c_int32),
                ("gmres_status", ctypes.c_int32), ("converged", ctypes.c_int32),
                ("outer_steps", ctypes.c_int64), ("inner_attempts", ctypes.c_int64),
                ("inner_iterations", ctypes.c_int64), ("nnz_p", ctypes.c_int64),
                ("first_failed_column", ctypes.c_int64), ("backward_error", ctypes.c_double),
                ("componentwise_backward_error", ctypes.c_double), ("residual_inf", ctypes.c_double),
                ("forward_error", ctypes.c_double), ("spai_ms", ctypes.c_double),
                ("solve_ms", ctypes.c_double), ("spai_fits", ctypes.c_int64),
                ("spai_growths", ctypes.c_int64), ("spai_overflow_columns", ctypes.c_int64),
                ("kernel_launches", ctypes.c_int64)]

    def as_dict(self):
        d = {name: getattr(self, name) for name, _ in self._fields_}
        d["converged"] = bool(d["converged"])
        return d


I64P = ctypes.POINTER(ctypes.c_int64)
I32P = ctypes.POINTER(ctypes.c_int32)
F64P = ctypes.POINTER(ctypes.c_double)
VP = ctypes.c_void_p

# Every exported entry point of include/spai_ir.h with its ctypes signature.
SIGNATURES = {
    "spai_default_options": (ctypes.c_int, [ctypes.POINTER(Options), ctypes.c_int32]),
    "spai_status_name": (ctypes.c_char_p, [ctypes.c_int32]),
    "gmres_status_name": (ctypes.c_char_p, [ctypes.c_int32]),
    "ir_status_name": (ctypes.c_char_p, [ctypes.c_int32]),
    "spai_last_error": (ctypes.c_char_p, []),
    "spai_create": (ctypes.c_int, [ctypes.POINTER(Csr), ctypes.c_int32, ctypes.c_int, VP, ctypes.POINTER(VP)]),
    "spai_destroy": (ctypes.c_int, [VP]),
    "spai_build": (ctypes.c_int, [VP, ctypes.POINTER(Options), ctypes.POINTER(Report)]),
    "spai_solve": (ctypes.c_int, [VP, F64P, F64P, F64P, ctypes.POINTER(Options), ctypes.POINTER(Report)]),
    "spai_solve_device": (ctypes.c_int, [VP, VP, VP, ctypes.POINTER(Options), ctypes.POINTER(Report)]),
    "spai_ir_solve": (ctypes.c_int, [ctypes.POINTER(Csr), F64P, F64P, F64P, ctypes.POINTER(Options),
                                     ctypes.POINTER(Report), VP]),
    "spai_get_preconditioner": (ctypes.c_int, [VP, I64P, I64P, I64P, F64P]),
    "spai_get_columns": (ctypes.c_int, [VP, I32P, I32P, I32P, I32P, F64P, F64P]),
    "spai_get_column": (ctypes.c_int, [VP, ctypes.c_int64, I64P, I64P, F64P]),
    "spai_spmv": (ctypes.c_int, [VP, ctypes.c_int32, F64P, F64P]),
    "spai_gmres": (ctypes.c_int, [VP, F64P, F64P, ctypes.c_double, ctypes.c_int64, I32P, I64P, F64P]),
    "spai_score": (ctypes.c_int, [ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double, F64P]),
    "spai_ir_solve_batched": (ctypes.c_int, [ctypes.c_int64, ctypes.POINTER(Csr), ctypes.POINTER(F64P),
                                             ctypes.POINTER(F64P), ctypes.POINTER(Options),
                                             ctypes.POINTER(Report), VP]),
    "spai_adjoint": (ctypes.c_int, [VP, ctypes.c_int64, F64P, F64P, F64P, F64P, ctypes.POINTER(Options),
                                    ctypes.POINTER(Report)]),
    "spai_adjoint_device": (ctypes.c_int, [VP, ctypes.c_int64, VP, VP, VP, VP, ctypes.POINTER(Options),
                                           ctypes.POINTER(Report)]),
    "spai_mm_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int64, ctypes.POINTER(VP)]),
    "spai_mm_csr": (ctypes.c_int, [VP, ctypes.POINTER(Csr), I64P, I64P]),
    "spai_mm_free": (ctypes.c_int, [VP]),
    "spai_history": (ctypes.c_int, [VP, VP, ctypes.c_int64, I64P, VP, ctypes.c_int64, I64P, VP, ctypes.c_int64, I64P]),
    "spai_profile": (ctypes.c_int, [VP, ctypes.c_int32]),
    "spai_profile_read": (ctypes.c_int, [VP, ctypes.c_int32, F64P, I64P, F64P]),
    "spai_backward_error_noalloc": (ctypes.c_int, [VP, VP, VP, VP, VP]),
    "spai_tuning": (ctypes.c_int, [VP, I32P, F64P]),
    "spai_hypot_device": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, F64P, F64P, F64P]),
    "spai_set_preconditioner": (ctypes.c_int, [VP, ctypes.POINTER(Csr)]),
    "spai_record": (ctypes.c_int, [VP, ctypes.c_int32]),
    "spai_fit_log": (ctypes.c_int, [VP, I32P, ctypes.c_int64, I64P, F64P, ctypes.c_int64, I64P]),
    "spai_record_counts": (ctypes.c_int, [VP, I64P, I64P]),
    "spai_record_state": (ctypes.c_int, [VP, ctypes.c_int64, F64P, F64P]),
    "spai_record_inner": (ctypes.c_int, [VP, ctypes.c_int64, F64P, F64P, F64P, F64P, F64P, F64P, F64P]),
    "spai_hypot": (ctypes.c_double, [ctypes.c_double, ctypes.c_double]),
    "spai_hypotf": (ctypes.c_float, [ctypes.c_float, ctypes.c_float]),
}

_lib = None


def lib():
    """Load the in-tree CUDA library; raises if it has not been built (no CPU fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libspai_ir.so not built at {LIB_PATH}; run __graft_entry__.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc != OK:
        raise SpaiError(rc, lib().spai_last_error().decode())


def _p(a, t):
    return a.ctypes.data_as(t)


class _CsrHolder:
    """Keeps the int64/float64 arrays of a canonical CSR alive while C holds pointers to them."""

    def __init__(self, system):
        n, ptr, idx, val = system
        self.ptr = np.ascontiguousarray(ptr, np.int64)
        self.idx = np.ascontiguousarray(idx, np.int64)
        self.val = np.ascontiguousarray(val, np.float64)
        self.n = int(n)
        self.csr = Csr(self.n, len(self.val), _p(self.ptr, I64P), _p(self.idx, I64P), _p(self.val, F64P))


def options(precision="f64", epsilon=0.3, alpha=5, beta=8, tau=0.0, innercap=0, outercap=20,
            be_tolerance=0.0, flags=0):
    """IrOptions with the reference defaults (spai.hpp:24-28, gmres.hpp:23-26, ir.hpp:20-24)."""
    o = Options()
    _check(lib().spai_default_options(ctypes.byref(o), PRECISION[precision]))
    o.epsilon, o.alpha, o.beta, o.tau = epsilon, alpha, beta, tau
    o.innercap, o.outercap, o.be_tolerance, o.flags = innercap, outercap, be_tolerance, flags
    return o


def cli_options(n, precision="f64", epsilon=0.3, outercap=20, innercap=0, **kw):
    """Options the drop-in CLI uses: alpha = ceil(n/8), beta = 8 (src/solver_main.cpp:75-76)."""
    return options(precision, epsilon=epsilon, alpha=(n + 7) // 8, beta=8, outercap=outercap,
                   innercap=innercap, **kw)


class Handle:
    """Device-resident matrix, SPAI preconditioner and Krylov workspace (spai_handle)."""

    def __init__(self, system, precision="f64", device=0, stream=None):
        self.precision = precision
        self._csr = _CsrHolder(system)
        self.n = self._csr.n
        h = VP()
        _check(lib().spai_create(ctypes.byref(self._csr.csr), PRECISION[precision], device, stream,
                                 ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().spai_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def build(self, opts):
        rep = Report()
        _check(lib().spai_build(self._h, ctypes.byref(opts), ctypes.byref(rep)))
        return rep.as_dict()

    def solve(self, b, opts, reference=None):
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros(self.n)
        ref = None if reference is None else np.ascontiguousarray(reference, np.float64)
        rep = Report()
        _check(lib().spai_solve(self._h, _p(b, F64P), _p(x, F64P), None if ref is None else _p(ref, F64P),
                                ctypes.byref(opts), ctypes.byref(rep)))
        return x, rep.as_dict()

    def solve_device(self, b_ptr, x_ptr, opts):
        rep = Report()
        _check(lib().spai_solve_device(self._h, VP(b_ptr), VP(x_ptr), ctypes.byref(opts), ctypes.byref(rep)))
        return rep.as_dict()

    def preconditioner(self):
        nnz = ctypes.c_int64()
        _check(lib().spai_get_preconditioner(self._h, ctypes.byref(nnz), None, None, None))
        ptr = np.zeros(self.n + 1, np.int64)
        idx = np.zeros(nnz.value, np.int64)
        val = np.zeros(nnz.value)
        _check(lib().spai_get_preconditioner(self._h, ctypes.byref(nnz), _p(ptr, I64P), _p(idx, I64P), _p(val, F64P)))
        return (self.n, ptr, idx, val)

    def columns(self):
        n = self.n
        st, fi, gr, cl = (np.zeros(n, np.int32) for _ in range(4))
        res, sc = np.zeros(n), np.zeros(n)
        _check(lib().spai_get_columns(self._h, _p(st, I32P), _p(fi, I32P), _p(gr, I32P), _p(cl, I32P),
                                      _p(res, F64P), _p(sc, F64P)))
        return dict(status=st, fits=fi, growths=gr, clamps=cl, residual=res, scaling=sc)

    def column(self, k):
        q = ctypes.c_int64()
        _check(lib().spai_get_column(self._h, k, ctypes.byref(q), None, None))
        pat = np.zeros(q.value, np.int64)
        coef = np.zeros(q.value)
        _check(lib().spai_get_column(self._h, k, ctypes.byref(q), _p(pat, I64P), _p(coef, F64P)))
        return pat, coef

    def spmv(self, which, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(self.n)
        _check(lib().spai_spmv(self._h, {"A": 0, "P": 1}[which], _p(x, F64P), _p(y, F64P)))
        return y

    def gmres(self, rhs, tau, cap=0):
        rhs = np.ascontiguousarray(rhs, np.float64)
        x = np.zeros(self.n)
        st, it, rel = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_double()
        _check(lib().spai_gmres(self._h, _p(rhs, F64P), _p(x, F64P), tau, cap, ctypes.byref(st),
                                ctypes.byref(it), ctypes.byref(rel)))
        return x, dict(status=st.value, iterations=it.value, final_relative=rel.value)

    def set_preconditioner(self, p):
        """Solve with a caller-supplied preconditioner P (canonical CSR (n, ptr, idx, val))."""
        self._p = _CsrHolder(p)
        _check(lib().spai_set_preconditioner(self._h, ctypes.byref(self._p.csr)))

    def record(self, enable=True):
        """Record mode (binary64): fit log of the next build, every step of the next solves."""
        _check(lib().spai_record(self._h, 1 if enable else 0))

    def fit_log(self):
        """Fit histories of the last recorded build: {column: [fit dict, ...]} in fit order.

        Each fit: J, I (index lists), coefficients, residual, pivot_ratio and, for fits that
        went on to candidate scoring, candidates, scores, mean_score, selected (selection
        order). Records of abandoned workspace tiers are dropped (the column's highest tier
        holds its history)."""
        ni, nv = ctypes.c_int64(), ctypes.c_int64()
        _check(lib().spai_fit_log(self._h, None, 0, ctypes.byref(ni), None, 0, ctypes.byref(nv)))
        ints = np.zeros(max(ni.value, 1), np.int32)
        vals = np.zeros(max(nv.value, 1))
        _check(lib().spai_fit_log(self._h, _p(ints, I32P), ni.value, ctypes.byref(ni), _p(vals, F64P), nv.value,
                                  ctypes.byref(nv)))
        recs = {}
        pos = 0
        while pos < ni.value:
            kind, k, tier, fit, a, b, c, vo = (int(v) for v in ints[pos:pos + 8])
            body = ints[pos + 8:]
            if kind == 1:
                rec = dict(J=body[:a].tolist(), I=body[a:a + b].tolist(), residual=float(vals[vo]),
                           pivot_ratio=float(vals[vo + 1]), coefficients=vals[vo + 2:vo + 2 + a].copy())
                pos += 8 + a + b
            elif kind == 2:
                rec = dict(candidates=body[:a].tolist(), mean_score=float(vals[vo]),
                           scores=vals[vo + 1:vo + 1 + a].copy())
                pos += 8 + a
            elif kind == 3:
                rec = dict(selected=body[:a].tolist())
                pos += 8 + a
            else:
                raise SpaiError(-1, f"corrupt fit log record kind {kind} at {pos}")
            recs.setdefault(k, []).append((tier, fit, kind, rec))
        out = {}
        for k, lst in recs.items():
            top = max(t for t, _, _, _ in lst)
            fits = {}
            for tier, fit, kind, rec in lst:
                if tier == top:
                    fits.setdefault(fit, {}).update(rec)
            out[k] = [fits[f] for f in sorted(fits)]
        return out

    def recorded(self):
        """Record of the last recorded solve: dict(states=[(x, residual)], inner=[dict])."""
        L = lib()
        ns, nin = ctypes.c_int64(), ctypes.c_int64()
        _check(L.spai_record_counts(self._h, ctypes.byref(ns), ctypes.byref(nin)))
        n = self.n
        states = []
        for s in range(ns.value):
            x, r = np.zeros(n), np.zeros(n)
            _check(L.spai_record_state(self._h, s, _p(x, F64P), _p(r, F64P)))
            states.append((x, r))
        inner = []
        for i in range(nin.value):
            sm = np.zeros(12)
            _check(L.spai_record_inner(self._h, i, _p(sm, F64P), None, None, None, None, None, None))
            m, nb, hr, hc = int(sm[2]), int(sm[8]), int(sm[9]), int(sm[10])
            rhs, sol = np.zeros(n), np.zeros(n)
            basis = np.zeros((max(nb, 1), n))
            hess = np.zeros((max(hr, 1), max(hc, 1)))
            steps = np.zeros((max(m, 1), 8))
            cands = np.zeros((max(m, 1), n))
            _check(L.spai_record_inner(self._h, i, _p(sm, F64P), _p(rhs, F64P), _p(sol, F64P), _p(basis, F64P),
                                       _p(hess, F64P), _p(steps, F64P), _p(cands, F64P)))
            inner.append(dict(status=int(sm[0]), converged=bool(sm[1]), steps=m, applied=bool(sm[3]),
                              initial_original=float(sm[4]), initial_preconditioned=float(sm[5]),
                              final_original=float(sm[6]), final_preconditioned=float(sm[7]),
                              iterations=int(sm[11]), rhs=rhs, solution=sol, basis=basis[:nb],
                              hessenberg=hess[:hr, :hc], step_rows=steps[:m], candidates=cands[:m]))
        return dict(states=states, inner=inner)

    def backward_error_noalloc(self, d_b, d_x, d_out, stream=None):
        """Allocation-free backward error of device vector x (see spai_backward_error_noalloc)."""
        _check(lib().spai_backward_error_noalloc(self._h, VP(d_b), VP(d_x), VP(d_out), stream))

    def tuning(self):
        """Autotuner choices of the last build / solve set-up (see spai_tuning)."""
        out = np.zeros(5, np.int32)
        ms = np.zeros(2)
        _check(lib().spai_tuning(self._h, _p(out, I32P), _p(ms, F64P)))
        return dict(group_lanes=int(out[0]), ws_bytes=int(out[1]), spai_tuned=bool(out[2]),
                    spmv_layout_a=int(out[3]), spmv_layout_p=int(out[4]),
                    sample_ms=float(ms[0]), default_sample_ms=float(ms[1]))

    def history(self):
        """History of the last solve run with FLAG_HISTORY: (outer, inner, iterations) record lists."""
        no, ni, nt = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _check(lib().spai_history(self._h, None, 0, ctypes.byref(no), None, 0, ctypes.byref(ni), None, 0,
                                  ctypes.byref(nt)))
        outer = (OuterRecord * max(no.value, 1))()
        inner = (InnerRecord * max(ni.value, 1))()
        its = (IterationRecord * max(nt.value, 1))()
        _check(lib().spai_history(self._h, outer, no.value, ctypes.byref(no), inner, ni.value, ctypes.byref(ni),
                                  its, nt.value, ctypes.byref(nt)))
        return _records(outer, no.value), _records(inner, ni.value), _records(its, nt.value)

    KERNEL_CLASSES = ("spmv_A", "spmv_P", "cgs_pass1", "cgs_pass2", "cgs_pass3")

    def profile(self, enable=True):
        _check(lib().spai_profile(self._h, 1 if enable else 0))

    def profile_read(self):
        out = {}
        for c, name in enumerate(self.KERNEL_CLASSES):
            ms, ln, by = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double()
            _check(lib().spai_profile_read(self._h, c, ctypes.byref(ms), ctypes.byref(ln), ctypes.byref(by)))
            out[name] = dict(ms=ms.value, launches=ln.value, bytes=by.value)
        return out

    def adjoint(self, x, dldx, opts):
        x = np.asfortranarray(x, np.float64)
        dldx = np.asfortranarray(dldx, np.float64)
        nrhs = 1 if x.ndim == 1 else x.shape[1]
        dldb = np.zeros_like(dldx)
        dlda = np.zeros(len(self._csr.val))
        rep = Report()
        _check(lib().spai_adjoint(self._h, nrhs, _p(x, F64P), _p(dldx, F64P), _p(dldb, F64P), _p(dlda, F64P),
                                  ctypes.byref(opts), ctypes.byref(rep)))
        return dldb, dlda, rep.as_dict()

    def adjoint_device(self, nrhs, x_ptr, dldx_ptr, dldb_ptr, dlda_ptr, opts):
        """Adjoint with device pointers (column-major n x nrhs vectors, nnz gradient values)."""
        rep = Report()
        _check(lib().spai_adjoint_device(self._h, nrhs, x_ptr, dldx_ptr, dldb_ptr, dlda_ptr,
                                         ctypes.byref(opts), ctypes.byref(rep)))
        return rep.as_dict()


def ir_solve(system, b, opts, reference=None, stream=None):
    """One-shot solve (cuda_gpu_spai_gmres_ir / fp32_cuda_spai_gmres_ir): returns (x, report)."""
    holder = _CsrHolder(system)
    b = np.ascontiguousarray(b, np.float64)
    x = np.zeros(holder.n)
    ref = None if reference is None else np.ascontiguousarray(reference, np.float64)
    rep = Report()
    _check(lib().spai_ir_solve(ctypes.byref(holder.csr), _p(b, F64P), _p(x, F64P),
                               None if ref is None else _p(ref, F64P), ctypes.byref(opts),
                               ctypes.byref(rep), stream))
    return x, rep.as_dict()


def ir_solve_batched(systems, bs, opts, stream=None):
    holders = [_CsrHolder(s) for s in systems]
    arr = (Csr * len(holders))(*[h.csr for h in holders])
    bs = [np.ascontiguousarray(b, np.float64) for b in bs]
    xs = [np.zeros(h.n) for h in holders]
    bp = (F64P * len(bs))(*[_p(b, F64P) for b in bs])
    xp = (F64P * len(xs))(*[_p(x, F64P) for x in xs])
    reps = (Report * len(holders))()
    _check(lib().spai_ir_solve_batched(len(holders), arr, bp, xp, ctypes.byref(opts), reps, stream))
    return xs, [r.as_dict() for r in reps]


def score(rsq, dot, den, precision="f64"):
    out = np.zeros(3)
    _check(lib().spai_score(PRECISION[precision], rsq, dot, den, _p(out, F64P)))
    return int(out[0]), float(out[1]), bool(out[2])


def mm_read(path, device_min_lines=0):
    """Matrix Market file -> canonical CSR (n, ptr, idx, val) parsed on the device (spai_mm_read);
    also returns the column count and how many value tokens the host converted."""
    h = VP()
    _check(lib().spai_mm_read(str(path).encode(), device_min_lines, ctypes.byref(h)))
    try:
        c = Csr()
        cols, conv = ctypes.c_int64(), ctypes.c_int64()
        _check(lib().spai_mm_csr(h, ctypes.byref(c), ctypes.byref(cols), ctypes.byref(conv)))
        n, nnz = c.n, c.nnz
        ptr = np.ctypeslib.as_array(c.row_offsets, (n + 1,)).copy()
        idx = np.ctypeslib.as_array(c.col_indices, (nnz,)).copy() if nnz else np.zeros(0, np.int64)
        val = np.ctypeslib.as_array(c.values, (nnz,)).copy() if nnz else np.zeros(0)
        return (n, ptr, idx, val), cols.value, conv.value
    finally:
        lib().spai_mm_free(h)


HYPOT_KINDS = {"f64": 0, "f32": 1, "f64-chain": 2, "f32-chain": 3}


def hypot_device(a, b, precision="f64"):
    """The device hypot on arrays (binary32 for "f32": operands rounded, result widened);
    "f64-chain" / "f32-chain": the SPAI norm-chain step with |a| as the running norm."""
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    out = np.zeros(len(a))
    _check(lib().spai_hypot_device(HYPOT_KINDS[precision], len(a), _p(a, F64P), _p(b, F64P), _p(out, F64P)))
    return out


def hypot(a, b):
    return lib().spai_hypot(a, b)


def hypotf(a, b):
    return lib().spai_hypotf(a, b)


def cli_path(name):
    return os.path.join(CLI_DIR, name)
