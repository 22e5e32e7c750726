"""Release snapshot, schema 2, of this library's binary64 solver.

Prints the records the reference's release snapshot prints for its CPU library
(tests/release_cpu_snapshot.cpp:281-398): one ``RELEASE_CPU_SNAPSHOT {json}`` line per case, on
the same small systems, with every binary64 datum as a C99 hex-float string followed by ``@`` and
its IEEE-754 bits in hex (release_cpu_snapshot.cpp:38-57), so that the reference's Decimal80
audit (tests/check_release_cpu_decimal.py) can check this build unchanged.

Every number comes from the device: the SPAI fits from the column kernel's fit log, P and the
scaling D from the handle, the Krylov data from record mode (every step's candidate, the basis,
the unrotated Hessenberg, every iterate and residual; see spai_record in include/spai_ir.h).
Two fields are assembled here from device data: B = A^T D, whose entries the fits form on the fly
(B(i, j) = A(j, i) d_j, the product the device takes) and never store as a matrix, and N, the
unscaled columns (N(j, k) = m_jk, exact zero coefficients dropped). A fit's full residual is its
reduced residual: rows outside the shadow contribute exact zeros to the hypot chain.

One of the reference's sixteen cases is not emitted: ``gmres_exact_initial`` runs GMRES from a
nonzero initial guess, which this solver's GMRES does not take (the refinement always starts it
from zero).
"""
import json
import math
import struct
import sys

import numpy as np

from . import Handle, lib, options

__all__ = ["cases", "main"]


def spai_status_name(s):
    return lib().spai_status_name(int(s)).decode()


def gmres_status_name(s):
    return lib().gmres_status_name(int(s)).decode()


def ir_status_name(s):
    return lib().ir_status_name(int(s)).decode()


def _hex(x):
    """C99 hex-float of a finite binary64 plus '@' and its IEEE bits (exact round trip)."""
    x = float(x)
    if not math.isfinite(x):
        raise ValueError("snapshot values must be finite binary64")
    bits = struct.unpack(">Q", struct.pack(">d", x))[0]
    exponent = (bits >> 52) & 0x7FF
    fraction = bits & ((1 << 52) - 1)
    sign = "-" if bits >> 63 else ""
    lead, e = (1, exponent - 1023) if exponent else (0, -1022)
    return f"{sign}0x{lead}.{fraction:013x}p{e}@{bits:x}"


def _vals(v):
    return [_hex(x) for x in np.asarray(v, np.float64).ravel()]


def _csr(n, ptr, idx, val):
    return {"rows": int(n), "cols": int(n), "offsets": [int(v) for v in ptr],
            "indices": [int(v) for v in idx], "values": _vals(val)}


def _dense(rows):
    """Canonical CSR (n, ptr, idx, val) of a small dense matrix (stored zeros dropped)."""
    n = len(rows)
    ptr, idx, val = [0], [], []
    for row in rows:
        for j, v in enumerate(row):
            if v != 0:
                idx.append(j)
                val.append(float(v))
        ptr.append(len(idx))
    return (n, np.array(ptr, np.int64), np.array(idx, np.int64), np.array(val, np.float64))


def _from_entries(n, entries):
    entries = sorted(entries)
    ptr = np.zeros(n + 1, np.int64)
    for r, _, _ in entries:
        ptr[r + 1] += 1
    return (n, np.cumsum(ptr), np.array([c for _, c, _ in entries], np.int64),
            np.array([v for _, _, v in entries], np.float64))


def _identity(n):
    return _from_entries(n, [(i, i, 1.0) for i in range(n)])


def _gmres_obj(inner):
    """GmresResult (include/bspai/gmres.hpp:38-50) of one recorded inner solve."""
    steps = []
    for j, row in enumerate(inner["step_rows"]):
        it, est, rec, orig, sub, brk, trig, acc = row
        steps.append({"iteration": int(it), "solution": _vals(inner["candidates"][j]), "estimate": _hex(est),
                      "recomputed": _hex(rec), "original": _hex(orig), "subdiagonal": _hex(sub),
                      "breakdown": bool(brk), "verified": bool(trig), "accepted": bool(acc)})
    return {"status": gmres_status_name(inner["status"]), "converged": inner["converged"],
            "iterations": inner["steps"], "solution": _vals(inner["solution"]),
            "initial_original": _hex(inner["initial_original"]),
            "initial_preconditioned": _hex(inner["initial_preconditioned"]),
            "final_original": _hex(inner["final_original"]),
            "final_preconditioned": _hex(inner["final_preconditioned"]),
            "basis": [_vals(v) for v in inner["basis"]], "H": [_vals(r) for r in inner["hessenberg"]],
            "history": steps}


def _ir_obj(h, rep, record):
    """IrResult (include/bspai/ir.hpp:44-56) of one recorded refinement solve."""
    outer, _, _ = h.history()
    states = record["states"]
    inner = record["inner"]
    applied = [i for i, r in enumerate(inner) if r["applied"]]
    history = []
    for s, (x, r) in enumerate(states):
        d = outer[s]
        item = {"step": s, "x": _vals(x),
                "diagnostics": {"residual": _vals(r), "inf": _hex(d["residual_inf"]), "norm2": _hex(d["residual_2"]),
                                "nbe": _hex(d["normwise_backward_error"]),
                                "cbe": _hex(d["componentwise_backward_error"])},
                "has_inner": s > 0}
        if s > 0:
            item["inner"] = _gmres_obj(inner[applied[s - 1]])
        history.append(item)
    solution = states[-1][0] if states else np.zeros(h.n)
    return {"status": ir_status_name(rep["ir_status"]), "converged": bool(rep["converged"]),
            "outer_steps": int(rep["outer_steps"]), "inner_attempts": int(rep["inner_attempts"]),
            "solution": _vals(solution), "history": history, "rhs": [_vals(r["rhs"]) for r in inner],
            "updates": [bool(r["applied"]) for r in inner], "inner_history": [_gmres_obj(r) for r in inner]}


def _empty_ir(n):
    """IrResult(n) as constructed (the reference keeps it beside a construction-only record)."""
    return {"status": "invalid_input", "converged": False, "outer_steps": 0, "inner_attempts": 0,
            "solution": [], "history": [], "rhs": [], "updates": [], "inner_history": []}


def _construction(h, status):
    """SpaiResult (include/bspai/spai.hpp:57-66) of a recorded build."""
    n = h.n
    aptr, aidx, aval = h._csr.ptr, h._csr.idx, h._csr.val
    cols = h.columns()
    d = cols["scaling"]
    log = h.fit_log()
    # B = A^T D: B(i, j) = A(j, i) d_j.
    b_entries = [(int(aidx[t]), j, float(aval[t]) * float(d[j])) for j in range(n) for t in range(aptr[j], aptr[j + 1])]
    n_entries, columns = [], []
    for k in range(n):
        pattern, coef = h.column(k)
        n_entries += [(int(j), k, float(c)) for j, c in zip(pattern, coef) if c != 0]
        fits = []
        for f in log.get(k, []):
            scored = "candidates" in f
            fits.append({"J": f["J"], "I": f["I"], "coefficients": _vals(f["coefficients"]),
                         "candidates": f["candidates"] if scored else [],
                         "scores": _vals(f["scores"]) if scored else [],
                         "selected": f.get("selected", []),
                         "residual": _hex(f["residual"]), "full_residual": _hex(f["residual"]),
                         "mean_score": _hex(f["mean_score"] if scored else 0.0),
                         "pivot_ratio": _hex(f["pivot_ratio"])})
        columns.append({"status": spai_status_name(int(cols["status"][k])), "pattern": [int(j) for j in pattern],
                        "coefficients": _vals(coef), "history": fits})
    p = h.preconditioner()
    return {"status": spai_status_name(status), "scaling": _vals(d), "B": _csr(*_from_entries(n, b_entries)),
            "N": _csr(*_from_entries(n, n_entries)), "P": _csr(*p), "columns": columns}


def _head(name, a, b, eps, alpha, beta):
    return {"schema": 2, "case": name, "A": _csr(*a), "b": _vals(b), "epsilon": _hex(eps), "alpha": int(alpha),
            "beta": int(beta)}


def _status_line(name, family, expected, actual):
    return {"schema": 2, "case": name, "family": family, "expected_status": expected, "actual_status": actual}


def cases():
    """The snapshot records (dicts), in the reference's case order."""
    out = []
    a = _dense([[4, 1, 0], [2, 5, 1], [0, 1, 3]])
    ident = _identity(3)
    b = np.array([2.0, -5.0, 7.0])
    general = np.array([0.1, -0.7, 1.3])
    xref = np.array([1.0, -2.0, 3.0])

    # GMRES with a fixed identity preconditioner (tolerance 1e-8, cap n).
    with Handle(a, "f64") as h:
        h.set_preconditioner(ident)
        h.record()
        h.gmres(general, 1e-8, 0)
        rec = h.recorded()
        item = _head("gmres_identity_nonsymmetric", a, general, 1e-12, 2, 8)
        item["fixed_P"] = _csr(*ident)
        item["gmres"] = _gmres_obj(rec["inner"][0])
        out.append(item)

    # Direct construction (epsilon 1e-12, alpha 2, beta 8).
    with Handle(a, "f64") as h:
        h.record()
        rep = h.build(options("f64", epsilon=1e-12, alpha=2, beta=8))
        item = _head("spai_direct_full", a, b, 1e-12, 2, 8)
        item["construction"] = _construction(h, rep["spai_status"])
        item["ir"] = _empty_ir(3)
        out.append(item)

    # SPAI-GMRES-IR (epsilon 0.3, alpha 2, beta 8, tau 1e-8) with the reference solution.
    with Handle(a, "f64") as h:
        h.record()
        o = options("f64", epsilon=0.3, alpha=2, beta=8, tau=1e-8)
        brep = h.build(o)
        _, rep = h.solve(b, o, reference=xref)
        item = _head("spai_gmres_ir", a, b, 0.3, 2, 8)
        item["construction"] = _construction(h, brep["spai_status"])
        item["ir"] = _ir_obj(h, rep, h.recorded())
        out.append(item)

    # Refinement with the identity preconditioner: three outer steps, then an inner cap of one.
    for name, inner_cap in (("ir_identity_preconditioner_correction", 0), ("ir_inner_iteration_limit", 1)):
        with Handle(a, "f64") as h:
            h.set_preconditioner(ident)
            h.record()
            o = options("f64", epsilon=0.3, alpha=2, beta=8, tau=1e-8, outercap=3, innercap=inner_cap)
            _, rep = h.solve(b, o, reference=xref)
            item = _head(name, a, b, 0.3, 2, 8)
            item["fixed_P"] = _csr(*ident)
            item["ir"] = _ir_obj(h, rep, h.recorded())
            out.append(item)

    # Growth on the tie matrix (epsilon 1e-12, alpha 1, beta 1).
    tie = _dense([[1, 1, 1], [1, 1, 0], [1, 0, 1]])
    with Handle(tie, "f64") as h:
        h.record()
        rep = h.build(options("f64", epsilon=1e-12, alpha=1, beta=1))
        item = _head("spai_tie_growth", tie, [1.0, 0.0, 0.0], 1e-12, 1, 1)
        item["construction"] = _construction(h, rep["spai_status"])
        item["ir"] = _empty_ir(3)
        out.append(item)

    # Near-dependent 2 x 2 (delta = 2^-30; epsilon 1e-5, alpha 1, beta 1).
    delta = math.ldexp(1.0, -30)
    near = _dense([[1, 1], [1, 1 + delta]])
    with Handle(near, "f64") as h:
        h.record()
        rep = h.build(options("f64", epsilon=1e-5, alpha=1, beta=1))
        item = _head("spai_near_dependent", near, [1.0, 1 + delta], 1e-5, 1, 1)
        item["construction"] = _construction(h, rep["spai_status"])
        item["ir"] = _empty_ir(2)
        out.append(item)

    # Status-only cases.
    def build_status(m, columns=False, **kw):
        with Handle(m, "f64") as h:
            rep = h.build(options("f64", **kw))
            return rep["spai_status"], h.columns() if columns else None

    _, cols = build_status(a, True, epsilon=1e-12, alpha=0, beta=8)
    eps0 = float(cols["residual"][0])
    _, cols = build_status(a, True, epsilon=eps0, alpha=0, beta=8)
    out.append(_status_line("spai_epsilon_equal_column0", "spai", "success", spai_status_name(int(cols["status"][0]))))
    st, _ = build_status(a, epsilon=math.nextafter(eps0, 0.0), alpha=0, beta=8)
    out.append(_status_line("spai_epsilon_one_ulp_below", "spai", "iteration_limit", spai_status_name(st)))
    st, _ = build_status(a, epsilon=1e-12, alpha=2, beta=0)
    out.append(_status_line("spai_beta_zero", "spai", "no_growth", spai_status_name(st)))
    st, _ = build_status(_dense([[1, 2], [1, 2]]), epsilon=1e-12, alpha=2, beta=8)
    out.append(_status_line("spai_rank_zero_pivot", "spai", "rank_deficient", spai_status_name(st)))
    st, _ = build_status(_dense([[1e-320, 0], [0, 1]]), epsilon=1e-12, alpha=2, beta=8)
    out.append(_status_line("spai_scaling_overflow", "spai", "invalid_input", spai_status_name(st)))
    with Handle(a, "f64") as h:
        h.set_preconditioner(ident)
        _, r = h.gmres(np.zeros(3), 1e-8, 0)
        out.append(_status_line("gmres_zero_rhs", "gmres", "zero_rhs", gmres_status_name(r["status"])))
        _, r = h.gmres(b, 1e-30, 1)
        out.append(_status_line("gmres_iteration_cap", "gmres", "iteration_limit", gmres_status_name(r["status"])))
        _, rep = h.solve(np.zeros(3), options("f64", epsilon=0.3, alpha=2, beta=8, tau=1e-8, outercap=3))
        out.append(_status_line("ir_zero_rhs", "ir", "success", ir_status_name(rep["ir_status"])))
    return out


def main(argv=None):
    try:
        for item in cases():
            sys.stdout.write("RELEASE_CPU_SNAPSHOT " + json.dumps(item, separators=(",", ":")) + "\n")
    except Exception as e:  # the reference's snapshot reports failures on stderr with exit 1
        sys.stderr.write(f"RELEASE_CPU_SNAPSHOT_ERROR {e}\n")
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
