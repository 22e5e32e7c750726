"""Regenerate tests/golden/*.npz from the reference's own CPU solvers.

Needs the reference tree (only present where fixtures are regenerated, never on the GPU machine):
    make -C oracle ref REF=<reference tree>   # compiles golden_gen.cpp against its src/*.cpp
    python tests/golden/make_golden.py
Each fixture stores the inputs' generator parameters plus the reference's outputs (statuses,
patterns, exact binary64 values), so the oracle and the GPU path can be pinned to them.
"""
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "spai-gmres-ir_gb300"))
from spai_ir import matrices as M  # noqa: E402

GEN = os.path.join(ROOT, "oracle", "_ref", "golden_gen")
OUT = os.path.dirname(os.path.abspath(__file__))


def band(n, diagonal):
    """Banded family of tests/test_cuda_spai_sparse.cpp:7 (scale 2^(i%5-2))."""
    rows, cols, vals = [], [], []
    for i in range(n):
        scale = 2.0 ** ((i % 5) - 2)
        rows.append(i); cols.append(i); vals.append(diagonal * scale)
        if i:
            rows.append(i); cols.append(i - 1); vals.append(2 * scale)
        if i + 1 < n:
            rows.append(i); cols.append(i + 1); vals.append(scale)
    return (n,) + M._canonical(n, np.array(rows), np.array(cols), np.array(vals))


CASES = {
    "tiny": lambda: M.from_dense([[4, 1, 0], [2, 5, 1], [0, 1, 3]]),
    "band16_8": lambda: band(16, 8.0), "band64_8": lambda: band(64, 8.0),
    "band256_8": lambda: band(256, 8.0), "band1024_8": lambda: band(1024, 8.0),
    "band16_5": lambda: band(16, 5.0), "band64_5": lambda: band(64, 5.0),
    "band256_5": lambda: band(256, 5.0), "band1024_5": lambda: band(1024, 5.0),
    "cd2d_32": lambda: M.convection_diffusion_2d(32),
    "cd2d_64": lambda: M.convection_diffusion_2d(64),  # the FP64 drop-in configuration
    "cd3d_12": lambda: M.convection_diffusion_3d(12),
    "irregular_3000": lambda: M.irregular(3000, seed=7),
    "aniso_24": lambda: M.anisotropic_diffusion(24, seed=3),
}


class Reader:
    def __init__(self, data):
        self.d, self.o = data, 0

    def i64(self):
        v = struct.unpack_from("<q", self.d, self.o)[0]
        self.o += 8
        return v

    def f64(self):
        v = struct.unpack_from("<d", self.d, self.o)[0]
        self.o += 8
        return v

    def vi(self):
        n = self.i64()
        v = np.frombuffer(self.d, "<i8", n, self.o).copy()
        self.o += 8 * n
        return v

    def vf(self):
        n = self.i64()
        v = np.frombuffer(self.d, "<f8", n, self.o).copy()
        self.o += 8 * n
        return v


def run(args):
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "out.bin")
        subprocess.run([GEN] + [str(a) for a in args] + [out], check=True)
        return Reader(open(out, "rb").read())


def spai(mtx, n, eps, alpha, beta):
    r = run(["spai", mtx, eps, alpha, beta])
    d = dict(status=r.i64())
    assert r.i64() == n
    d["scaling"] = r.vf()
    cs, fits, gr, cl, res, qsz, pats, coefs = [], [], [], [], [], [], [], []
    for _ in range(n):
        cs.append(r.i64()); fits.append(r.i64()); gr.append(r.i64()); cl.append(r.i64())
        res.append(r.f64())
        p, c = r.vi(), r.vf()
        qsz.append(len(p)); pats.append(p); coefs.append(c)
    d.update(col_status=np.array(cs), fits=np.array(fits), growths=np.array(gr), clamps=np.array(cl),
             residual=np.array(res), qsize=np.array(qsz),
             pattern=np.concatenate(pats) if pats else np.zeros(0, np.int64),
             coefficients=np.concatenate(coefs) if coefs else np.zeros(0))
    d["p_ptr"], d["p_idx"], d["p_val"] = r.vi(), r.vi(), r.vf()
    return d


def ir(mode, mtx, eps, alpha, beta, tau, inner, outer):
    r = run([mode, mtx, eps, alpha, beta, tau, inner, outer])
    return dict(status=r.i64(), converged=r.i64(), outer_steps=r.i64(), nnz_p=r.i64(),
                inner_iterations=r.i64(), nbe=r.f64(), residual_inf=r.f64(), x=r.vf())


def main():
    if not os.path.exists(GEN):
        sys.exit("build the reference generator first: make -C oracle ref")
    for name, make in CASES.items():
        system = make()
        n = system[0]
        with tempfile.TemporaryDirectory() as tmp:
            mtx = os.path.join(tmp, "a.mtx")
            M.write_matrix_market(mtx, system)
            fixture = {"n": n, "a_ptr": system[1], "a_idx": system[2], "a_val": system[3]}
            alpha = (n + 7) // 8
            if name == "tiny":
                for key, (eps, al) in {"exact": (1e-12, 2), "cap1": (1e-12, 1), "cap0": (1e-12, 0)}.items():
                    for k, v in spai(mtx, n, eps, al, 8).items():
                        fixture[f"spai_{key}_{k}"] = v
                spai_args = (0.3, 2, 8)
            else:
                spai_args = (0.3, alpha, 8)
            for k, v in spai(mtx, n, *spai_args).items():
                fixture[f"spai_{k}"] = v
            fixture["spai_args"] = np.array(spai_args, np.float64)
            ir_args = (0.3, spai_args[1], 8, 1e-8, 0, 20)
            for k, v in ir("ir", mtx, *ir_args).items():
                fixture[f"ir64_{k}"] = v
            ir32_args = (0.3, spai_args[1], 8, 1e-4, 0, 20)
            for k, v in ir("ir32", mtx, *ir32_args).items():
                fixture[f"ir32_{k}"] = v
            fixture["ir_args"] = np.array(ir_args, np.float64)
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **fixture)
        print(name, n, "spai", int(fixture["spai_status"]), "ir64", int(fixture["ir64_status"]),
              int(fixture["ir64_outer_steps"]), "ir32", int(fixture["ir32_status"]))


if __name__ == "__main__":
    main()
