"""Host-side checks that need no GPU: the C ABI library loads and exports every declared symbol,
the host build of the device hypot agrees with the oracle, the drop-in CLIs' input-error exit
codes (tests/check_solver_cli.py cases that fail before any device work), the seeded generators,
and the replica reduction of bench.py over a world_size-2 gloo group."""
import os
import re
import subprocess

import numpy as np
import pytest

import oracle as O
import spai_ir
from conftest import ROOT
from spai_ir import matrices as M

TINY_MTX = """%%MatrixMarket matrix coordinate real general
% A*[1,-2,3]' = [2,-5,7]'
3 3 7
1 1 4
1 2 1
2 1 2
2 2 5
2 3 1
3 2 1
3 3 3
"""


def declared_functions():
    text = open(os.path.join(ROOT, "include", "spai_ir.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b([a-z_]+)\s*\([^;{]*\)\s*;", text)) - {"if", "while"})


def test_library_exports_every_declared_symbol(built):
    lib = spai_ir.lib()
    names = declared_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) <= set(spai_ir.SIGNATURES), set(names) - set(spai_ir.SIGNATURES)


def test_status_names_match_reference(built):
    lib = spai_ir.lib()
    for i, s in enumerate(spai_ir.SPAI_STATUS):
        assert lib.spai_status_name(i).decode() == s
    for i, s in enumerate(spai_ir.GMRES_STATUS):
        assert lib.gmres_status_name(i).decode() == s
    for i, s in enumerate(spai_ir.IR_STATUS):
        assert lib.ir_status_name(i).decode() == s


def test_device_hypot_host_build_matches_oracle(built):
    rng = np.random.default_rng(11)
    ex = rng.integers(-300, 300, 40000)
    x = rng.uniform(1, 2, ex.size) * np.exp2(ex)
    y = rng.uniform(1, 2, ex.size) * np.exp2(ex + rng.integers(-40, 40, ex.size))
    for a, b in zip(x.tolist(), y.tolist()):
        assert spai_ir.hypot(a, b) == O.hypot(a, b)
    xf = (rng.uniform(-3, 3, 40000) * np.exp2(rng.integers(-60, 60, 40000))).astype(np.float32)
    yf = (rng.uniform(-3, 3, 40000) * np.exp2(rng.integers(-60, 60, 40000))).astype(np.float32)
    for a, b in zip(xf.tolist(), yf.tolist()):
        assert spai_ir.hypotf(a, b) == O.hypotf(a, b)


@pytest.mark.parametrize("cli", ["gpu_fp64_ir", "gpu_fp32_ir", "gpu_mixed_ir", "gpu_diag_ir"])
def test_cli_input_errors(built, tmp_path, cli):
    exe = spai_ir.cli_path(cli)
    mtx = tmp_path / "tiny.mtx"
    mtx.write_text(TINY_MTX)

    def rc(*args):
        return subprocess.run([exe, *map(str, args)], capture_output=True, text=True, timeout=60).returncode

    assert rc() == 2
    assert rc(mtx, "nan") == 2
    assert rc(mtx, ".5", "21") == 2
    assert rc(mtx, ".5", "20", "4") == 2
    assert rc(mtx, ".5", "-1") == 2
    assert rc(mtx, "0") == 2
    assert rc(mtx, "1e400") == 2
    assert rc(tmp_path / "missing.mtx") == 2
    bad = tmp_path / "bad.mtx"
    bad.write_text("%%MatrixMarket matrix array real general\n3 3\n")
    assert rc(bad) == 1  # unsupported format: runtime_error -> solver error exit 1
    nonsq = tmp_path / "nonsq.mtx"
    nonsq.write_text("%%MatrixMarket matrix coordinate real general\n2 3 1\n1 1 1\n")
    assert rc(nonsq) == 2


def test_generators():
    n, ptr, idx, val = M.convection_diffusion_2d(64)
    assert n == 4096 and len(val) == 5 * n - 4 * 64
    n, ptr, idx, val = M.convection_diffusion_3d(20)
    assert len(val) == 7 * n - 6 * 20 * 20
    for system in (M.convection_diffusion_2d(9, 7, (0.3, -0.9), 25.0), M.irregular(5000, seed=2),
                   M.anisotropic_diffusion(16, seed=1)):
        n, ptr, idx, val = system
        assert ptr[0] == 0 and ptr[-1] == len(idx) and np.all(np.diff(ptr) >= 1)
        for r in range(0, n, max(1, n // 50)):
            row = idx[ptr[r]:ptr[r + 1]]
            assert np.all(np.diff(row) > 0) and r in row
        assert np.all(val != 0) and np.all(np.isfinite(val))
    n, ptr, idx, val = M.irregular(200000, seed=5)
    assert 11.0 < len(val) / n - 1 < 14.0  # Zipf(1.5) on [1,256]: mean ~12.3 off-diagonals
    d = M.dense(M.anisotropic_diffusion(12, seed=4))
    assert np.allclose(d, d.T) and np.all(np.linalg.eigvalsh(d) > 0)


def _replica_worker(rank, world, port, out):
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    out[rank] = bench.max_over_ranks(10.0 + rank, world)
    dist.destroy_process_group()


def test_bench_replica_max_over_ranks_gloo():
    import multiprocessing as mp
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        ps = [ctx.Process(target=_replica_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in ps:
            p.start()
        for p in ps:
            p.join(120)
        assert all(p.exitcode == 0 for p in ps)
        assert out[0] == out[1] == 11.0
