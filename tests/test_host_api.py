"""The reference-named C++ host API (include/a2c_host.hpp): it compiles
against the C ABI alone, and on a GPU one DMD outer step through it gives
the C-ABI path's numbers."""
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "host_api_check.cpp"
LIB = ROOT / "a2c_gb300" / "_lib"


def compile_check(out: Path) -> None:
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", str(ROOT / "include"), str(SRC), "-o", str(out),
           "-L", str(LIB), "-la2c_gpp", f"-Wl,-rpath,{LIB}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_host_api_compiles_and_links(tmp_path):
    compile_check(tmp_path / "host_api_check")


@pytest.mark.gpu
def test_host_api_dmd_step_matches_c_abi(gpu, tmp_path):
    import a2c_gb300 as A

    exe = tmp_path / "host_api_check"
    compile_check(exe)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["status"] == 0 and out["restart_round_trip"] is True
    # the same step through the Python view of the C ABI
    X, xH, surf, box, nPd, nH = A.lattice_fcc(4, periodic=(1, 1, 0), pos_std=0.02, sigma=(0.1, 0.1), x_center=0.05,
                                             x_half=0.01, seed=11)
    with A.Gpp(nPd, nH, box=box, periodic=(1, 1, 0)) as g:
        g.set_occupancy(xH)
        g.build_neighbors(X)
        f0, _ = g.eval(X)
        res = g.minimize(X, gatol=1e-6)
    assert out["f0"] == f0
    assert out["fmin"] == res.fmin and out["iters"] == res.iters
