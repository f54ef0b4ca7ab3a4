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


LATTICE_INPUT = """
under Lattice[0] {
  OAx = 3.89; OBy = 3.89; OCz = 3.89;
  MinDistance = 1.5;
  under Site[0] { La = 0.0; Lb = 0.0; Lc = 0.0; MaterialID = 0; AtomicFrequency = 0.1; }
  under Site[1] { La = 0.0; Lb = 0.5; Lc = 0.5; MaterialID = 0; AtomicFrequency = 0.1; }
  under Site[2] { La = 0.5; Lb = 0.0; Lc = 0.5; MaterialID = 0; AtomicFrequency = 0.1; }
  under Site[3] { La = 0.5; Lb = 0.5; Lc = 0.0; MaterialID = 0; AtomicFrequency = 0.1; }
  under Sphere[0] { Center_x = 9.0; Center_y = 9.0; Center_z = 9.0; Radius = 9.5;
                    Side = Interior; Inclusion = Intersection; OperationOrder = 0; }
}
under Lattice[1] {
  OAx = 3.89; OBy = 3.89; OCz = 3.89;
  under Site[0] { La = 0.5; Lb = 0.0; Lc = 0.0; MaterialID = 1; AtomicFrequency = 0.12;
                  under LocalSpecies[0] { SpeciesID = 1; MolarFraction = 0.02; } }
  under Site[1] { La = 0.5; Lb = 0.5; Lc = 0.5; MaterialID = 1; AtomicFrequency = 0.12;
                  under LocalSpecies[0] { SpeciesID = 1; MolarFraction = 0.02; } }
  under Parallelepiped[0] { Px = 1.0; Py = 1.0; Pz = 1.0; Ax = 17.0; Ay = 1.0; Az = 1.0;
                            Bx = 1.0; By = 17.0; Bz = 1.0; Cx = 1.0; Cy = 1.0; Cz = 17.0;
                            Side = Interior; Inclusion = Intersection; OperationOrder = 0; }
}
under RegionalInitialCondition[0] {
  LatticeID = 1; MaterialID = 1; SiteID = 1; Tag = 3; AtomicFrequency = 0.15;
  under LocalSpecies[0] { SpeciesID = 1; MolarFraction = 0.7; }
  under Sphere[0] { Center_x = 9.0; Center_y = 9.0; Center_z = 9.0; Radius = 5.0;
                    Side = Interior; Inclusion = Intersection; OperationOrder = 0; }
}
"""


def test_host_api_lattice_setup_matches_python(tmp_path):
    """SetupLatticeVariables through the C++ host API gives the Python
    path's lattices (build_lattices with the file's regions)."""
    import a2c_gb300 as A

    src = ROOT / "tests" / "cpp" / "lattice_setup_check.cpp"
    exe = tmp_path / "lattice_setup_check"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
           "-L", str(LIB), "-la2c_gpp", f"-Wl,-rpath,{LIB}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    f = tmp_path / "input.st"
    f.write_text(LATTICE_INPUT)
    r = subprocess.run([str(exe), str(f), "2"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    out = json.loads(r.stdout.strip().splitlines()[-1])
    lats = A.build_lattices([A.lattice_from_input(str(f), k) for k in range(2)], A.regions_from_input(str(f)))
    assert len(out["lattices"]) == 2
    def seq(a):  # the check program's left-to-right sum
        t = 0.0
        for v in np.asarray(a, dtype=np.float64).ravel():
            t += float(v)
        return t

    for got, want in zip(out["lattices"], lats):
        assert got["n"] == len(want["q"])
        assert got["sum_q"] == seq(want["q"])  # same sites in the same order
        assert got["sum_tag"] == seq(want["tag"]) and got["sum_sigma"] == seq(want["sigma"])
        assert got["sum_x"] == seq(want["x"])
    assert out["lattices"][1]["sum_tag"] > 0  # the region reached lattice 1
