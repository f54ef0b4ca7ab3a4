"""The snapshot writers against the reference's own: Output.cpp (VTP with
its PVD collection, extended XYZ), compiled unmodified under oracle/_ref
with single-rank shims for IoData, MPI and the generated version header
(`make -C oracle out`).  The library's files must equal the reference's
byte for byte: every precision, both formats, several frames appended to
one collection, named and unnamed materials.  Skipped where the reference
tree is absent (the library alone is then tested by test_snapshot_io.py)."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import a2c_gb300 as A

REF_OUT = Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "libout_ref.so"
pytestmark = pytest.mark.skipif(not REF_OUT.exists(), reason="reference snapshot writer not built (no reference tree)")

P, D, I = C.c_void_p, C.c_double, C.c_int


def ref_lib():
    L = C.CDLL(str(REF_OUT))
    L.ref_output_write.argtypes = [C.c_char_p, C.c_char_p, I, I, I, P, P, P, P, P, P, I, P, P, P, P, P, P, I, P, I, P]
    L.ref_output_write.restype = I
    return L


def ptr(a):
    return a.ctypes.data


def sites(n=18, seed=3):
    rng = np.random.default_rng(seed)
    q0 = rng.uniform(-5.0, 25.0, size=(n, 3))
    return {"q": q0 + rng.normal(scale=0.05, size=(n, 3)), "q0": q0, "l": np.zeros((n, 3)),
            "siteid": rng.integers(0, 8, n).astype(np.int32), "matid": (np.arange(n) % 3 == 2).astype(np.int32),
            "tag": rng.integers(0, 2, n).astype(np.int32), "sigma": rng.uniform(0.05, 0.15, n),
            "x": rng.uniform(0.0, 1.0, n)}


def write_ref(tmp, base, s, gamma, names, precision, fmt, times, axes, origin, periodic):
    n = len(s["q"])
    nx = np.ones(n, dtype=np.int32)
    cn = (C.c_char_p * len(names))(*[m.encode() for m in names])
    arr = {k: np.ascontiguousarray(v) for k, v in s.items()}
    ax, org, per = (np.ascontiguousarray(v, dtype=t) for v, t in ((axes, np.float64), (origin, np.float64),
                                                                  (periodic, np.int32)))
    tm = np.ascontiguousarray(times, dtype=np.float64)
    g = np.ascontiguousarray(gamma, dtype=np.float64)
    rc = ref_lib().ref_output_write(f"{tmp}/".encode(), base.encode(), precision, fmt, n, ptr(arr["q"]),
                                    ptr(arr["q0"]), ptr(arr["sigma"]), ptr(arr["siteid"]), ptr(arr["matid"]),
                                    ptr(arr["tag"]), 1, ptr(nx), ptr(arr["x"]), ptr(g), ptr(ax), ptr(org), ptr(per),
                                    len(names), cn, len(tm), ptr(tm))
    assert rc == 0


@pytest.mark.parametrize("precision", [0, 1, 2])
@pytest.mark.parametrize("names", [["Pd", "H"], ["", "H2"]])
def test_lattice_snapshots_equal_reference(tmp_path, precision, names):
    s = sites()
    gamma = np.linspace(-3.0, 2.0, len(s["q"]))
    axes = (3.89, 0.0, 0.0, 0.0, 3.89, 0.0, 0.1, 0.0, 3.89)
    origin, periodic, times = (0.5, -1.0, 2.0), (1, 1, 0), (0.0, 1.5e-12, 3.0e-12)
    ref, ours = tmp_path / "ref", tmp_path / "ours"
    ref.mkdir()
    ours.mkdir()
    write_ref(ref, "sol", s, gamma, names, precision, 2, times, axes, origin, periodic)
    d = A.snapshot_desc(str(ours / "sol"), fmt="both", precision=precision, origin=origin, periodic=periodic)
    for k in range(9):
        d.axes[k] = axes[k]
    A.snapshot_begin(d)
    for f, t in enumerate(times):
        A.snapshot_write_lattice(d, f, t, s, gamma=gamma, material_names=names)
    want = sorted(p.name for p in ref.iterdir())
    assert want == sorted(p.name for p in ours.iterdir())
    assert "sol_L0.pvd" in want and "sol_L0_0002.xyz" in want
    for name in want:
        assert (ours / name).read_bytes() == (ref / name).read_bytes(), name


@pytest.mark.parametrize("precision", [0, 2])
def test_evaluator_snapshot_equals_reference(tmp_path, precision):
    """The evaluator's layout (Pd sites then H sites, material 0 "Pd" with
    occupancy 1 and chemical potential 0, material 1 "H")."""
    nPd, nH = 8, 8
    n = nPd + nH
    rng = np.random.default_rng(7)
    X0 = np.c_[rng.uniform(0, 8, (n, 3)), np.full(n, 0.1)].reshape(-1)
    X = X0 + np.c_[rng.normal(scale=0.02, size=(n, 3)), rng.normal(scale=0.01, size=n)].reshape(-1)
    xH = rng.uniform(0.0, 1.0, nH)
    gam = rng.normal(size=nH)
    sid = (np.arange(n) % 4).astype(np.int8)
    tag = (np.arange(n) % 3).astype(np.int8)
    box = (7.78, 7.78, 11.67)
    s = {"q": X.reshape(-1, 4)[:, :3].copy(), "q0": X0.reshape(-1, 4)[:, :3].copy(), "l": np.zeros((n, 3)),
         "siteid": sid.astype(np.int32), "matid": np.r_[np.zeros(nPd), np.ones(nH)].astype(np.int32),
         "tag": tag.astype(np.int32), "sigma": X.reshape(-1, 4)[:, 3].copy(), "x": np.r_[np.ones(nPd), xH]}
    axes = (box[0], 0, 0, 0, box[1], 0, 0, 0, box[2])
    ref, ours = tmp_path / "ref", tmp_path / "ours"
    ref.mkdir()
    ours.mkdir()
    write_ref(ref, "ev", s, np.r_[np.zeros(nPd), gam], ["Pd", "H"], precision, 2, (0.0, 2e-12), axes, (0, 0, 0),
              (1, 1, 0))
    d = A.snapshot_desc(str(ours / "ev"), fmt="both", precision=precision, box=box, periodic=(1, 1, 0))
    A.snapshot_begin(d)
    for f, t in enumerate((0.0, 2e-12)):
        A.snapshot_write(d, f, t, nPd, nH, X, xH, X0=X0, gamma=gam, siteid=sid, tag=tag)
    for name in sorted(p.name for p in ref.iterdir()):
        assert (ours / name).read_bytes() == (ref / name).read_bytes(), name
