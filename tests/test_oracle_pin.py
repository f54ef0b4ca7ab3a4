"""The CPU oracle against the reference.

The reference ships no tests or fixtures, so parity is pinned two ways:
  * against fixtures in tests/golden produced by the reference's OWN
    hot-path sources (tests/golden/make_golden.py), checked here on every
    run; bit-exact where the C library's exp/pow/log is the one the fixtures
    were made with (x86-64 glibc), else to the finite-difference rounding
    floor;
  * live against the reference library itself (oracle/_ref) where the
    reference tree is present: bit-exact on random inputs.
"""
import platform
from pathlib import Path

import numpy as np
import pytest

import a2c_gb300 as A
from oracle import oracle as O

GOLD = Path(__file__).resolve().parent / "golden"
SAME_LIBM = platform.machine() == "x86_64"


def close(a, b, rtol):
    a, b = np.asarray(a), np.asarray(b)
    if SAME_LIBM:
        return np.array_equal(a.view(np.int64) if a.dtype == np.float64 else a,
                              b.view(np.int64) if b.dtype == np.float64 else b) or np.array_equal(a, b)
    return np.allclose(a, b, rtol=rtol, atol=0)


def test_eam_against_reference_golden():
    g = np.load(GOLD / "golden_eam.npz")
    for name in O.EAM_FUNCS:
        x = g["rho"] if name.startswith("F_") else g["r"]
        got = O.eam(name, x)
        assert close(got, g[name], 1e-10 if name.endswith("deriv") else 1e-14), name


def test_free3_against_reference_golden():
    g = np.load(GOLD / "golden_free3.npz")
    nPd, nH = int(g["nPd"]), int(g["nH"])
    pb = O.Problem(nPd, nH, coe_Pd=(0.3, 0.0, 0.02, -0.01), coe_H=(0.2, 0.01, -0.03, 0.004))
    X, xH = g["X"], g["xH"]
    off, nbr, shell, o1, i1 = O.neighbors(pb, X)
    mine = O.split_lists(nPd, nH, off, nbr)
    for name in ("PdPd", "PdH", "HPd", "HH"):  # sets equal; the reference order is a KD-tree artefact
        ro, ri = g[f"ref_{name}_off"], g[f"ref_{name}_idx"]
        mo, mi = mine[name]
        assert np.array_equal(np.diff(ro), np.diff(mo)), name
        for s in range(len(ro) - 1):
            assert np.array_equal(np.sort(ri[ro[s]:ro[s + 1]]), mi[mo[s]:mo[s + 1]]), (name, s)
    ro, ri = g["ref_HH1_off"], g["ref_HH1_idx"]
    assert np.array_equal(ro, o1)
    for s in range(nH):
        assert np.array_equal(np.sort(ri[ro[s]:ro[s + 1]]), i1[o1[s]:o1[s + 1]])
    assert np.array_equal(g["ref_PdPdnum_idx"].reshape(-1, 3), shell)
    assert int(np.diff(off).max()) == int(g["maxNeib"][0]) == int(g["maxNeib"][1])
    # objective and gradient with the reference's loop order (mode 0)
    assert np.array_equal(off, g["off"]) and np.array_equal(nbr, g["nbr"])
    f, G, rho, _ = O.evaluate(pb, X, xH, off, nbr, mode=0, threads=1)
    assert close(rho, g["rho"], 1e-14)
    assert close(np.array([f]), np.array([g["f"]]), 1e-12)
    assert close(G, g["G"], 1e-9)
    gam, fh = O.chem_potential(pb, X, xH, off, nbr, float(g["gamma_bd"]), g["gamma0"], g["full0"])
    assert np.array_equal(fh, g["full_H"])
    assert close(gam, g["gamma"], 1e-10)
    x0d, gd, fd = O.dirichlet(g["sites"], 4.0, 1 - 1e-16, xH, g["gamma"], g["full_H"])
    assert np.array_equal(x0d, g["x0_dir"]) and np.array_equal(gd, g["gamma_dir"]) and np.array_equal(fd, g["full_dir"])
    x = O.diffuse(nH, x0d, o1, i1, gd, fd, 300.0, 1e-13, 1e13, 0.23, 1e-3, 1 - 1e-16, g["xprev"])
    assert close(x, g["x_diff"], 1e-13)
    assert close(np.array(O.macro_results(x, g["sites"])), g["macro"], 1e-14)


def test_config1_golden():
    g = np.load(GOLD / "golden_config1.npz")
    nPd, nH = int(g["nPd"]), int(g["nH"])
    pb = O.Problem(nPd, nH, box=tuple(g["box"]), periodic=(1, 1, 1))
    X, xH, *_ = A.lattice_fcc(6, periodic=(1, 1, 1), pos_std=0.02, sigma=(0.1, 0.1), x_center=0.05, x_half=0.01,
                             seed=1)
    assert close(X, g["X"], 1e-15) and close(xH, g["xH"], 1e-15)
    X, xH = g["X"], g["xH"]
    off, nbr, shell, o1, i1 = O.neighbors(pb, X)
    assert np.array_equal(off, g["off"]) and np.array_equal(nbr, g["nbr"]) and np.array_equal(shell, g["shell"])
    assert np.array_equal(o1, g["hh1_off"]) and np.array_equal(i1, g["hh1"])
    f, G, rho, _ = O.evaluate(pb, X, xH, off, nbr, mode=0, threads=1)
    assert close(np.array([f]), np.array([g["f"]]), 1e-12)
    assert close(G, g["G"], 1e-9)


ref_only = pytest.mark.skipif(not O.ref_available(), reason="reference library not built (no reference tree)")


@ref_only
@pytest.mark.parametrize("seed", [21, 22])
def test_oracle_bit_exact_vs_reference_live(seed):
    rng = np.random.default_rng(seed)
    n = tuple(int(v) for v in rng.integers(2, 5, size=3))
    X, xH, surf, box, nPd, nH = A.lattice_fcc(n, periodic=(0, 0, 0), pos_std=0.05, sigma=(0.06, 0.16),
                                             x_center=0.4, x_half=0.39, seed=seed)
    coe_Pd = tuple(rng.normal(size=4) * 0.05)
    coe_H = tuple(rng.normal(size=4) * 0.05)
    pb = O.Problem(nPd, nH, T=float(rng.uniform(200, 600)), coe_Pd=coe_Pd, coe_H=coe_H)
    off, nbr, *_ = O.neighbors(pb, X)
    f0, G0, r0 = O.ref_evaluate(pb, X, xH, off, nbr)
    f1, G1, r1, _ = O.evaluate(pb, X, xH, off, nbr, mode=0, threads=1)
    assert f0 == f1 and np.array_equal(G0, G1) and np.array_equal(r0, r1)
    gamma0 = rng.normal(size=nH)
    full0 = (rng.random(nH) < 0.2).astype(np.int32)
    ga, fa = O.ref_chem_potential(pb, X, xH, off, nbr, 1.0, gamma0, full0)
    gb, fb = O.chem_potential(pb, X, xH, off, nbr, 1.0, gamma0, full0)
    assert np.array_equal(ga, gb) and np.array_equal(fa, fb)


def test_gradient_translation_invariance():
    """Free boundaries: a rigid translation leaves the energy unchanged, so
    the position gradients sum to zero (pair-symmetric neighbor lists)."""
    X, xH, surf, box, nPd, nH = A.lattice_fcc(3, periodic=(0, 0, 0), pos_std=0.03, sigma=(0.08, 0.12),
                                             x_center=0.2, x_half=0.1, seed=5)
    pb = O.Problem(nPd, nH)
    off, nbr, *_ = O.neighbors(pb, X)
    f, G, _, _ = O.evaluate(pb, X, xH, off, nbr)
    gq = G.reshape(-1, 4)[:, :3]
    assert np.abs(gq.sum(axis=0)).max() < 1e-8 * np.abs(gq).sum()


def test_neighbor_lists_symmetric_and_fd_consistent():
    """j in list(i) <=> i in list(j); the gradient agrees with a central
    difference of the objective along a random direction."""
    X, xH, surf, box, nPd, nH = A.lattice_fcc(4, periodic=(1, 1, 1), pos_std=0.03, sigma=(0.08, 0.12),
                                             x_center=0.2, x_half=0.1, seed=6)
    pb = O.Problem(nPd, nH, box=box, periodic=(1, 1, 1))
    off, nbr, *_ = O.neighbors(pb, X)
    ids = (nbr & O.ID_MASK).astype(np.int64)
    pairs = set()
    for s in range(pb.N):
        for j in ids[off[s]:off[s + 1]]:
            pairs.add((s, int(j)))
    assert all((j, i) in pairs for (i, j) in pairs)
    f, G, _, _ = O.evaluate(pb, X, xH, off, nbr)
    d = np.random.default_rng(0).normal(size=X.size) * 1e-3
    h = 1e-3
    fp, *_ = O.evaluate(pb, X + h * d, xH, off, nbr)
    fm, *_ = O.evaluate(pb, X - h * d, xH, off, nbr)
    fd = (fp - fm) / (2 * h)
    assert abs(fd - G @ d) < 1e-5 * abs(G @ d)


def test_oracle_lbfgs_converges():
    X, xH, surf, box, nPd, nH = A.lattice_fcc(2, periodic=(0, 0, 0), pos_std=0.02, sigma=(0.1, 0.1), seed=9)
    pb = O.Problem(nPd, nH)
    off, nbr, *_ = O.neighbors(pb, X)
    r = O.minimize(pb, X, xH, off, nbr, gatol=1e-6)
    assert r["reason"] == 3 and r["gnorm"] <= 1e-6
    f0, *_ = O.evaluate(pb, X, xH, off, nbr)
    assert r["fmin"] < f0


def test_device_arithmetic_close_to_reference_arithmetic():
    """The portable exp/pow/log and the GPU reduction order (the arithmetic
    the device reproduces bit for bit) stay within the plain form's 1e-11
    of the reference's arithmetic."""
    X, xH, surf, box, nPd, nH = A.lattice_fcc(6, periodic=(1, 1, 1), pos_std=0.02, sigma=(0.1, 0.1), x_center=0.05,
                                             x_half=0.01, seed=1)
    pb = O.Problem(nPd, nH, box=box, periodic=(1, 1, 1))
    off, nbr, *_ = O.neighbors(pb, X)
    f0, G0, r0, _ = O.evaluate(pb, X, xH, off, nbr)
    with O.arithmetic("device"):
        f1, G1, r1, _ = O.evaluate(pb, X, xH, off, nbr)
    assert abs(f1 - f0) <= 1e-13 * abs(f0)
    assert np.linalg.norm(G1 - G0) <= 1e-11 * np.linalg.norm(G0)
    assert np.max(np.abs(r1 - r0) / r0) < 1e-14


def test_minimizer_sensitivity_between_arithmetics():
    """L-BFGS trajectories are sensitive to last-bit differences: in the two
    arithmetics both runs converge (gatol 1e-6) to the same minimum, within
    the position uncertainty that gatol leaves on this flat landscape (a few
    1e-4 A), not to 1e-8 A.  Bit-identical trajectories need identical
    arithmetic, which the device arithmetic provides (test_gpu_fp64)."""
    X, xH, surf, box, nPd, nH = A.lattice_fcc(3, periodic=(0, 0, 0), pos_std=0.02, sigma=(0.1, 0.1), x_center=0.05,
                                             x_half=0.01, seed=1)
    pb = O.Problem(nPd, nH)
    off, nbr, *_ = O.neighbors(pb, X)
    r0 = O.minimize(pb, X, xH, off, nbr, gatol=1e-6, max_it=400)
    with O.arithmetic("device"):
        r1 = O.minimize(pb, X, xH, off, nbr, gatol=1e-6, max_it=400)
    assert r0["reason"] == 3 and r1["reason"] == 3
    assert np.abs(r1["X"] - r0["X"]).max() < 2e-3
    assert abs(r1["fmin"] - r0["fmin"]) < 1e-9 * abs(r0["fmin"])


def test_batch_reduction_order_changes_only_rounding():
    """The batched-instance reduction order (partials of 2048 consecutive
    terms per instance) leaves the per-site arithmetic alone -- the
    gradient is identical -- and moves the objective by rounding only."""
    X, xH, surf, box, nPd, nH = A.lattice_fcc(8, periodic=(1, 1, 1), pos_std=0.02, sigma=(0.1, 0.1), x_center=0.3,
                                             x_half=0.02, seed=3)
    pb = O.Problem(nPd, nH, box=box, periodic=(1, 1, 1), T=450.0)
    off, nbr, *_ = O.neighbors(pb, X)  # 4096 sites: two site chunks, eight element chunks
    with O.arithmetic("device"):
        f1, G1, *_ = O.evaluate(pb, X, xH, off, nbr)
        with O.reduction("batch"):
            f2, G2, *_ = O.evaluate(pb, X, xH, off, nbr)
            f3, G3, *_ = O.evaluate(pb, X, xH, off, nbr, threads=1)
    assert np.array_equal(G1, G2)
    assert abs(f2 - f1) <= 1e-14 * abs(f1)
    assert f3 == f2 and np.array_equal(G3, G2)  # independent of the thread count
    assert O.olib().orc_get_reduction() == 0
