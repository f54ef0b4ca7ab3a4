"""The device-resident DMD outer loop (a2c_gpp_dmd_run) against the same
loop orchestrated from the oracle.  FP64 plain form vs the oracle in the
device arithmetic: positions, widths, occupancies, chemical potentials and
full_H bit for bit after several outer steps (macro results to 1e-14, their
sums being ordered differently).  Mixed precision: the DMD trajectory is
sensitive to last-bit differences inside each minimization (two FP64 runs
whose exp/pow/log differ by an ulp drift 2.4e-3 apart in H content after one
outer step at gatol 1e-5), so the mixed run is held to a small multiple of
that measured FP64-vs-FP64 spread, not to a fixed 1e-6."""
import numpy as np
import pytest

import a2c_gb300 as A
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DMD = dict(dt=1e-12, nu=1e13, Qm=0.23, x_bd=0.80, xLb=1e-3, xUb=1 - 1e-16)


def slab():
    """Periodic in x, y; free surfaces in z; H on the z = 0 layer held at 0.8."""
    X, xH, surf, box, nPd, nH = A.lattice_fcc((4, 4, 5), periodic=(1, 1, 0), pos_std=0.02, sigma=(0.1, 0.1),
                                             x_center=0.01, x_half=0.0, seed=5)
    bd = np.nonzero(surf)[0].astype(np.int32)
    return X, xH, bd, box, nPd, nH


def test_dmd_fp64_bit_exact_vs_oracle(gpu):
    X, xH, bd, box, nPd, nH = slab()
    per = (1, 1, 0)
    pb = O.Problem(nPd, nH, T=400.0, box=box, periodic=per)
    off, nbr, shell, o1, i1 = O.neighbors(pb, X)
    gamma0 = np.zeros(nH)
    full0 = np.zeros(nH, dtype=np.int32)
    gbd = 2.0
    kw = dict(gatol=1e-5, max_it=300)
    with O.arithmetic("device"):
        ref = O.dmd_run(pb, X, xH, gamma0, full0, off, nbr, o1, i1, bd, bd, 3, gamma_bd=gbd, **DMD, **kw)
    with A.Gpp(nPd, nH, T=400.0, box=box, periodic=per) as g:
        g.set_occupancy(xH)
        g.build_neighbors(X)
        out = g.dmd_run(X, xH, gamma0, full0, bd, bd, 3, gamma_bd=gbd, **DMD, **kw)
    print("iters", out["iters"], ref["iters"], "xH", out["xH_mean"], ref["xH_mean"])
    assert np.array_equal(out["iters"], ref["iters"])
    for k in ("X", "xH", "gamma", "full_H", "fmin"):
        assert np.array_equal(out[k], ref[k]), k
    assert np.allclose(out["xH_mean"], ref["xH_mean"], rtol=1e-14, atol=0)
    assert np.allclose(out["xH_interior"], ref["xH_interior"], rtol=1e-14, atol=0)
    assert out["xH_mean"][-1] > out["xH_mean"][0]  # hydrogen enters through the held surface


def test_dmd_fp64_neighbor_update_bit_exact(gpu):
    """Lists re-derived every outer step (skin refilter on the device, a
    full build in the oracle): still bit for bit."""
    X, xH, bd, box, nPd, nH = slab()
    per = (1, 1, 0)
    pb = O.Problem(nPd, nH, T=400.0, box=box, periodic=per)
    off, nbr, shell, o1, i1 = O.neighbors(pb, X)
    gamma0 = np.zeros(nH)
    full0 = np.zeros(nH, dtype=np.int32)
    kw = dict(gatol=1e-5, max_it=300)
    with O.arithmetic("device"):
        ref = O.dmd_run(pb, X, xH, gamma0, full0, off, nbr, o1, i1, bd, bd, 3, gamma_bd=2.0, neighbor_update=True,
                        **DMD, **kw)
    with A.Gpp(nPd, nH, T=400.0, box=box, periodic=per) as g:
        g.set_occupancy(xH)
        g.set_neighbor_skin(0.5)
        g.update_neighbors(X)
        out = g.dmd_run(X, xH, gamma0, full0, bd, bd, 3, gamma_bd=2.0, neighbor_update=True, **DMD, **kw)
    assert np.array_equal(out["iters"], ref["iters"])
    for k in ("X", "xH", "gamma", "full_H", "fmin"):
        assert np.array_equal(out[k], ref[k]), k


def test_dmd_mixed_follows_fp64(gpu):
    X, xH, bd, box, nPd, nH = slab()
    per = (1, 1, 0)
    gamma0 = np.zeros(nH)
    full0 = np.zeros(nH, dtype=np.int32)
    kw = dict(gatol=1e-5, max_it=300)
    steps = 3
    res = {}
    for prec in ("fp64", "mixed"):
        with A.Gpp(nPd, nH, T=400.0, box=box, periodic=per, precision=prec) as g:
            g.set_occupancy(xH)
            g.build_neighbors(X)
            res[prec] = g.dmd_run(X, xH, gamma0, full0, bd, bd, steps, gamma_bd=2.0, **DMD, **kw)
    # the same FP64 loop in the reference's own arithmetic (glibc exp/pow/log)
    pb = O.Problem(nPd, nH, T=400.0, box=box, periodic=per)
    off, nbr, shell, o1, i1 = O.neighbors(pb, X)
    res["ref"] = O.dmd_run(pb, X, xH, gamma0, full0, off, nbr, o1, i1, bd, bd, steps, gamma_bd=2.0, **DMD, **kw)
    base = res["fp64"]["xH_mean"]
    d_mixed = np.abs(res["mixed"]["xH_mean"] - base) / base
    d_fp64 = np.abs(res["ref"]["xH_mean"] - base) / base
    x_mixed = np.abs(res["mixed"]["xH"] - res["fp64"]["xH"]).max()
    x_fp64 = np.abs(res["ref"]["xH"] - res["fp64"]["xH"]).max()
    print("H content fp64", base, "mixed", res["mixed"]["xH_mean"], "rel", d_mixed, "fp64 spread", d_fp64,
          "max dx", x_mixed, x_fp64)
    assert d_fp64.max() > 0  # the spread is real, not a rerun of the same arithmetic
    assert d_mixed.max() <= 4 * d_fp64.max() + 1e-4
    assert x_mixed <= 4 * x_fp64 + 1e-4
    assert res["mixed"]["xH_mean"][-1] > res["mixed"]["xH_mean"][0]


@pytest.mark.parametrize("prec,minimizer", [("mixed", "default"), ("fp64", "device")])
def test_dmd_graph_equals_host_steps(gpu, prec, minimizer):
    """Steps 2..n of a DMD run as one CUDA graph (a device loop over outer
    steps, each a device loop over L-BFGS ticks, then the chemical
    potential, the Dirichlet condition, the diffusion step and the macro
    results) give the host-sequenced loop's results bit for bit."""
    X, xH, bd, box, nPd, nH = slab()
    per = (1, 1, 0)
    gamma0 = np.zeros(nH)
    full0 = np.zeros(nH, dtype=np.int32)
    kw = dict(gatol=1e-5, max_it=300)
    res = {}
    for host_steps in (True, False):
        with A.Gpp(nPd, nH, T=400.0, box=box, periodic=per, precision=prec) as g:
            g.set_occupancy(xH)
            g.build_neighbors(X)
            g.set_minimizer(minimizer)
            res[host_steps] = g.dmd_run(X, xH, gamma0, full0, bd, bd, 4, gamma_bd=2.0, host_steps=host_steps, **DMD,
                                        **kw)
    a, b = res[True], res[False]
    print("iters", a["iters"], b["iters"], "xH", a["xH_mean"], b["xH_mean"])
    for k in ("X", "xH", "gamma", "full_H", "fmin", "iters", "xH_mean", "xH_interior"):
        assert np.array_equal(a[k], b[k]), k
    assert a["xH_mean"][-1] > a["xH_mean"][0]
