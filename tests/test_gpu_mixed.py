"""Mixed-precision form (FP32 pair quadrature, compensated per-site sums,
FP64 finish and reductions) against the FP64 oracle.

Stated bounds: free entropy within 1e-6 relative of the FP64 oracle; the
gradient within 1e-4 in the 2-norm relative (FP32 rounding of terms that
cancel in the net per-site force); densities-derived quantities are checked
through the objective.  Every threads-per-site mapping gives the same
result to FP32 rounding.
"""
import numpy as np
import pytest

import a2c_gb300 as A
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL_F = 1e-6
TOL_G = 1e-4

CASES = {
    "free3": ((3, 3, 3), (0, 0, 0), 0.02, (0.10, 0.10), 0.05, 0.01, 1),
    "config1_6cube": ((6, 6, 6), (1, 1, 1), 0.02, (0.10, 0.10), 0.05, 0.01, 1),
    "slab_4x5x6": ((4, 5, 6), (1, 1, 0), 0.03, (0.08, 0.14), 0.15, 0.15, 7),
    "config2_16cube": ((16, 16, 16), (1, 1, 1), 0.03, (0.08, 0.14), 0.15, 0.15, 2),
}


def make(case):
    ncell, per, ps, sg, xc, xh, seed = CASES[case]
    X, xH, surf, box, nPd, nH = A.lattice_fcc(ncell, periodic=per, pos_std=ps, sigma=sg, x_center=xc, x_half=xh,
                                             seed=seed)
    return X, xH, box, per, nPd, nH, O.Problem(nPd, nH, box=box, periodic=per)


@pytest.mark.parametrize("case", list(CASES))
def test_mixed_objective_gradient(gpu, case):
    X, xH, box, per, nPd, nH, pb = make(case)
    off, nbr, *_ = O.neighbors(pb, X)
    f_ref, G_ref, _, _ = O.evaluate(pb, X, xH, off, nbr, mode=1)
    with A.Gpp(nPd, nH, box=box, periodic=per, precision="mixed") as g:
        g.set_occupancy(xH)
        g.build_neighbors(X)
        res = {}
        for tps in (1, 2, 4, 8):
            g.set_threads_per_site(tps)
            res[tps] = g.eval(X)
    for tps, (f, G) in res.items():
        rel_f = abs(f - f_ref) / abs(f_ref)
        rel_g = np.linalg.norm(G - G_ref) / np.linalg.norm(G_ref)
        print(f"{case} tps={tps}: rel_f={rel_f:.3e} rel_G={rel_g:.3e}")
        assert rel_f < TOL_F
        assert rel_g < TOL_G


def test_mixed_minimize_close_to_fp64(gpu):
    """Mixed-precision L-BFGS (FP32 evaluator, FP64 vector algebra) reaches
    the FP64 minimum.  Without polish it stops at the mixed gradient's noise
    floor; with polish (the default) it finishes with FP64 evaluations to
    gatol.  Bounds: free entropy within 1e-6 relative of the FP64 minimum;
    positions of the polished result within 1e-4 A, or within 3x the
    distance between two FP64 minimizations of the same problem that differ
    only in their summation order (host-driven vs device engine) when gatol
    determines the minimum less well than that; positions of the unpolished
    result within 1e-3 A (it stops at the mixed gradient's floor, ~5e-6)."""
    X, xH, box, per, nPd, nH, pb = make("config1_6cube")
    kw = dict(m=5, max_it=2000, gatol=1e-6)
    with A.Gpp(nPd, nH, box=box, periodic=per) as g:
        g.set_occupancy(xH)
        g.build_neighbors(X)
        r64 = g.minimize(X, **kw)
        g.set_minimizer("device")
        r64e = g.minimize(X, **kw)
        g.set_minimizer("default")
        g.set_precision("mixed")
        rmx = g.minimize(X, **kw)
        rraw = g.minimize(X, **dict(kw, polish=0))
        g.set_precision("fp64")
        f_at_mixed, G_at_mixed = g.eval(rmx.X)
        f_at_raw, _ = g.eval(rraw.X)
    dq = np.abs(rmx.X.reshape(-1, 4)[:, :3] - r64.X.reshape(-1, 4)[:, :3]).max()
    dq_raw = np.abs(rraw.X.reshape(-1, 4)[:, :3] - r64.X.reshape(-1, 4)[:, :3]).max()
    print(f"fp64: it={r64.iters} f={r64.fmin:.12e} reason={r64.reason}; mixed+polish: it={rmx.iters} "
          f"(mixed {rmx.mixed_iters}, fp64 {rmx.fp64_iters}, mixed |g| {rmx.mixed_gnorm:.2e}) reason={rmx.reason} "
          f"max|dq|={dq:.2e}; mixed only: it={rraw.iters} reason={rraw.reason} |g|={rraw.gnorm:.2e} "
          f"max|dq|={dq_raw:.2e} rel df={abs(f_at_raw - r64.fmin) / abs(r64.fmin):.1e}")
    spread = np.abs(r64e.X.reshape(-1, 4)[:, :3] - r64.X.reshape(-1, 4)[:, :3]).max()
    print(f"FP64 vs FP64 (two summation orders): max|dq|={spread:.2e} A, reasons {r64.reason}/{r64e.reason}")
    assert r64.reason == 3 and rmx.reason == 3 and r64e.reason == 3
    assert abs(f_at_mixed - r64.fmin) <= 1e-6 * abs(r64.fmin)
    assert abs(f_at_raw - r64.fmin) <= 1e-6 * abs(r64.fmin)
    assert dq < max(1e-4, 3.0 * spread)
    assert dq_raw < 1e-3


def test_span_guard_free_direction(gpu):
    """In a free direction the mixed form encodes coordinates modulo a 64 A
    span, exact while a listed pair is less than 32 A apart.  A site moved
    10 A (z, free) from where the lists were built is within the guard and
    the mixed form follows the FP64 form; moved 40 A, the mixed form returns
    A2C_ERR_LISTS_STALE instead of a wrapped pair vector, and serves the
    moved state again once the lists are rebuilt there."""
    X, xH, _, box, nPd, nH = A.lattice_fcc((5, 5, 6), periodic=(1, 1, 0), pos_std=0.02, sigma=(0.1, 0.1),
                                           x_center=0.05, x_half=0.01, seed=9)
    s = nPd + nH // 2  # an H site of a middle layer
    with A.Gpp(nPd, nH, box=box, periodic=(1, 1, 0)) as g:
        g.set_occupancy(xH)
        g.build_neighbors(X)

        def both(Xs):
            g.set_precision("fp64")
            f64, G64 = g.eval(Xs)
            g.set_precision("mixed")
            return f64, G64

        for dz in (10.0, 40.0):
            X2 = X.copy()
            X2[4 * s + 2] += dz
            f64, G64 = both(X2)
            if dz < 13.0:
                f, G = g.eval(X2)
                assert abs(f - f64) <= TOL_F * abs(f64)
                assert np.linalg.norm(G - G64) <= TOL_G * np.linalg.norm(G64)
            else:
                with pytest.raises(A.A2CError) as e:
                    g.eval(X2)
                assert e.value.status == A.A2C_ERR_LISTS_STALE
        g.build_neighbors(X2)
        f64, G64 = both(X2)
        f, G = g.eval(X2)
        assert abs(f - f64) <= TOL_F * abs(f64)
        assert np.linalg.norm(G - G64) <= TOL_G * np.linalg.norm(G64)


def test_minimize_keeps_widths_bound(gpu):
    """Long minimizations of a hydride-nucleus lattice: without a cap on the
    first trial step, accepted steps carried some Gaussian widths over the
    binding barrier (-3 kB x ln sigma falls without bound once a site leaves
    its neighbors; widths reached 300 A at 32^3 cells).  With the default
    max_step every width stays physical and both forms converge."""
    X, xH, _, box, nPd, nH = A.lattice_fcc(16, periodic=(1, 1, 1), pos_std=0.02, sigma=(0.1, 0.1), x_mode=1,
                                           x_matrix=0.02, x_nucleus=0.60, nucleus_radius=20.0, interface_width=5.0,
                                           x_half=0.0, seed=3)
    for prec in ("mixed", "fp64"):
        with A.Gpp(nPd, nH, box=box, periodic=(1, 1, 1), precision=prec) as g:
            g.set_occupancy(xH)
            g.build_neighbors(X)
            r = g.minimize(X, gatol=1e-5, max_it=4000, polish=0)
        sig = r.X[3::4]
        assert sig.max() < 0.5 and sig.min() > 0.03, (prec, sig.min(), sig.max())
        assert r.reason in (A.CONVERGED_GATOL, A.CONVERGED_STALLED), (prec, r.reason)


def test_host_pointer_eval_pinned_equals_pageable(gpu):
    """a2c_gpp_eval with pinned caller buffers (the prep kernel reads X and
    pass 2 writes G over the coherent host link) gives the same bits as with
    pageable buffers (bulk copies); a non-finite pinned input is rejected and
    the context stays usable."""
    import torch

    X, xH, _, box, nPd, nH = A.lattice_fcc(6, periodic=(1, 1, 1), pos_std=0.03, sigma=(0.08, 0.14), x_center=0.15,
                                           x_half=0.15, seed=2)
    with A.Gpp(nPd, nH, box=box, periodic=(1, 1, 1), precision="mixed") as g:
        g.set_occupancy(xH)
        g.build_neighbors(X)
        f0, G0 = g.eval(X)  # pageable numpy buffers
        Xp = torch.empty(X.size, dtype=torch.float64, pin_memory=True)
        Gp = torch.empty(X.size, dtype=torch.float64, pin_memory=True)
        Xp.numpy()[:] = X
        import ctypes as C

        fv = C.c_double()
        L = A._native.lib()

        def call():
            return L.a2c_gpp_eval(g.handle, C.c_void_p(Xp.data_ptr()), C.byref(fv), C.c_void_p(Gp.data_ptr()))

        for _ in range(2):
            A._native.check(call(), "a2c_gpp_eval")
            assert fv.value == f0 and np.array_equal(Gp.numpy(), G0)
        Xp.numpy()[7] = np.nan
        assert call() == A._native.A2C_ERR_NONFINITE
        Xp.numpy()[:] = X
        A._native.check(call(), "a2c_gpp_eval")
        assert fv.value == f0 and np.array_equal(Gp.numpy(), G0)


def test_device_driven_minimizer_matches_host_loop(gpu):
    """Mixed-precision a2c_gpp_minimize runs as replayed CUDA-graph ticks of
    the one-instance batch engine; it reaches the same minimum as the
    host-driven loop (their global sums differ in order only), and after a
    neighbor rebuild that reallocates the list array it re-captures.

    "The same minimum" is up to the resolution the stopping rule leaves and
    up to a uniform translation (a zero mode of the periodic box, along which
    the FP32 noise of the summed gradient moves each run differently): the
    bound on the distance of positions, mean displacement removed, is three
    times the largest distance between host-loop runs whose evaluators
    differ by FP32 rounding alone (4 vs 1, 2 and 8 threads per site), with
    floors of 5e-4 A and 1e-9 relative in the free entropy."""
    X, xH, _, box, nPd, nH = A.lattice_fcc(6, periodic=(1, 1, 1), pos_std=0.03, sigma=(0.08, 0.14), x_center=0.15,
                                           x_half=0.15, seed=2)
    res = {}
    for host, tps in ((True, 4), (True, 1), (True, 2), (True, 8), (False, 4)):
        with A.Gpp(nPd, nH, box=box, periodic=(1, 1, 1), precision="mixed") as g:
            g.set_occupancy(xH)
            g.build_neighbors(X)
            g.set_threads_per_site(tps)
            g.set_minimizer(host)
            res[host, tps] = g.minimize(X, gatol=1e-5, polish=0)
            if not host:
                again = g.minimize(X, gatol=1e-5, polish=0)  # replays the captured tick
                assert np.array_equal(again.X, res[host, tps].X) and again.iters == res[host, tps].iters
    for key, r in res.items():
        assert r.reason in (A.CONVERGED_GATOL, A.CONVERGED_STALLED), (key, r.reason)

    def dq(a, b):
        d = a.X.reshape(-1, 4)[:, :3] - b.X.reshape(-1, 4)[:, :3]
        return np.abs(d - d.mean(axis=0)).max()

    host, dev = res[True, 4], res[False, 4]
    others = [res[True, t] for t in (1, 2, 8)]
    spread = max(dq(host, o) for o in others)
    spread_f = max(abs(host.fmin - o.fmin) for o in others)
    d, d_f = dq(host, dev), abs(host.fmin - dev.fmin)
    print(f"host vs device-driven: max|dq| {d:.2e} A, |df| {d_f:.2e}; host 4 vs 1/2/8 threads/site: "
          + ", ".join(f"{dq(host, o):.2e} A {abs(host.fmin - o.fmin):.2e}" for o in others))
    assert d < max(3 * spread, 5e-4), (d, spread)
    assert d_f <= max(3 * spread_f, 1e-9 * abs(host.fmin)), (d_f, spread_f)
    # re-capture after the list array moves: a 3% compression pulls the 4th
    # Pd-Pd shell (5.50 A) inside rc, so the rebuilt lists need a larger array
    Y = X.copy()
    Y.reshape(-1, 4)[:, :3] *= 0.97
    with A.Gpp(nPd, nH, box=box, periodic=(1, 1, 1), precision="mixed") as g:
        g.set_occupancy(xH)
        g.build_neighbors(X)
        g.minimize(X, gatol=1e-4, polish=0)  # captures with the first array
        g.build_neighbors(Y)
        r2 = g.minimize(Y, gatol=1e-5, max_it=300, polish=0)
    with A.Gpp(nPd, nH, box=box, periodic=(1, 1, 1), precision="mixed") as h:
        h.set_occupancy(xH)
        h.build_neighbors(Y)
        ref = h.minimize(Y, gatol=1e-5, max_it=300, polish=0)
    assert np.array_equal(r2.X, ref.X) and r2.iters == ref.iters


def test_tile_block_sizes_do_not_change_results(gpu):
    """The block sizes of the tile only group sites into blocks: a site's
    arithmetic is the same in every block, so at fixed threads per site every
    pass-1 and pass-2 block size gives the same bits; the tuner returns a
    valid tile and sets it."""
    X, xH, box, per, nPd, nH, pb = make("slab_4x5x6")
    with A.Gpp(nPd, nH, box=box, periodic=per, precision="mixed") as g:
        g.set_occupancy(xH)
        g.build_neighbors(X)
        for tps in (2, 4):
            ref = None
            for rb in (256, 512, 768):
                for gb in (128, 256, 512):
                    g.set_tile(tps, rb, gb)
                    assert g.tile() == (tps, rb, gb)
                    f, G = g.eval(X)
                    if ref is None:
                        ref = (f, G)
                    assert f == ref[0] and np.array_equal(G, ref[1]), (tps, rb, gb)
        tile, cands = g.autotune_tile(reps=2)
        assert tile[0] in (1, 2, 4, 8) and tile[1] in (256, 512, 768) and tile[2] in (128, 256, 512)
        assert g.tile() == tile and len(cands) == 10 and all(ms > 0 for _, ms in cands)


def test_mixed_chemical_potential_follows_fp64(gpu):
    """The mixed form's chemical potential (pair quadrature in FP32,
    compensated per-site sums, F' from its pass 1; the correction terms and
    log(x/(1-x)) in FP64) against the FP64 form's on the same state: gamma
    within 1e-4 absolute (gamma ~ chi/kT ~ 1e2 here, so ~1e-6 relative) and
    the same full_H flags, with and without correction coefficients."""
    X, xH, box, per, nPd, nH, pb = make("slab_4x5x6")
    rng = np.random.default_rng(5)
    gamma0 = rng.normal(size=nH)
    full0 = (rng.random(nH) < 0.1).astype(np.int32)
    xH = xH.copy()
    xH[:4] = [1e-3, 0.99995, 0.5, 0.2]
    for coe in (dict(), dict(coe_Pd=(0.3, 0.0, 0.02, -0.01), coe_H=(0.2, 0.01, -0.03, 0.004))):
        res = {}
        for prec in ("fp64", "mixed"):
            with A.Gpp(nPd, nH, box=box, periodic=per, precision=prec, **coe) as g:
                g.set_occupancy(xH)
                g.build_neighbors(X)
                res[prec] = g.chem_potential(2.5, gamma0, full0)
        g64, f64 = res["fp64"]
        gm, fm = res["mixed"]
        err = np.abs(gm - g64).max()
        print(f"coe={bool(coe)}: max |dgamma| = {err:.2e}, |gamma| max {np.abs(g64).max():.1f}")
        assert np.array_equal(fm, f64)
        assert err < 1e-4

