"""Batched independent instances (a2c_gpp_batch_*).

Per instance, the batch must reproduce one system: the gradient bit for bit
against a single context (the per-site arithmetic is the same code), the
objective and the whole minimization trajectory bit for bit against the
oracle in the device arithmetic with the batch's reduction order, and an
instance's results must not depend on the other instances.  The captured
CUDA-graph tick and the same launches issued one by one must agree bit for
bit.  The mixed form follows the FP64 minima."""
import numpy as np
import pytest

import a2c_gb300 as A
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SPECS = [  # (cells, T, mean x): 216, 1000, 2744 and 288 sites
    (3, 250.0, 0.05),
    (5, 450.0, 0.40),
    (7, 600.0, 0.65),
    ((3, 4, 3), 320.0, 0.20),
]


def make(specs=SPECS, seed=11):
    inst, Xs, xs = [], [], []
    for k, (cells, T, xm) in enumerate(specs):
        X, xH, _, box, nPd, nH = A.lattice_fcc(cells, periodic=(1, 1, 1), pos_std=0.02, sigma=(0.1, 0.1),
                                               x_center=xm, x_half=0.02, seed=seed + k)
        inst.append(dict(nPd=nPd, nH=nH, T=T, box=box, periodic=(1, 1, 1)))
        Xs.append(X)
        xs.append(xH)
    return inst, np.concatenate(Xs), np.concatenate(xs), Xs, xs


def open_batch(inst, X, xH, precision="fp64"):
    b = A.Batch(inst, precision=precision)
    b.set_occupancy(xH)
    b.build_neighbors(X)
    return b


def test_batch_eval_matches_single_and_oracle(gpu):
    inst, X, xH, Xs, xs = make()
    with open_batch(inst, X, xH) as b:
        f, G = b.eval(X)
    Gs = b.split(G)
    for k, it in enumerate(inst):
        with A.Gpp(it["nPd"], it["nH"], T=it["T"], box=it["box"], periodic=it["periodic"]) as g:
            g.set_occupancy(xs[k])
            g.build_neighbors(Xs[k])
            f1, G1 = g.eval(Xs[k])
        assert np.array_equal(Gs[k], G1), k
        assert abs(f[k] - f1) <= 1e-13 * abs(f1), (k, f[k], f1)
        pb = O.Problem(it["nPd"], it["nH"], T=it["T"], box=it["box"], periodic=it["periodic"])
        off, nbr, *_ = O.neighbors(pb, Xs[k])
        with O.arithmetic("device"), O.reduction("batch"):
            fo, Go, *_ = O.evaluate(pb, Xs[k], xs[k], off, nbr)
        assert fo == f[k], (k, fo, f[k])
        assert np.array_equal(Go, Gs[k]), k


def test_batch_mixed_eval_matches_single(gpu):
    inst, X, xH, Xs, xs = make()
    with open_batch(inst, X, xH, "mixed") as b:
        b.set_threads_per_site(4)
        f, G = b.eval(X)
    Gs = b.split(G)
    for k, it in enumerate(inst):
        with A.Gpp(it["nPd"], it["nH"], T=it["T"], box=it["box"], periodic=it["periodic"], precision="mixed") as g:
            g.set_occupancy(xs[k])
            g.build_neighbors(Xs[k])
            g.set_threads_per_site(4)
            f1, G1 = g.eval(Xs[k])
        assert np.array_equal(Gs[k], G1), k
        assert abs(f[k] - f1) <= 1e-13 * abs(f1), (k, f[k], f1)


KW = dict(gatol=1e-5, max_it=150)


def test_batch_minimize_fp64_bit_exact_vs_oracle(gpu):
    inst, X, xH, Xs, xs = make()
    with open_batch(inst, X, xH) as b:
        r = b.minimize(X, **KW)
    Xk = b.split(r.X)
    print("iters", r.iters, "nfev", r.nfev, "reason", r.reason, "ticks", r.ticks)
    for k, it in enumerate(inst):
        pb = O.Problem(it["nPd"], it["nH"], T=it["T"], box=it["box"], periodic=it["periodic"])
        off, nbr, *_ = O.neighbors(pb, Xs[k])
        with O.arithmetic("device"), O.reduction("batch"):
            o = O.minimize(pb, Xs[k], xs[k], off, nbr, **KW)
        assert (r.iters[k], r.nfev[k], r.reason[k]) == (o["iters"], o["nfev"], o["reason"]), k
        assert r.fmin[k] == o["fmin"], k
        assert r.gnorm[k] == o["gnorm"], k
        assert np.array_equal(Xk[k], o["X"]), k
    # every live instance is evaluated once per tick; the host polls every 8
    assert r.nfev.max() <= r.ticks <= r.nfev.max() + 17


def test_batch_graph_equals_eager_and_instances_independent(gpu):
    inst, X, xH, Xs, xs = make()
    res = {}
    for graphs in (True, False):
        with open_batch(inst, X, xH) as b:
            b.set_graphs(graphs)
            res[graphs] = b.minimize(X, **KW)
    assert np.array_equal(res[True].X, res[False].X)
    assert np.array_equal(res[True].iters, res[False].iters)
    assert np.array_equal(res[True].fmin, res[False].fmin)
    # instance 2 alone gives what it gave inside the batch
    k = 2
    with open_batch([inst[k]], Xs[k], xs[k]) as b1:
        r1 = b1.minimize(Xs[k], **KW)
    full = b.split(res[True].X)[k]
    assert np.array_equal(r1.X, full)
    assert r1.iters[0] == res[True].iters[k] and r1.fmin[0] == res[True].fmin[k]


def test_batch_mixed_minimize_follows_fp64(gpu):
    inst, X, xH, Xs, xs = make()
    kw = dict(gatol=1e-6, max_it=3000, max_fev=6000)
    with open_batch(inst, X, xH) as b:
        r64 = b.minimize(X, **kw)
    with open_batch(inst, X, xH, "mixed") as b:
        rmx = b.minimize(X, **kw)
    print("fp64", r64.iters, r64.reason, "mixed", rmx.mixed_iters, rmx.fp64_iters, rmx.reason)
    assert np.all(np.isin(rmx.reason, (A.CONVERGED_GATOL, A.CONVERGED_STALLED)))
    assert np.all(rmx.mixed_iters > 0)
    for k in range(len(inst)):
        a, c = b.split(rmx.X)[k].reshape(-1, 4), b.split(r64.X)[k].reshape(-1, 4)
        dq = np.abs(a[:, :3] - c[:, :3]).max()
        assert dq < 2e-3, (k, dq)
        assert abs(rmx.fmin[k] - r64.fmin[k]) <= 1e-9 * abs(r64.fmin[k]), k


def test_batch_rejects_bad_input(gpu):
    inst, X, xH, Xs, xs = make(SPECS[:2])
    bad = [dict(inst[0]), dict(inst[1])]
    bad[1]["box"] = (5.0, 5.0, 5.0)  # periodic box below 2 rc
    with pytest.raises(A.A2CError):
        A.Batch(bad)
    with open_batch(inst, X, xH) as b:
        Y = X.copy()
        Y[5] = np.nan
        with pytest.raises(A.A2CError):
            b.minimize(Y)
        with pytest.raises(A.A2CError):
            b.set_occupancy(np.full(xH.size, 1.5))


def test_batch_tile_tuner(gpu):
    """The batch's tile tuner picks a valid tile on the whole batch; block
    sizes leave every instance's results unchanged."""
    inst, X, xH = A.batch_workload(n=6, edge=(3, 5))
    with A.Batch(inst, precision="mixed") as b:
        b.set_occupancy(xH)
        b.build_neighbors(X)
        b.set_tile(4, 256, 256)
        f0, G0 = b.eval(X)
        b.set_tile(4, 512, 128)
        f1, G1 = b.eval(X)
        assert np.array_equal(f0, f1) and np.array_equal(G0, G1)
        tile, cands = b.autotune_tile(X, reps=2)
        assert tile[0] in (1, 2, 4, 8) and tile[1] in (256, 512, 768) and tile[2] in (128, 256, 512)
        assert b.tile() == tile and len(cands) == 10
