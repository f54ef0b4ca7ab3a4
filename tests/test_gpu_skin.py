"""Skin (Verlet) neighbor lists: the device refilter of extended candidate
lists at rc + skin (Minimizer::findLocalNeighbors, minimizer.cpp:833-1144)
must give exactly the lists a full cell-list build gives at the same
positions -- all five reference lists in order, the Pd shell counts -- and
must rebuild the candidates once a site has moved more than skin/2."""
import numpy as np
import pytest

import a2c_gb300 as A

pytestmark = pytest.mark.gpu

CASES = {
    "periodic": dict(ncell=5, periodic=(1, 1, 1)),
    "slab": dict(ncell=(5, 5, 4), periodic=(1, 1, 0)),
    "free": dict(ncell=3, periodic=(0, 0, 0)),
}


def lists(g):
    return [g.neighbors(k) for k in range(5)], g.shell_counts()


def same(a, b):
    (la, sa), (lb, sb) = a, b
    for (oa, ia), (ob, ib) in zip(la, lb):
        if not (np.array_equal(oa, ob) and np.array_equal(ia, ib)):
            return False
    return np.array_equal(sa, sb)


@pytest.mark.parametrize("case", sorted(CASES))
def test_refilter_equals_full_build(gpu, case):
    c = CASES[case]
    skin = 0.6
    X, xH, _, box, nPd, nH = A.lattice_fcc(c["ncell"], periodic=c["periodic"], pos_std=0.02, sigma=(0.1, 0.1),
                                           x_center=0.2, x_half=0.05, seed=7)
    rng = np.random.default_rng(3)
    with A.Gpp(nPd, nH, box=box, periodic=c["periodic"]) as g, A.Gpp(nPd, nH, box=box, periodic=c["periodic"]) as ref:
        g.set_neighbor_skin(skin)
        m0, r0 = g.update_neighbors(X)
        assert r0  # first call builds the candidates
        ref.build_neighbors(X)
        assert same(lists(g), lists(ref))
        Y = X.copy()
        for step in range(3):  # drift, every site well inside skin/2 of the candidate build
            d = rng.normal(0.0, 0.04, size=(nPd + nH, 3))
            d *= np.minimum(1.0, 0.09 / np.linalg.norm(d, axis=1))[:, None]
            Y4 = (X.reshape(-1, 4)).copy()
            Y4[:, :3] += d
            Y = Y4.reshape(-1)
            m, r = g.update_neighbors(Y)
            assert not r, step
            mref = ref.build_neighbors(Y)
            assert m == mref
            assert same(lists(g), lists(ref)), step
        # a site beyond skin/2: the candidates are rebuilt, the lists still match
        Y4 = Y.reshape(-1, 4).copy()
        Y4[nPd + 3, 0] += 0.5 * skin + 0.05
        Y = Y4.reshape(-1)
        m, r = g.update_neighbors(Y)
        assert r
        ref.build_neighbors(Y)
        assert same(lists(g), lists(ref))


def test_skin_validation(gpu):
    X, xH, _, box, nPd, nH = A.lattice_fcc(3, periodic=(1, 1, 1), seed=1)  # box 11.67 A
    with A.Gpp(nPd, nH, box=box, periodic=(1, 1, 1)) as g:
        with pytest.raises(A.A2CError):
            g.set_neighbor_skin(1.0)  # 2 (rc + skin) > box
        with pytest.raises(A.A2CError):
            g.set_neighbor_skin(-0.1)
        g.set_neighbor_skin(0.0)  # no skin: an update is a full build
        _, r = g.update_neighbors(X)
        assert r


def test_refilter_pinned_positions_and_checks(gpu):
    """Positions in pinned host memory (read by the device directly) give
    the lists pageable positions give; non-finite positions and periodic
    coordinates outside [-L/2, 3L/2] are refused (checked on the device) and
    leave the lists as they were."""
    import torch

    from a2c_gb300 import _native as N

    X, xH, _, box, nPd, nH = A.lattice_fcc(5, periodic=(1, 1, 1), pos_std=0.02, sigma=(0.1, 0.1),
                                           x_center=0.2, x_half=0.05, seed=11)
    rng = np.random.default_rng(5)
    Y4 = X.reshape(-1, 4).copy()
    Y4[:, :3] += rng.uniform(-0.05, 0.05, size=(nPd + nH, 3))
    Y = Y4.reshape(-1)
    Yp = torch.empty(Y.size, dtype=torch.float64, pin_memory=True)
    Yp.copy_(torch.from_numpy(Y))
    with A.Gpp(nPd, nH, box=box, periodic=(1, 1, 1)) as g, A.Gpp(nPd, nH, box=box, periodic=(1, 1, 1)) as ref:
        g.set_neighbor_skin(0.6)
        g.update_neighbors(X)
        m, r = g.update_neighbors(Yp.numpy())
        assert not r
        ref.build_neighbors(Y)
        assert same(lists(g), lists(ref))
        before = lists(g)
        bad = Y.copy()
        bad[4 * 7 + 3] = np.nan
        with pytest.raises(A.A2CError) as e:
            g.update_neighbors(bad)
        assert e.value.status == N.A2C_ERR_NONFINITE
        with pytest.raises(A.A2CError) as e:
            ref.build_neighbors(bad)  # the full build's checks
        assert e.value.status == N.A2C_ERR_NONFINITE
        bad = Y.copy()
        bad[4 * 9 + 1] = 1.6 * box[1]
        with pytest.raises(A.A2CError) as e:
            g.update_neighbors(bad)
        assert e.value.status == N.A2C_ERR_INVALID
        # the refused calls changed nothing: the last positions still give the same lists
        m2, r2 = g.update_neighbors(Y)
        assert not r2 and m2 == m
        assert same(lists(g), before)
