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
