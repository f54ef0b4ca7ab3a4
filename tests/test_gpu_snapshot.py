"""The asynchronous snapshot (a2c_gpp_snapshot_async): the context's state
copied into pinned memory on its stream and written by a host thread gives
the same files, byte for byte, as the synchronous writer."""
import numpy as np
import pytest

import a2c_gb300 as A

pytestmark = pytest.mark.gpu


def test_async_snapshot_matches_sync(gpu, tmp_path):
    X, xH, _, box, nPd, nH = A.lattice_fcc(4, periodic=(1, 1, 1), pos_std=0.02, sigma=(0.1, 0.1), x_center=0.3,
                                           x_half=0.1, seed=2)
    gam = np.linspace(-3.0, 1.0, nH)
    with A.Gpp(nPd, nH, box=box, periodic=(1, 1, 1), precision="mixed") as g:
        g.set_occupancy(xH)
        g.build_neighbors(X)
        r = g.minimize(X, gatol=1e-3, max_it=30)
        da = A.snapshot_desc(str(tmp_path / "a"), box=box, periodic=(1, 1, 1))
        A.snapshot_begin(da)
        g.snapshot_async(da, 0, 0.0, X0=X, gamma=gam)
        g.eval(r.X)  # later work on the same stream while the writer runs
        g.snapshot_wait()
    ds = A.snapshot_desc(str(tmp_path / "s"), box=box, periodic=(1, 1, 1))
    A.snapshot_begin(ds)
    A.snapshot_write(ds, 0, 0.0, nPd, nH, r.X, xH, X0=X, gamma=gam)
    for ext in ("vtp", "xyz"):
        assert (tmp_path / f"a_L0_0000.{ext}").read_bytes() == (tmp_path / f"s_L0_0000.{ext}").read_bytes()
    assert (tmp_path / "a_L0.pvd").read_text().replace("a_L0", "s_L0") == (tmp_path / "s_L0.pvd").read_text()
