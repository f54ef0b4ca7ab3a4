"""Restart files in the reference's format (readresults.cpp:10-55): the
writer/reader round-trip, and the reader against the reference's own
readResults (compiled from its source where the reference tree exists)."""
import numpy as np
import pytest

import a2c_gb300 as A
from oracle import oracle as O


def state():
    X, xH, surf, box, nPd, nH = A.lattice_fcc((2, 2, 3), pos_std=0.03, sigma=(0.08, 0.14), x_center=0.4,
                                             x_half=0.39, seed=3)
    rng = np.random.default_rng(1)
    g = rng.normal(size=nH) * 3.0
    fh = (rng.random(nH) < 0.3).astype(np.int32)
    xH = xH.copy()
    xH[:3] = [0.0, 1.0, 0.5]
    return X, xH, g, fh, nPd, nH


def test_restart_round_trip_and_clamp(tmp_path):
    X, xH, g, fh, nPd, nH = state()
    p = tmp_path / "run.3.dat"
    A.restart_write(p, nPd, nH, X, xH, g, fh, step=3, time=1.5e-9)
    X2, xH2, g2, fh2 = A.restart_read(p, nPd, nH, xLb=1e-3, xUb=1 - 1e-16)
    assert np.array_equal(X2, X) and np.array_equal(g2, g) and np.array_equal(fh2, fh)
    want = np.clip(xH, 1e-3, 1 - 1e-16)
    assert np.array_equal(xH2, want)
    assert len(p.read_text().splitlines()) == 9 + nPd + nH


def test_restart_truncated_file_is_an_error(tmp_path):
    X, xH, g, fh, nPd, nH = state()
    p = tmp_path / "run.0.dat"
    A.restart_write(p, nPd, nH, X, xH, g, fh)
    p.write_text("\n".join(p.read_text().splitlines()[:20]) + "\n")
    with pytest.raises(A.A2CError):
        A.restart_read(p, nPd, nH)


@pytest.mark.skipif(not O.ref_available(), reason="reference library not built (no reference tree)")
def test_restart_reader_matches_reference(tmp_path):
    X, xH, g, fh, nPd, nH = state()
    A.restart_write(tmp_path / "base.12.dat", nPd, nH, X, xH, g, fh, step=12)
    mine = A.restart_read(tmp_path / "base.12.dat", nPd, nH, xLb=2e-3, xUb=0.97)
    ref = O.ref_read_results(tmp_path, "base", 12, nPd, nH, xLb=2e-3, xUb=0.97)
    for a, b in zip(mine, ref):
        assert np.array_equal(a, b)
