"""Snapshot writers (a2c_snapshot_begin / a2c_snapshot_write) in the
layout of the reference's Output class (Output.cpp:60-90, 133-480): the VTP
piece and the collection parse as XML and carry the state; the extended-XYZ
header has the reference's fields and every row its columns; frame names
are padded to four digits.  Host code only: no GPU."""
import xml.etree.ElementTree as ET

import numpy as np
import pytest

import a2c_gb300 as A


def state(nPd=8, nH=8, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.uniform(0.0, 10.0, size=(nPd + nH, 4))
    X[:, 3] = rng.uniform(0.05, 0.15, size=nPd + nH)
    return X.reshape(-1), rng.uniform(0.0, 1.0, size=nH), rng.normal(size=nH), X.reshape(-1) - 0.01


@pytest.mark.parametrize("precision,rtol", [(2, 1e-10), (1, 1e-6), (0, 1e-4)])
def test_vtp_pvd_xyz(tmp_path, precision, rtol):
    nPd, nH = 8, 8
    X, xH, gam, X0 = state(nPd, nH)
    prefix = str(tmp_path / "sol")
    d = A.snapshot_desc(prefix, fmt="both", precision=precision, box=(10.0, 11.0, 12.0), periodic=(1, 1, 0))
    A.snapshot_begin(d)
    tag = np.zeros(nPd + nH, dtype=np.int8)
    tag[nPd:nPd + 2] = 1
    for frame, t in ((0, 0.0), (1, 1e-12)):
        A.snapshot_write(d, frame, t, nPd, nH, X, xH, X0=X0, gamma=gam, tag=tag)
    # VTP
    root = ET.parse(prefix + "_L0_0001.vtp").getroot()
    assert root.get("type") == "PolyData"
    piece = root.find("PolyData/Piece")
    assert piece.get("NumberOfPoints") == str(nPd + nH)
    pts = np.array(piece.find("Points/DataArray").text.split(), dtype=float).reshape(-1, 3)
    assert np.allclose(pts, X.reshape(-1, 4)[:, :3], rtol=rtol, atol=0)
    arrays = {a.get("Name"): np.array(a.text.split(), dtype=float) for a in piece.find("PointData")}
    assert list(arrays) == ["SiteID", "MaterialID", "Tag", "AtomicFrequency", "MolarFraction", "ChemicalPotential"]
    assert np.array_equal(arrays["MaterialID"], [0] * nPd + [1] * nH)
    assert np.array_equal(arrays["Tag"], tag)
    assert np.allclose(arrays["AtomicFrequency"], X.reshape(-1, 4)[:, 3], rtol=rtol)
    assert np.allclose(arrays["MolarFraction"], np.r_[np.ones(nPd), xH], rtol=rtol)
    assert np.allclose(arrays["ChemicalPotential"], np.r_[np.zeros(nPd), gam], rtol=rtol, atol=1e-300)
    # PVD collection: two data sets, still well-formed after the in-place append
    coll = ET.parse(prefix + "_L0.pvd").getroot()
    files = [ds.get("file") for ds in coll.find("Collection")]
    assert files == ["sol_L0_0000.vtp", "sol_L0_0001.vtp"]
    # XYZ
    lines = open(prefix + "_L0_0001.xyz").read().splitlines()
    assert int(lines[0]) == nPd + nH
    hdr = lines[1]
    assert hdr.startswith('Lattice="1.000000e+01 0.000000e+00 0.000000e+00 0.000000e+00 1.100000e+01')
    assert 'pbc="T T F"' in hdr and 'Time=1.000000e-12' in hdr
    assert ('Properties="species:S:1:pos:R:3:disp:R:3:type:I:1:atomic_freq:R:1:tag:I:1:'
            'molar_frac:R:1:chem_potent:R:1"') in hdr
    rows = [ln.split() for ln in lines[2:]]
    assert len(rows) == nPd + nH and all(len(r) == 12 for r in rows)
    assert [r[0] for r in rows] == ["Pd"] * nPd + ["H"] * nH
    v = np.array([r[1:] for r in rows], dtype=float)
    Y, Y0 = X.reshape(-1, 4), X0.reshape(-1, 4)
    assert np.allclose(v[:, 0:3], Y[:, :3], rtol=rtol)
    assert np.allclose(v[:, 3:6], Y[:, :3] - Y0[:, :3], rtol=max(rtol, 1e-6), atol=1e-12)
    assert np.allclose(v[:, 7], Y[:, 3], rtol=rtol)
    assert np.allclose(v[:, 9], np.r_[np.ones(nPd), xH], rtol=rtol)


def test_frame_names_and_errors(tmp_path):
    X, xH, gam, _ = state()
    d = A.snapshot_desc(str(tmp_path / "a"), fmt="vtp")
    with pytest.raises(A.A2CError):  # the collection must exist first
        A.snapshot_write(d, 7, 0.0, 8, 8, X, xH)
    A.snapshot_begin(d)
    A.snapshot_write(d, 1234, 0.0, 8, 8, X, xH)
    A.snapshot_write(d, 12, 0.0, 8, 8, X, xH)
    assert (tmp_path / "a_L0_1234.vtp").exists() and (tmp_path / "a_L0_0012.vtp").exists()
    dx = A.snapshot_desc(str(tmp_path / "b"), fmt="xyz", precision=0)
    A.snapshot_write(dx, 3, 0.0, 8, 8, X, xH)  # XYZ needs no collection
    assert (tmp_path / "b_L0_0003.xyz").exists() and not (tmp_path / "b_L0.pvd").exists()


def test_lattice_id_in_names(tmp_path):
    """Output.cpp names every file by its lattice (_L<k>): two lattices of
    one run keep separate collections."""
    X, xH, gam, _ = state()
    for k, (nPd, nH) in enumerate(((8, 0), (0, 8))):
        d = A.snapshot_desc(str(tmp_path / "sol"), lattice_id=k)
        A.snapshot_begin(d)
        Xk = X[: 4 * 8] if nPd else X[4 * 8:]
        A.snapshot_write(d, 5, 0.25, nPd, nH, Xk, xH if nH else xH[:0])
    for k in (0, 1):
        assert (tmp_path / f"sol_L{k}_0005.vtp").exists() and (tmp_path / f"sol_L{k}_0005.xyz").exists()
        coll = open(tmp_path / f"sol_L{k}.pvd").read()
        assert f'file="sol_L{k}_0005.vtp"' in coll
    rows = open(tmp_path / "sol_L1_0005.xyz").read().splitlines()[2:]
    assert all(r.split()[0] == "H" for r in rows) and len(rows) == 8
    with pytest.raises(A.A2CError):
        A.snapshot_begin(A.snapshot_desc(str(tmp_path / "bad"), lattice_id=-1))


def test_lattice_sites_writer_matches_evaluator_layout(tmp_path):
    """A set-up lattice written with its own fields gives the evaluator
    writer's bytes when it describes the same sites (material 0 "Pd" with
    occupancy 1, material 1 "H")."""
    X, xH, gam, X0 = state()
    nPd, nH = 8, 8
    n = nPd + nH
    sid = (np.arange(n) % 4).astype(np.int8)
    tag = (np.arange(n) % 3).astype(np.int8)
    sites = {"q": X.reshape(-1, 4)[:, :3].copy(), "q0": X0.reshape(-1, 4)[:, :3].copy(),
             "l": np.zeros((n, 3)), "siteid": sid.astype(np.int32), "matid": np.r_[np.zeros(nPd), np.ones(nH)].astype(np.int32),
             "tag": tag.astype(np.int32), "sigma": X.reshape(-1, 4)[:, 3].copy(), "x": np.r_[np.ones(nPd), xH]}
    g_all = np.r_[np.zeros(nPd), gam]
    for prec in (0, 1, 2):
        a = A.snapshot_desc(str(tmp_path / f"a{prec}"), precision=prec, box=(10.0, 11.0, 12.0))
        b = A.snapshot_desc(str(tmp_path / f"b{prec}"), precision=prec, box=(10.0, 11.0, 12.0))
        A.snapshot_begin(a)
        A.snapshot_begin(b)
        A.snapshot_write(a, 2, 0.5, nPd, nH, X, xH, X0=X0, gamma=gam, siteid=sid, tag=tag)
        A.snapshot_write_lattice(b, 2, 0.5, sites, gamma=g_all, material_names=["Pd", "H"])
        for ext in ("_L0_0002.vtp", "_L0_0002.xyz"):
            assert open(tmp_path / f"a{prec}{ext}").read() == open(tmp_path / f"b{prec}{ext}").read()
    # unnamed materials are labelled Mat<id>, as Output.cpp:26-33 does for
    # no name and for an empty MaterialName alike
    c = A.snapshot_desc(str(tmp_path / "c"), fmt="xyz")
    A.snapshot_write_lattice(c, 0, 0.0, sites)
    rows = open(tmp_path / "c_L0_0000.xyz").read().splitlines()[2:]
    assert [r.split()[0] for r in rows] == ["Mat0"] * nPd + ["Mat1"] * nH
    d = A.snapshot_desc(str(tmp_path / "d"), fmt="xyz")
    A.snapshot_write_lattice(d, 0, 0.0, sites, material_names=["", "H"])
    rows = open(tmp_path / "d_L0_0000.xyz").read().splitlines()[2:]
    assert [r.split()[0] for r in rows] == ["Mat0"] * nPd + ["H"] * nH
    assert all(len(r.split()) == len(rows[0].split()) for r in rows)
