"""Lattice set-up from a lattice description (a2c_lattice_build,
a2c_lattice_conflicts, a2c_input_lattice) against the reference's
SpaceInitializer loop restated in the oracle over the reference's own
GeoTools signed distances and bounding boxes (oracle/_ref/libgeo_ref.so).

Bounds: identical site lists (positions, lattice coordinates, order,
attributes) wherever the reference's distance of a tested site to a surface
exceeds 1e-9; plane, sphere and parallelepiped decisions are the same
expressions as the reference's, so their boundary sites agree too."""
import textwrap

import numpy as np
import pytest

import a2c_gb300 as A
from oracle import oracle as O

A_PD = 3.89
FCC = [(0.0, 0.0, 0.0), (0.0, 0.5, 0.5), (0.5, 0.0, 0.5), (0.5, 0.5, 0.0)]
OCT = [(0.5, 0.0, 0.0), (0.0, 0.5, 0.0), (0.0, 0.0, 0.5), (0.5, 0.5, 0.5)]

needs_ref = pytest.mark.skipif(not O.geo_available(), reason="reference geometry library not built")


def sites(basis, **kw):
    return [dict({"l": l, "materialid": 0, "atomic_frequency": 0.1}, **kw) for l in basis]


def cubic(a=A_PD, origin=(0.0, 0.0, 0.0)):
    return {"abc": [a, 0, 0, 0, a, 0, 0, 0, a], "origin": list(origin)}


def box(p0, edges, order=0, inclusion="intersection", exterior=0):
    P = np.asarray(p0, dtype=float)
    E = np.asarray(edges, dtype=float).reshape(3, 3)
    return {"type": "parallelepiped", "order": order, "inclusion": inclusion, "exterior": exterior,
            "p": list(P) + list(P + E[0]) + list(P + E[1]) + list(P + E[2])}


def sphere(c, r, order=0, inclusion="intersection", exterior=0):
    return {"type": "sphere", "order": order, "inclusion": inclusion, "exterior": exterior, "p": list(c) + [r]}


def plane(pt, n, order=0, inclusion="intersection"):
    return {"type": "plane", "order": order, "inclusion": inclusion, "p": list(pt) + list(n)}


def compare(desc, tol=1e-9):
    ours = A.build_lattice(desc)
    ref = O.ref_lattice_sites(desc)
    if len(ours["q"]) == len(ref["q"]) and np.array_equal(ours["l"], ref["l"]):
        for k in A.LATTICE_SITE_FIELDS:
            assert np.array_equal(ours[k], ref[k]), k
        return len(ours["q"])
    # differences only at sites within tol of a surface the reference tested
    a = {tuple(r) for r in ours["l"]}
    b = {tuple(r) for r in ref["l"]}
    near = {tuple(r) for r, d in zip(ref["l_all"], ref["dist_min_all"]) if d <= tol}
    assert (a ^ b) <= near, sorted(a ^ b)[:5]
    return len(ours["q"])


@needs_ref
def test_boundary_aligned_parallelepiped():
    """Faces on lattice planes: the boundary sites are outside in both."""
    a = A_PD
    d = dict(cubic(), sites=sites(FCC), geoms=[box((0, 0, 0), [[4 * a, 0, 0], [0, 4 * a, 0], [0, 0, 4 * a]])])
    n = compare(d)
    assert n == 27 + 3 * 48  # the sites strictly inside the 4^3-cell block


@needs_ref
@pytest.mark.parametrize("case", ["sphere", "shell", "union", "slab", "half_offset_box", "displaced_origin"])
def test_geometry_combinations(case):
    a = A_PD
    c = (2.1 * a, 1.9 * a, 2.0 * a)
    if case == "sphere":
        g = [sphere(c, 6.0)]
    elif case == "shell":
        g = [sphere(c, 9.0), sphere(c, 4.0, order=1, exterior=1)]
    elif case == "union":
        g = [sphere(c, 5.0), sphere((c[0] + 6, c[1], c[2]), 4.0, order=1, inclusion="union")]
    elif case == "slab":
        g = [box((-0.3, -0.2, -0.1), [[5 * a, 0, 0], [0, 5 * a, 0], [0, 0, 5 * a]]),
             plane((0, 0, 4.0), (0, 0, 1), order=1), plane((0, 0, 12.0), (0, 0, -1), order=2)]
    elif case == "half_offset_box":
        g = [box((-a / 4, -a / 4, -a / 4), [[3 * a, 0, 0], [0, 3 * a, 0], [0, 0, 3 * a]])]
    else:
        g = [sphere((10.0, 10.0, 10.0), 7.5)]
    d = dict(cubic(origin=(0.3, -0.7, 1.1) if case == "displaced_origin" else (0, 0, 0)), sites=sites(FCC), geoms=g)
    assert compare(d) > 0


@needs_ref
@pytest.mark.parametrize("shape", ["spheroid", "cylinder_cone", "cylinder_sphere"])
def test_curved_shapes(shape):
    rng = np.random.default_rng(3)
    for _ in range(6):
        c = list(rng.uniform(5, 15, 3))
        ax = list(rng.normal(size=3))
        if shape == "spheroid":
            g = {"type": "spheroid", "order": 0, "inclusion": "intersection",
                 "p": c + ax + [float(rng.uniform(4, 9)), float(rng.uniform(3, 7))]}
        elif shape == "cylinder_cone":
            g = {"type": "cylinder_cone", "order": 0, "inclusion": "intersection",
                 "p": c + ax + [float(rng.uniform(3, 6)), float(rng.uniform(4, 10)), float(rng.uniform(20, 60)),
                                float(rng.uniform(1, 6))]}
        else:
            g = {"type": "cylinder_sphere", "order": 0, "inclusion": "intersection",
                 "p": c + ax + [float(rng.uniform(3, 6)), float(rng.uniform(4, 10)), float(rng.integers(0, 2)),
                                float(rng.integers(0, 2))]}
        assert compare(dict(cubic(), sites=sites(FCC + OCT), geoms=[g])) > 0


@needs_ref
def test_skewed_lattice_follows_the_reference_box():
    """Non-orthogonal lattice vectors (fcc primitive cell): the reference's
    bounding box projects on the lattice directions, which is not the
    lattice coordinate; the same cells are visited, so the same sites."""
    a = A_PD
    d = {"abc": [0, a / 2, a / 2, a / 2, 0, a / 2, a / 2, a / 2, 0], "origin": [0.2, 0.1, -0.3],
         "sites": [{"l": (0.0, 0.0, 0.0), "materialid": 0, "atomic_frequency": 0.1}],
         "geoms": [sphere((6.0, 5.0, 7.0), 6.3)]}
    assert compare(d) > 0


@needs_ref
def test_random_descriptions():
    rng = np.random.default_rng(7)
    for trial in range(20):
        a = rng.uniform(2.5, 4.5)
        skew = rng.normal(scale=0.15, size=(3, 3))
        abc = (np.eye(3) + skew) * a
        if np.linalg.det(abc) <= 0:
            abc[2] *= -1
        geoms = []
        n = int(rng.integers(1, 4))
        for k in range(n):
            t = rng.integers(0, 3)
            inc = "intersection" if k == 0 else ("union" if rng.random() < 0.5 else "intersection")
            ext = int(k > 0 and rng.random() < 0.3)
            if t == 0:
                geoms.append(sphere(list(rng.uniform(5, 12, 3)), float(rng.uniform(3, 8)), k, inc, ext))
            elif t == 1:
                E = np.diag(rng.uniform(6, 14, 3)) + rng.normal(scale=1.0, size=(3, 3))
                if np.linalg.det(E) <= 0:
                    E[2] *= -1
                geoms.append(box(list(rng.uniform(0, 4, 3)), E, k, inc, ext))
            else:
                if k == 0:
                    geoms.append(sphere(list(rng.uniform(5, 12, 3)), float(rng.uniform(4, 9)), k, inc, 0))
                else:
                    geoms.append(plane(list(rng.uniform(4, 10, 3)), list(rng.normal(size=3)), k, inc))
        d = {"abc": list(abc.reshape(9)), "origin": list(rng.uniform(-1, 1, 3)), "sites": sites(FCC),
             "geoms": geoms}
        compare(d)


def test_attributes_and_displacement():
    a = A_PD
    grp = [{"l": (0.0, 0.0, 0.0), "materialid": 0, "tag": 3, "atomic_frequency": 0.11,
            "mean_displacement": (0.01, -0.02, 0.03), "x": 1.0},
           {"l": (0.5, 0.5, 0.5), "materialid": 1, "tag": 7, "atomic_frequency": 0.09, "x": 0.25}]
    d = dict(cubic(), sites=grp, geoms=[box((-0.1, -0.1, -0.1), [[2 * a, 0, 0], [0, 2 * a, 0], [0, 0, 2 * a]])])
    r = A.build_lattice(d)
    assert len(r["q"]) == 16
    s0 = r["siteid"] == 0
    assert np.allclose(r["q"][s0] - r["q0"][s0], (0.01, -0.02, 0.03), atol=0, rtol=0) or \
        np.allclose(r["q"][s0] - r["q0"][s0], (0.01, -0.02, 0.03), atol=1e-15)
    assert np.array_equal(r["q"][~s0], r["q0"][~s0])
    assert set(r["tag"][s0]) == {3} and set(r["tag"][~s0]) == {7}
    assert set(r["matid"][~s0]) == {1} and set(r["sigma"][s0]) == {0.11} and set(r["x"][~s0]) == {0.25}
    # order: cells c, b, a from the box's lowest cell, then site groups
    assert np.array_equal(r["l"][0], (0.0, 0.0, 0.0)) and np.array_equal(r["l"][1], (0.5, 0.5, 0.5))


@pytest.mark.parametrize("bad, msg", [
    ({"geoms": [plane((0, 0, 0), (0, 0, 1))]}, "unbounded"),
    ({"geoms": [sphere((0, 0, 0), 5.0, 0), sphere((1, 1, 1), 5.0, 0)]}, "order"),
    ({"geoms": [dict(sphere((0, 0, 0), 5.0), inclusion=0)]}, "inclusion"),
    ({"sites": [{"l": (1.0, 0.0, 0.0), "materialid": 0}]}, "[0, 1)"),
    ({"sites": []}, "no lattice sites"),
    ({"geoms": [box((0, 0, 0), [[0, 5, 0], [5, 0, 0], [0, 0, 5]])]}, "right-hand"),
    ({"geoms": [sphere((0, 0, 0), 1.0e12)]}, "too large"),
])
def test_errors(bad, msg):
    d = dict(cubic(), sites=sites(FCC), geoms=[sphere((0, 0, 0), 5.0)])
    d.update(bad)
    with pytest.raises(A.A2CError, match=None) as e:
        A.build_lattice(d)
    assert msg in str(e.value)


def test_conflicts_box_test():
    """a2c_lattice_conflicts against a brute-force max-norm search."""
    rng = np.random.default_rng(1)
    q = rng.uniform(0, 20, (3000, 3))
    qo = rng.uniform(0, 20, (2000, 3))
    for dmin in (0.3, 1.0, 2.5):
        keep = A.lattice_conflicts(q, qo, dmin)
        cheb = np.abs(q[:, None, :] - qo[None, :, :]).max(axis=2)
        assert np.array_equal(keep, ~(cheb <= dmin).any(axis=1))
    # exactly dmin apart in one coordinate: a conflict (<= dmin)
    assert not A.lattice_conflicts([[0.0, 0.0, 0.0]], [[1.5, 0.0, 0.0]], 1.5)[0]
    # all other sites in one plane (a zero-width axis) and a grid far coarser than dmin
    qo = np.c_[rng.uniform(0, 50, (500, 2)), np.zeros(500)]
    q = np.c_[rng.uniform(0, 50, (800, 2)), rng.uniform(-0.5, 0.5, 800)]
    for dmin in (0.05, 0.7):
        keep = A.lattice_conflicts(q, qo, dmin)
        cheb = np.abs(q[:, None, :] - qo[None, :, :]).max(axis=2)
        assert np.array_equal(keep, ~(cheb <= dmin).any(axis=1))


def test_separate_pd_and_h_lattices_min_distance():
    """Pd and octahedral H as two lattices (the reference's own set-up):
    with the default MinDistance (the lattice constant) the box test finds
    an H site within a of every Pd site, so lattice 0 (Pd) loses all its
    sites; MinDistance below a/2 keeps both."""
    a = A_PD
    dom = [box((-0.2, -0.2, -0.2), [[3 * a, 0, 0], [0, 3 * a, 0], [0, 0, 3 * a]])]
    pd = dict(cubic(), sites=sites(FCC), geoms=dom)
    h = dict(cubic(), sites=sites(OCT), geoms=dom)
    out = A.build_lattices([pd, h])
    assert len(out[0]["q"]) == 0 and len(out[1]["q"]) == 108
    out = A.build_lattices([dict(pd, dmin=1.0), dict(h, dmin=1.0)])
    assert len(out[0]["q"]) == 108 and len(out[1]["q"]) == 108


def test_input_file_lattice(tmp_path):
    f = tmp_path / "input.st"
    f.write_text(textwrap.dedent("""
        under Lattice[0] {
          OAx = 3.89; OBy = 3.89; OCz = 3.89;
          Ox = 0.1; PeriodicOA = True;
          MinDistance = 1.0;
          under Site[0] { La = 0.0; Lb = 0.0; Lc = 0.0; MaterialID = 0; AtomicFrequency = 0.1; Tag = 2; }
          under Site[1] { La = 0.0; Lb = 0.5; Lc = 0.5; MaterialID = 0; AtomicFrequency = 0.1;
                          MeanDisplacementZ = 0.01; }
          under Site[2] { La = 0.5; Lb = 0.0; Lc = 0.5; MaterialID = 0; AtomicFrequency = 0.1; }
          under Site[3] { La = 0.5; Lb = 0.5; Lc = 0.0; MaterialID = 0; AtomicFrequency = 0.1;
                          under LocalSpecies[0] { SpeciesID = 1; MolarFraction = 0.3; } }
          under Parallelepiped[0] {
            Px = -0.2; Py = -0.2; Pz = -0.2;
            Ax = 11.47; Ay = -0.2; Az = -0.2;
            Bx = -0.2; By = 11.47; Bz = -0.2;
            Cx = -0.2; Cy = -0.2; Cz = 11.47;
            Side = Interior; Inclusion = Intersection; OperationOrder = 0;
          }
          under Sphere[0] { Center_x = 5.0; Center_y = 5.0; Center_z = 5.0; Radius = 2.0;
                            Side = Exterior; Inclusion = Intersection; OperationOrder = 1; }
          under CylinderAndCone[0] { CylinderRadius = 2.0; CylinderHeight = 3.0; Inclusion = Union;
                                     OperationOrder = 2; }
        }
    """))
    d = A.lattice_from_input(str(f), 0)
    assert d["abc"] == [3.89, 0, 0, 0, 3.89, 0, 0, 0, 3.89] and d["origin"] == [0.1, 0.0, 0.0]
    assert d["periodic"] == [1, 0, 0] and d["dmin"] == 1.0
    assert [s["l"] for s in d["sites"]] == [list(l) for l in FCC]
    assert d["sites"][0]["tag"] == 2 and d["sites"][1]["mean_displacement"] == [0.0, 0.0, 0.01]
    assert d["sites"][3]["x"] == 0.3 and d["sites"][0]["x"] == -1.0e-3
    kinds = {g["type"]: g for g in d["geoms"]}
    assert kinds[A.GEOMETRY_TYPES["sphere"]]["exterior"] == 1
    cone = kinds[A.GEOMETRY_TYPES["cylinder_cone"]]
    assert cone["p"][3:6] == [0.0, 0.0, 1.0] and cone["p"][8] == 45.0 and cone["inclusion"] == 2  # defaults
    r = A.build_lattice(d)
    assert len(r["q"]) > 0
    if O.geo_available():
        compare(d)


def test_input_file_rejects_plugin(tmp_path):
    f = tmp_path / "input.st"
    f.write_text('under Lattice[0] { under Site[0] { La = 0.0; Lb = 0.0; Lc = 0.0; MaterialID = 0; }\n'
                 '  under CustomGeometry { GeometrySpecifier = "libgeom.so"; } }\n')
    with pytest.raises(A.A2CError) as e:
        A.lattice_from_input(str(f), 0)
    assert "plug-ins are not supported" in str(e.value)


def region(geoms, **kw):
    r = {"lattice_id": -1, "materialid": 0, "siteid": 0, "tag": 5, "atomic_frequency": 0.2,
         "mean_displacement": (0.0, 0.0, 0.05), "x": 0.8, "geoms": geoms}
    r.update(kw)
    return r


@needs_ref
def test_regions_follow_the_reference():
    a = A_PD
    d = dict(cubic(), sites=sites(FCC + OCT, x=0.01), geoms=[box((-0.2, -0.2, -0.2), [[5 * a, 0, 0],
                                                                                     [0, 5 * a, 0],
                                                                                     [0, 0, 5 * a]])])
    s = A.build_lattice(d)
    regs = [region([sphere((9.0, 9.0, 9.0), 6.0)]),
            region([sphere((9.0, 9.0, 9.0), 7.0), sphere((9.0, 9.0, 9.0), 3.0, order=1, exterior=1),
                    plane((0, 0, 8.0), (0, 0, 1), order=2, inclusion="union")], siteid=5, x=-1.0e-3, tag=9),
            region([box((0.5, 0.5, 0.5), [[8, 0, 0], [0, 8, 0], [0, 0, 8]])], materialid=1)]  # no such material
    ours, ref = s, s
    for r in regs:
        ours = A.apply_region(ours, r)
        ref = O.ref_apply_region(ref, r)
        for k in A.LATTICE_SITE_FIELDS:
            assert np.array_equal(ours[k], ref[k]), k
    changed = ours["tag"] != s["tag"]
    assert changed.any() and set(ours["tag"][changed]) <= {5, 9}
    assert np.array_equal(ours["sigma"][ours["tag"] == 5], np.full((ours["tag"] == 5).sum(), 0.2))


def test_regions_from_input(tmp_path):
    f = tmp_path / "input.st"
    f.write_text(textwrap.dedent("""
        under Lattice[0] {
          OAx = 3.89; OBy = 3.89; OCz = 3.89; MinDistance = 1.0;
          under Site[0] { La = 0.0; Lb = 0.0; Lc = 0.0; MaterialID = 0; AtomicFrequency = 0.1; }
          under Site[1] { La = 0.5; Lb = 0.5; Lc = 0.5; MaterialID = 0; AtomicFrequency = 0.1;
                          under LocalSpecies[0] { SpeciesID = 1; MolarFraction = 0.01; } }
          under Sphere[0] { Center_x = 8.0; Center_y = 8.0; Center_z = 8.0; Radius = 8.5;
                            Side = Interior; Inclusion = Intersection; OperationOrder = 0; }
        }
        under RegionalInitialCondition[0] {
          LatticeID = 0; MaterialID = 0; SiteID = 1; Tag = 4; AtomicFrequency = 0.12;
          MeanDisplacementZ = 0.02;
          under LocalSpecies[0] { SpeciesID = 1; MolarFraction = 0.75; }
          under Sphere[0] { Center_x = 8.0; Center_y = 8.0; Center_z = 8.0; Radius = 4.0;
                            Side = Interior; Inclusion = Intersection; OperationOrder = 0; }
        }
        under RegionalInitialCondition[1] {
          MaterialID = 0; SiteID = 0; Tag = 2;
          under Plane[0] { Point_z = 8.0; Normal_z = 1.0; Inclusion = Intersection; }
        }
    """))
    regs = A.regions_from_input(str(f))
    assert len(regs) == 2
    r0, r1 = regs
    assert (r0["lattice_id"], r0["materialid"], r0["siteid"], r0["tag"]) == (0, 0, 1, 4)
    assert r0["atomic_frequency"] == 0.12 and r0["mean_displacement"] == [0.0, 0.0, 0.02] and r0["x"] == 0.75
    assert len(r0["geoms"]) == 1 and r0["geoms"][0]["type"] == A.GEOMETRY_TYPES["sphere"]
    assert r1["lattice_id"] == -1 and r1["atomic_frequency"] == -1.0 and r1["x"] == -1.0e-3  # defaults
    assert r1["geoms"][0]["type"] == A.GEOMETRY_TYPES["plane"] and r1["geoms"][0]["p"][5] == 1.0
    [lat] = A.build_lattices([A.lattice_from_input(str(f), 0)], regs)
    base = A.build_lattice(A.lattice_from_input(str(f), 0))
    hit = (lat["siteid"] == 1) & (lat["tag"] == 4)
    assert hit.any() and np.all(lat["x"][hit] == 0.75) and np.all(lat["sigma"][hit] == 0.12)
    assert np.allclose(lat["q"][hit] - base["q"][hit], (0, 0, 0.02), rtol=0, atol=1e-15)
    top = (lat["siteid"] == 0) & (lat["q"][:, 2] > 8.0)
    assert np.all(lat["tag"][top] == 2) and np.all(lat["sigma"][top] == -1.0)  # set as given, as the reference
    if O.geo_available():
        ref = O.ref_apply_region(O.ref_apply_region(base, r0), r1)
        for k in A.LATTICE_SITE_FIELDS:
            assert np.array_equal(lat[k], ref[k]), k


def test_material_names_and_lattice_snapshot(tmp_path):
    f = tmp_path / "input.st"
    f.write_text(textwrap.dedent("""
        under Material[0] { MaterialName = "Pd"; }
        under Material[1] { MaterialName = "PdH"; }
        under Lattice[0] {
          OAx = 3.89; OBy = 3.89; OCz = 3.89;
          under Site[0] { La = 0.0; Lb = 0.0; Lc = 0.0; MaterialID = 0; AtomicFrequency = 0.1; }
          under Site[1] { La = 0.5; Lb = 0.5; Lc = 0.5; MaterialID = 1; AtomicFrequency = 0.1; }
          under Sphere[0] { Center_x = 4.0; Center_y = 4.0; Center_z = 4.0; Radius = 4.5;
                            Side = Interior; Inclusion = Intersection; OperationOrder = 0; }
        }
    """))
    names = A.material_names_from_input(str(f))
    assert names == ["Pd", "PdH"]
    lat = A.build_lattice(A.lattice_from_input(str(f), 0))
    d = A.snapshot_desc(str(tmp_path / "sol"), fmt="xyz", lattice_id=0)
    A.snapshot_write_lattice(d, 1, 0.0, lat, material_names=names)
    rows = open(tmp_path / "sol_L0_0001.xyz").read().splitlines()[2:]
    assert [r.split()[0] for r in rows] == [names[m] for m in lat["matid"]]
