"""Generate the golden fixtures in this directory.

The reference has no tests, fixtures or golden vectors of its own, so the
fixtures are produced by running the reference's OWN hot-path sources
(compiled from the reference tree against single-rank shims by
oracle/Makefile's `ref` target) on seeded synthetic inputs:

  golden_eam.npz    every EAM function and FD derivative on a grid of r /
                    rho, including both sides of the switch points
                    r = 5.0, 5.05, 5.35 and r <= 0
  golden_free3.npz  a 3x3x3-cell free-surface Pd-H lattice (216 sites):
                    neighbor lists in the reference's own KD-tree order,
                    PdPdnum, HH1, densities, objective, gradient,
                    chemical potential (non-zero correction coefficients),
                    Dirichlet condition, one diffusion step, macro results
  golden_config1.npz the 6x6x6-cell periodic lattice of the plain-method
                    configuration (1,728 sites): objective and gradient
                    from the oracle (the periodic minimum image is an
                    extension the reference does not have, so this fixture
                    is the oracle's, whose non-periodic path is pinned to
                    the reference bit for bit)

Run from the repository root where the reference tree exists:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import a2c_gb300 as A  # noqa: E402  (lattice generator only)
from oracle import oracle as O  # noqa: E402

HERE = Path(__file__).resolve().parent
COE_PD = (0.3, 0.0, 0.02, -0.01)
COE_H = (0.2, 0.01, -0.03, 0.004)


def eam_grid() -> dict:
    r = np.concatenate([np.linspace(-0.5, 7.0, 1501)] +
                       [np.array([s - 2e-5, s - 1e-12, s, s + 1e-12, s + 2e-5]) for s in (0.0, 5.0, 5.05, 5.35)])
    rho = np.concatenate([np.linspace(0.0, 60.0, 601), np.array([1e-6, 0.5, 7.0, 13.3, 25.0])])
    out = {"r": r, "rho": rho}
    for w, name in enumerate(O.EAM_FUNCS):
        x = rho if name.startswith("F_") else r
        out[name] = O.ref_eam(w, x)
    return out


def free3() -> dict:
    X, xH, surf, box, nPd, nH = A.lattice_fcc(3, periodic=(0, 0, 0), pos_std=0.02, sigma=(0.08, 0.14),
                                             x_center=0.15, x_half=0.14, seed=11)
    pb = O.Problem(nPd, nH, coe_Pd=COE_PD, coe_H=COE_H)
    ref = O.ref_neighbors(pb, X)
    out = {"X": X, "xH": xH, "surf": surf, "nPd": nPd, "nH": nH}
    for name in ("PdPd", "PdH", "HPd", "HH", "HH1", "PdPdnum"):
        out[f"ref_{name}_off"], out[f"ref_{name}_idx"] = ref[name]
    out["maxNeib"] = np.array(ref["maxNeib"])
    off, nbr, *_ = O.neighbors(pb, X)
    f, G, rho = O.ref_evaluate(pb, X, xH, off, nbr)
    out.update(off=off, nbr=nbr, f=f, G=G, rho=rho)
    rng = np.random.default_rng(3)
    gamma0 = rng.normal(size=nH)
    full0 = (rng.random(nH) < 0.1).astype(np.int32)
    g, fh = O.ref_chem_potential(pb, X, xH, off, nbr, 2.5, gamma0, full0)
    out.update(gamma0=gamma0, full0=full0, gamma_bd=2.5, gamma=g, full_H=fh)
    sites = np.nonzero(surf)[0].astype(np.int32)
    x0d, gd, fd = O.ref_dirichlet(nH, sites, 4.0, 1 - 1e-16, xH, g, fh)
    out.update(sites=sites, x0_dir=x0d, gamma_dir=gd, full_dir=fd)
    o1, i1 = ref["HH1"]
    xprev = np.full(nH, 0.123)
    x = O.ref_diffuse(nH, x0d, o1, i1, gd, fd, 300.0, 1e-13, 1e13, 0.23, 1e-3, 1 - 1e-16, xprev)
    out.update(xprev=xprev, x_diff=x)
    out["macro"] = np.array(O.ref_macro_results(x, sites))
    return out


def config1() -> dict:
    X, xH, surf, box, nPd, nH = A.lattice_fcc(6, periodic=(1, 1, 1), pos_std=0.02, sigma=(0.1, 0.1), x_center=0.05,
                                             x_half=0.01, seed=1)
    pb = O.Problem(nPd, nH, box=box, periodic=(1, 1, 1))
    off, nbr, shell, o1, i1 = O.neighbors(pb, X)
    f, G, rho, _ = O.evaluate(pb, X, xH, off, nbr, mode=0, threads=1)
    return dict(X=X, xH=xH, box=np.array(box), nPd=nPd, nH=nH, off=off, nbr=nbr, shell=shell, hh1_off=o1, hh1=i1,
                f=f, G=G, rho=rho)


def main() -> None:
    O.build(ref=True)
    np.savez_compressed(HERE / "golden_eam.npz", **eam_grid())
    np.savez_compressed(HERE / "golden_free3.npz", **free3())
    np.savez_compressed(HERE / "golden_config1.npz", **config1())
    for p in sorted(HERE.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
