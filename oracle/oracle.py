"""ctypes binding of the CPU oracle (liba2c_oracle.so) and, where it was
built, of the reference's own hot-path sources (_ref/liba2c_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the checker.  No product code imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "_build" / "liba2c_oracle.so"
REF_SO = HERE / "_ref" / "liba2c_ref.so"
# The reference tree: $A2C_REFERENCE_TREE when set, else a directory named
# "reference" beside the repository (absent on machines that run only the
# prebuilt libraries).
REFERENCE_TREE = Path(os.environ.get("A2C_REFERENCE_TREE") or (HERE.parent.parent / "reference"))

ID_MASK = (1 << 27) - 1
EAM_FUNCS = ["F_Pd", "F_Pd_deriv", "F_H", "F_H_deriv", "f_Pd", "f_Pd_deriv", "f_H", "f_H_deriv", "phi_Pd",
             "phi_Pd_deriv", "phi_PdH", "phi_PdH_deriv", "phi_H", "phi_H_deriv"]

P, D, I, I64 = C.c_void_p, C.c_double, C.c_int, C.c_int64


def build(ref: bool | None = None) -> None:
    """Compile the oracle (and the reference-shim library when the reference
    tree is present)."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    if ref is None:
        ref = REFERENCE_TREE.is_dir()
    if ref:
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={REFERENCE_TREE}"], check=True)
        subprocess.run(["make", "-s", "-C", str(HERE), "geo", f"REF={REFERENCE_TREE}"], check=True)
        subprocess.run(["make", "-s", "-C", str(HERE), "out", f"REF={REFERENCE_TREE}"], check=True)


class OrcParams(C.Structure):
    _fields_ = [("nPd", C.c_int), ("nH", C.c_int), ("T", D), ("QWp", D), ("eps", D), ("rc", D), ("a_Pd", D),
                ("box", D * 3), ("periodic", C.c_int * 3), ("coe_Pd", D * 4), ("coe_H", D * 4)]


class OrcLbfgs(C.Structure):
    _fields_ = [("m", C.c_int), ("max_it", C.c_int), ("max_fev", C.c_int), ("max_ls", C.c_int), ("gatol", D),
                ("c1", D), ("init_step", D), ("sigma_lb", D), ("f_noise", D), ("stall_window", C.c_int),
                ("stall_rtol", D), ("max_step", D)]


def _p(a):
    return None if a is None else a.ctypes.data


_olib = None
_rlib = None


def olib() -> C.CDLL:
    global _olib
    if _olib is None:
        if not ORACLE_SO.exists():
            build(ref=False)
        L = C.CDLL(str(ORACLE_SO))
        L.orc_set_arith.argtypes = [I]
        L.orc_set_arith.restype = None
        L.orc_set_reduction.argtypes = [I]
        L.orc_set_reduction.restype = None
        L.orc_eam.argtypes = [I, P, I64, D, P]
        L.orc_neighbor_counts.argtypes = [C.POINTER(OrcParams), P, P, P]
        L.orc_neighbor_fill.argtypes = [C.POINTER(OrcParams), P, P, P, P, P, P]
        L.orc_eval.argtypes = [C.POINTER(OrcParams), P, P, P, P, I, I, C.POINTER(D), P, P, P]
        L.orc_density.argtypes = [C.POINTER(OrcParams), P, P, P, P, I, P]
        L.orc_chem_potential.argtypes = [C.POINTER(OrcParams), P, P, P, P, D, I, P, P]
        L.orc_diffuse.argtypes = [I, P, P, P, P, P, D, D, D, D, D, D, P]
        L.orc_dirichlet.argtypes = [P, I, D, D, P, P, P]
        L.orc_dirichlet.restype = None
        L.orc_macro_results.argtypes = [I, P, P, I, C.POINTER(D), C.POINTER(D)]
        L.orc_macro_results.restype = None
        L.orc_minimize.argtypes = [C.POINTER(OrcParams), P, P, P, P, C.POINTER(OrcLbfgs), I, C.POINTER(D),
                                   C.POINTER(I), C.POINTER(I), C.POINTER(D), C.POINTER(I)]
        L.orc_lattice_fcc.argtypes = [P, D, D, D, D, I, D, D, D, D, D, D, D, D, C.c_uint64, P, P, P]
        _olib = L
    return _olib


class arithmetic:
    """Context manager selecting the oracle's arithmetic: "reference" (the C
    library and sequential sums, pinned to the reference) or "device" (the
    portable exp/pow/log and the GPU reduction tree)."""

    def __init__(self, mode: str):
        self.mode = {"reference": 0, "device": 1}[mode]

    def __enter__(self):
        olib().orc_set_arith(self.mode)
        return self

    def __exit__(self, *exc):
        olib().orc_set_arith(0)


# terms per reduction chunk of the batched-instance evaluator and L-BFGS
BATCH_CHUNK = 2048


class reduction:
    """Context manager selecting the reduction order of the device
    arithmetic: "single" (one system: grid-strided partials) or "batch" (one
    instance of a batch: partials of BATCH_CHUNK consecutive terms)."""

    def __init__(self, mode: str):
        self.chunk = {"single": 0, "batch": BATCH_CHUNK}[mode]

    def __enter__(self):
        olib().orc_set_reduction(self.chunk)
        return self

    def __exit__(self, *exc):
        olib().orc_set_reduction(0)


def ref_available() -> bool:
    return REF_SO.exists()


def rlib() -> C.CDLL:
    global _rlib
    if _rlib is None:
        if not REF_SO.exists():
            raise RuntimeError("reference library not built (oracle/_ref); needs the reference tree")
        L = C.CDLL(str(REF_SO))
        L.ref_eam.argtypes = [I, P, I64, D, P]
        L.ref_eval.argtypes = [I, I, D, D, D, D, D, P, P, P, P, P, C.POINTER(D), P, P]
        L.ref_density.argtypes = [I, I, D, D, D, P, P, P, P, P]
        L.ref_density.restype = None
        L.ref_chem_potential.argtypes = [I, I, D, D, D, D, D, P, P, P, P, P, D, P, P]
        L.ref_neighbors_run.argtypes = [I, I, D, D, P]
        L.ref_neighbors_total.argtypes = [I]
        L.ref_neighbors_total.restype = I64
        L.ref_neighbors_get.argtypes = [I, P, P]
        L.ref_neighbors_get.restype = None
        L.ref_neighbors_maxneib.argtypes = [I]
        L.ref_diffuse.argtypes = [I, P, P, P, P, P, D, D, D, D, D, D, P]
        L.ref_dirichlet.argtypes = [I, P, I, D, D, P, P, P]
        L.ref_macro_results.argtypes = [I, P, P, I, C.POINTER(D), C.POINTER(D)]
        L.ref_read_results.argtypes = [C.c_char_p, C.c_char_p, I, I, I, D, D, P, P, P, P]
        _rlib = L
    return _rlib


class Problem:
    """Parameters shared by oracle calls."""

    def __init__(self, nPd, nH, *, T=300.0, QWp=1.0 / 12.0, eps=1e-5, rc=5.35, a_Pd=3.89, box=(0, 0, 0),
                 periodic=(0, 0, 0), coe_Pd=(0, 0, 0, 0), coe_H=(0, 0, 0, 0)):
        p = OrcParams()
        p.nPd, p.nH, p.T, p.QWp, p.eps, p.rc, p.a_Pd = nPd, nH, T, QWp, eps, rc, a_Pd
        for d in range(3):
            p.box[d] = float(box[d])
            p.periodic[d] = int(bool(periodic[d]))
        for k in range(4):
            p.coe_Pd[k] = float(coe_Pd[k])
            p.coe_H[k] = float(coe_H[k])
        self.p = p
        self.nPd, self.nH, self.N = nPd, nH, nPd + nH

    @property
    def coe(self) -> np.ndarray:
        return np.array(list(self.p.coe_Pd) + list(self.p.coe_H), dtype=np.float64)


def lattice_fcc(ncell, *, a: float = 3.89, periodic=(1, 1, 1), pos_std: float = 0.0, sigma=(0.1, 0.1),
                x_mode: int = 0, x_center: float = 0.05, x_half: float = 0.0, x_matrix: float = 0.02,
                x_nucleus: float = 0.6, nucleus_radius: float = 80.0, interface_width: float = 5.0,
                xLb: float = 1e-3, xUb: float = 1.0 - 1e-16, seed: int = 1):
    """The seeded benchmark lattice from the oracle's own generator
    (orc_lattice_fcc; the library's a2c_lattice_fcc draws the same values):
    (X, xH, surface, box, nPd, nH)."""
    if isinstance(ncell, int):
        ncell = (ncell, ncell, ncell)
    nc = np.array([int(c) for c in ncell], dtype=np.int32)
    nPd = nH = 4 * int(nc[0]) * int(nc[1]) * int(nc[2])
    X = np.empty(4 * (nPd + nH))
    xH = np.empty(nH)
    surf = np.empty(nH, dtype=np.int32)
    rc = olib().orc_lattice_fcc(_p(nc), a, pos_std, float(sigma[0]), float(sigma[1]), int(x_mode), x_center, x_half,
                                x_matrix, x_nucleus, nucleus_radius, interface_width, xLb, xUb, int(seed), _p(X),
                                _p(xH), _p(surf))
    if rc != 0:
        raise ValueError("orc_lattice_fcc: invalid arguments")
    box = tuple(float(ncell[d]) * a for d in range(3))
    return X, xH, surf, box, nPd, nH


def nthreads() -> int:
    return int(os.environ.get("A2C_ORACLE_THREADS", os.cpu_count() or 1))


# -- oracle ----------------------------------------------------------------
def eam(which: int | str, x, eps=1e-5) -> np.ndarray:
    if isinstance(which, str):
        which = EAM_FUNCS.index(which)
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    olib().orc_eam(which, _p(x), x.size, eps, _p(out))
    return out


def neighbors(pb: Problem, X):
    """Oracle neighbor lists: (off, nbr, PdPdnum, hh1_off, hh1)."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    cnt = np.zeros(pb.N, dtype=np.int64)
    c1 = np.zeros(max(pb.nH, 1), dtype=np.int64)
    assert olib().orc_neighbor_counts(C.byref(pb.p), _p(X), _p(cnt), _p(c1)) == 0
    off = np.zeros(pb.N + 1, dtype=np.int64)
    off[1:] = np.cumsum(cnt)
    off1 = np.zeros(pb.nH + 1, dtype=np.int64)
    off1[1:] = np.cumsum(c1[: pb.nH])
    nbr = np.zeros(max(int(off[-1]), 1), dtype=np.uint32)
    hh1 = np.zeros(max(int(off1[-1]), 1), dtype=np.int32)
    shell = np.zeros(3 * max(pb.nPd, 1), dtype=np.int32)
    assert olib().orc_neighbor_fill(C.byref(pb.p), _p(X), _p(off), _p(nbr), _p(shell), _p(off1), _p(hh1)) == 0
    return off, nbr[: off[-1]], shell[: 3 * pb.nPd].reshape(pb.nPd, 3), off1, hh1[: off1[-1]]


def evaluate(pb: Problem, X, xH, off, nbr, mode=1, threads=None):
    """Oracle objective: (f, G, rho, Vsite)."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    xH = np.ascontiguousarray(xH, dtype=np.float64)
    G = np.empty(4 * pb.N)
    rho = np.empty(pb.N)
    Vs = np.empty(pb.N)
    f = C.c_double()
    assert olib().orc_eval(C.byref(pb.p), _p(X), _p(xH), _p(off), _p(nbr), mode, threads or nthreads(), C.byref(f),
                           _p(G), _p(rho), _p(Vs)) == 0
    return f.value, G, rho, Vs


def density(pb: Problem, X, xH, off, nbr, threads=None):
    rho = np.empty(pb.N)
    X = np.ascontiguousarray(X, dtype=np.float64)
    xH = np.ascontiguousarray(xH, dtype=np.float64)
    assert olib().orc_density(C.byref(pb.p), _p(X), _p(xH), _p(off), _p(nbr), threads or nthreads(), _p(rho)) == 0
    return rho


def chem_potential(pb: Problem, X, xH, off, nbr, gamma_bd, gamma, full_H, threads=None):
    g = np.ascontiguousarray(gamma, dtype=np.float64).copy()
    fh = np.ascontiguousarray(full_H, dtype=np.int32).copy()
    X = np.ascontiguousarray(X, dtype=np.float64)
    xH = np.ascontiguousarray(xH, dtype=np.float64)
    assert olib().orc_chem_potential(C.byref(pb.p), _p(X), _p(xH), _p(off), _p(nbr), gamma_bd,
                                     threads or nthreads(), _p(g), _p(fh)) == 0
    return g, fh


def diffuse(nH, x0, hh1_off, hh1, gamma, full_H, T, dt, nu, Qm, xLb, xUb, x):
    x = np.ascontiguousarray(x, dtype=np.float64).copy()
    args = [np.ascontiguousarray(a, dtype=t) for a, t in
            ((x0, np.float64), (hh1_off, np.int64), (hh1, np.int32), (gamma, np.float64), (full_H, np.int32))]
    assert olib().orc_diffuse(nH, *[_p(a) for a in args], T, dt, nu, Qm, xLb, xUb, _p(x)) == 0
    return x


def dirichlet(sites, gamma_bd, xUb, x0, gamma, full_H):
    s = np.ascontiguousarray(sites, dtype=np.int32)
    x0 = np.ascontiguousarray(x0, dtype=np.float64).copy()
    g = np.ascontiguousarray(gamma, dtype=np.float64).copy()
    fh = np.ascontiguousarray(full_H, dtype=np.int32).copy()
    olib().orc_dirichlet(_p(s), s.size, gamma_bd, xUb, _p(x0), _p(g), _p(fh))
    return x0, g, fh


def macro_results(x, HSurf):
    x = np.ascontiguousarray(x, dtype=np.float64)
    hs = np.ascontiguousarray(HSurf, dtype=np.int32)
    a, b = C.c_double(), C.c_double()
    olib().orc_macro_results(x.size, _p(x), _p(hs) if hs.size else None, hs.size, C.byref(a), C.byref(b))
    return a.value, b.value


def minimize(pb: Problem, X, xH, off, nbr, *, m=5, max_it=10000, max_fev=20000, max_ls=30, gatol=1e-6, c1=1e-4,
             init_step=1e-2, sigma_lb=1e-6, f_noise=0.0, stall_window=50, stall_rtol=0.0, max_step=0.25,
             threads=None):
    lp = OrcLbfgs(m, max_it, max_fev, max_ls, gatol, c1, init_step, sigma_lb, f_noise, stall_window, stall_rtol,
                  max_step)
    X = np.ascontiguousarray(X, dtype=np.float64).copy()
    xH = np.ascontiguousarray(xH, dtype=np.float64)
    f, it, nf, gn, why = C.c_double(), C.c_int(), C.c_int(), C.c_double(), C.c_int()
    assert olib().orc_minimize(C.byref(pb.p), _p(X), _p(xH), _p(off), _p(nbr), C.byref(lp), threads or nthreads(),
                               C.byref(f), C.byref(it), C.byref(nf), C.byref(gn), C.byref(why)) == 0
    return dict(X=X, fmin=f.value, iters=it.value, nfev=nf.value, gnorm=gn.value, reason=why.value)


# -- list conversions --------------------------------------------------------
def split_lists(nPd, nH, off, nbr):
    """Combined per-site lists -> reference lists {PdPd, PdH, HPd, HH} as
    (offsets, local indices)."""
    ids = (np.asarray(nbr, dtype=np.uint32) & ID_MASK).astype(np.int64)
    out = {}
    for name, lo, hi, pdn in (("PdPd", 0, nPd, True), ("PdH", 0, nPd, False), ("HPd", nPd, nPd + nH, True),
                              ("HH", nPd, nPd + nH, False)):
        o = [0]
        v = []
        for s in range(lo, hi):
            seg = ids[off[s]:off[s + 1]]
            seg = seg[seg < nPd] if pdn else seg[seg >= nPd] - nPd
            v.extend(seg.tolist())
            o.append(len(v))
        out[name] = (np.array(o, dtype=np.int64), np.array(v, dtype=np.int32))
    return out


# -- reference (compiled from its own sources against single-rank shims) -----
def ref_eam(which, x, eps=1e-5):
    if isinstance(which, str):
        which = EAM_FUNCS.index(which)
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    rlib().ref_eam(which, _p(x), x.size, eps, _p(out))
    return out


def ref_evaluate(pb: Problem, X, xH, off, nbr):
    X = np.ascontiguousarray(X, dtype=np.float64)
    xH = np.ascontiguousarray(xH, dtype=np.float64)
    G = np.empty(4 * pb.N)
    rho = np.empty(pb.N)
    f = C.c_double()
    p = pb.p
    coe = pb.coe
    assert rlib().ref_eval(p.nPd, p.nH, p.T, p.QWp, p.eps, p.rc, p.a_Pd, _p(coe), _p(X), _p(xH), _p(off), _p(nbr),
                           C.byref(f), _p(G), _p(rho)) == 0
    return f.value, G, rho


def ref_density(pb: Problem, X, xH, off, nbr):
    rho = np.empty(pb.N)
    X = np.ascontiguousarray(X, dtype=np.float64)
    xH = np.ascontiguousarray(xH, dtype=np.float64)
    rlib().ref_density(pb.nPd, pb.nH, pb.p.QWp, pb.p.eps, pb.p.rc, _p(X), _p(xH), _p(off), _p(nbr), _p(rho))
    return rho


def ref_chem_potential(pb: Problem, X, xH, off, nbr, gamma_bd, gamma, full_H):
    g = np.ascontiguousarray(gamma, dtype=np.float64).copy()
    fh = np.ascontiguousarray(full_H, dtype=np.int32).copy()
    X = np.ascontiguousarray(X, dtype=np.float64)
    xH = np.ascontiguousarray(xH, dtype=np.float64)
    p = pb.p
    coe = pb.coe
    assert rlib().ref_chem_potential(p.nPd, p.nH, p.T, p.QWp, p.eps, p.rc, p.a_Pd, _p(coe), _p(X), _p(xH), _p(off),
                                     _p(nbr), gamma_bd, _p(g), _p(fh)) == 0
    return g, fh


def ref_neighbors(pb: Problem, X):
    """Reference findNeighbors + findLocalNeighbors: dict of lists in the
    reference's own (KD-tree) order, PdPdnum, and the two maxNeib values."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    L = rlib()
    assert L.ref_neighbors_run(pb.nPd, pb.nH, pb.p.rc, pb.p.a_Pd, _p(X)) == 0
    out = {}
    for lid, name, n in ((0, "PdPd", pb.nPd), (1, "PdH", pb.nPd), (2, "HPd", pb.nH), (3, "HH", pb.nH),
                         (4, "HH1", pb.nH), (5, "PdPdnum", pb.nPd)):
        tot = L.ref_neighbors_total(lid)
        off = np.zeros(n + 1, dtype=np.int64)
        idx = np.zeros(max(tot, 1), dtype=np.int32)
        L.ref_neighbors_get(lid, _p(off), _p(idx))
        out[name] = (off, idx[:tot])
    out["maxNeib"] = (L.ref_neighbors_maxneib(0), L.ref_neighbors_maxneib(1))
    return out


def ref_diffuse(nH, x0, hh1_off, hh1, gamma, full_H, T, dt, nu, Qm, xLb, xUb, x):
    x = np.ascontiguousarray(x, dtype=np.float64).copy()
    args = [np.ascontiguousarray(a, dtype=t) for a, t in
            ((x0, np.float64), (hh1_off, np.int64), (hh1, np.int32), (gamma, np.float64), (full_H, np.int32))]
    assert rlib().ref_diffuse(nH, *[_p(a) for a in args], T, dt, nu, Qm, xLb, xUb, _p(x)) == 0
    return x


def ref_dirichlet(nH, sites, gamma_bd, xUb, x0, gamma, full_H):
    s = np.ascontiguousarray(sites, dtype=np.int32)
    x0 = np.ascontiguousarray(x0, dtype=np.float64).copy()
    g = np.ascontiguousarray(gamma, dtype=np.float64).copy()
    fh = np.ascontiguousarray(full_H, dtype=np.int32).copy()
    assert rlib().ref_dirichlet(nH, _p(s), s.size, gamma_bd, xUb, _p(x0), _p(g), _p(fh)) == 0
    return x0, g, fh


def ref_read_results(folder, base, num, nPd, nH, xLb=1e-3, xUb=1.0 - 1e-16):
    """The reference's readResults on <folder>/<base>.<num>.dat."""
    X, xH, g = np.empty(4 * (nPd + nH)), np.empty(nH), np.empty(nH)
    fh = np.empty(nH, dtype=np.int32)
    assert rlib().ref_read_results(str(folder).encode(), str(base).encode(), num, nPd, nH, xLb, xUb, _p(X), _p(xH),
                                   _p(g), _p(fh)) == 0
    return X, xH, g, fh


def ref_macro_results(x, HSurf):
    x = np.ascontiguousarray(x, dtype=np.float64)
    hs = np.ascontiguousarray(HSurf, dtype=np.int32)
    a, b = C.c_double(), C.c_double()
    assert rlib().ref_macro_results(x.size, _p(x), _p(hs) if hs.size else None, hs.size, C.byref(a),
                                    C.byref(b)) == 0
    return a.value, b.value


def dmd_run(pb: Problem, X, xH, gamma, full_H, off, nbr, hh1_off, hh1, bd_sites, surf_sites, nsteps, *, dt, nu, Qm,
            x_bd, gamma_bd, xLb=1e-3, xUb=1.0 - 1e-16, neighbor_update=False, **lbfgs):
    """The DMD outer loop in the order the device runs it: (lists rebuilt at
    the current positions when neighbor_update, from the second step) ->
    minimize -> chemical potential -> Dirichlet -> diffuse -> occupancy
    update -> macro results.  Returns the same fields as
    a2c_gb300.Gpp.dmd_run."""
    X = np.array(X, dtype=np.float64)
    x0 = np.array(xH, dtype=np.float64)
    g = np.array(gamma, dtype=np.float64)
    fh = np.array(full_H, dtype=np.int32)
    out = {"xH_mean": [], "xH_interior": [], "fmin": [], "iters": []}
    for k in range(nsteps):
        if neighbor_update and k > 0:
            off, nbr, _, hh1_off, hh1 = neighbors(pb, X)
        r = minimize(pb, X, x0, off, nbr, **lbfgs)
        X = r["X"]
        g, fh = chem_potential(pb, X, x0, off, nbr, gamma_bd, g, fh)
        x0, g, fh = dirichlet(bd_sites, gamma_bd, x_bd, x0, g, fh)
        x0 = diffuse(pb.nH, x0, hh1_off, hh1, g, fh, pb.p.T, dt, nu, Qm, xLb, xUb, x0.copy())
        a, b = macro_results(x0, surf_sites)
        out["xH_mean"].append(a)
        out["xH_interior"].append(b)
        out["fmin"].append(r["fmin"])
        out["iters"].append(r["iters"])
    res = {k: np.array(v) for k, v in out.items()}
    res.update(X=X, xH=x0, gamma=g, full_H=fh)
    return res


# ---------------------------------------------------------------------------
# Lattice set-up against the reference's geometry code (oracle/_ref/
# libgeo_ref.so, built from GeoTools by `make -C oracle geo`).
# ---------------------------------------------------------------------------
GEO_SO = HERE / "_ref" / "libgeo_ref.so"
_glib = None
_GEOM_TYPES = {"plane": 0, "cylinder_cone": 1, "cylinder_sphere": 2, "sphere": 3, "parallelepiped": 4, "spheroid": 5}


def geo_available() -> bool:
    return GEO_SO.exists()


def glib() -> C.CDLL:
    global _glib
    if _glib is None:
        if not GEO_SO.exists():
            raise RuntimeError("reference geometry library not built (oracle/_ref); needs the reference tree")
        L = C.CDLL(str(GEO_SO))
        L.geo_ref_distance.argtypes = [I, P, P, I64, P]
        L.geo_ref_bbox.argtypes = [I, P, P, P, P, P]
        _glib = L
    return _glib


def _gtype(g) -> int:
    t = g["type"]
    return _GEOM_TYPES[t] if isinstance(t, str) else int(t)


def ref_geo_distance(g: dict, q) -> np.ndarray:
    """The reference's signed distance (> 0 outside) of points q (n x 3)."""
    p = np.zeros(12)
    p[: len(g["p"])] = g["p"]
    q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 3)
    out = np.empty(len(q))
    assert glib().geo_ref_distance(_gtype(g), _p(p), _p(q), len(q), _p(out)) == 0
    return out


def ref_geo_bbox(g: dict, origin, abc):
    p = np.zeros(12)
    p[: len(g["p"])] = g["p"]
    O = np.ascontiguousarray(origin, dtype=np.float64)
    M = np.ascontiguousarray(abc, dtype=np.float64).reshape(9)
    lo, hi = np.empty(3), np.empty(3)
    assert glib().geo_ref_bbox(_gtype(g), _p(p), _p(O), _p(M), _p(lo), _p(hi)) == 0
    return lo, hi


def ref_lattice_sites(desc: dict) -> dict:
    """The sites of one lattice as the reference makes them, restated:
    SpaceInitializer::CreateOneLattice (SpaceInitializer.cpp:119-320) with
    CheckAndAddSitesInCell (:603-724) and FindLatticeDomainBoundingBox
    (:726-880), on one rank, with the reference's own signed distances and
    bounding boxes (GeoTools).  Returns the same fields as
    a2c_gb300.build_lattice, plus "dist_min": per site the smallest |signed
    distance| to any geometry surface it was tested against."""
    O = np.asarray(desc["origin"], dtype=np.float64)
    abc = np.asarray(desc["abc"], dtype=np.float64).reshape(3, 3)
    geoms = desc["geoms"]
    order = sorted(range(len(geoms)), key=lambda k: geoms[k]["order"])
    lmin = np.full(3, np.finfo(float).max)
    lmax = np.full(3, -np.finfo(float).max)
    for t in (1, 2, 3, 4, 5):  # cylinder-cones, cylinder-spheres, spheres, parallelepipeds, spheroids
        for g in geoms:
            if _gtype(g) != t or g.get("exterior", 0):
                continue
            lo, hi = ref_geo_bbox(g, O, abc)
            lmin = np.minimum(lmin, lo)
            lmax = np.maximum(lmax, hi)
    if not (np.all(np.isfinite(lmin)) and np.all(np.isfinite(lmax)) and np.all(lmin < lmax)):
        raise ValueError("unbounded lattice domain")
    lo_i = [int(np.floor(v)) for v in lmin]
    hi_i = [int(np.ceil(v)) + 1 for v in lmax]
    sites = desc["sites"]
    cells = [(li, lj, lk) for lk in range(lo_i[2], hi_i[2]) for lj in range(lo_i[1], hi_i[1])
             for li in range(lo_i[0], hi_i[0])]
    L, sid = [], []
    for (li, lj, lk) in cells:
        for s, sg in enumerate(sites):
            L.append((sg["l"][0] + li, sg["l"][1] + lj, sg["l"][2] + lk))
            sid.append(s)
    L = np.array(L, dtype=np.float64).reshape(-1, 3)
    sid = np.array(sid, dtype=np.int32)
    # LatticeStructure::GetXYZ: o + la a + lb b + lc c, left to right
    q0 = ((O + L[:, :1] * abc[0]) + L[:, 1:2] * abc[1]) + L[:, 2:3] * abc[2]
    inside = np.ones(len(q0), dtype=bool)
    dmin = np.full(len(q0), np.inf)
    inc = {"intersection": 1, "union": 2}
    for k in order:
        g = geoms[k]
        gi = g["inclusion"]
        intersect = (inc[gi] if isinstance(gi, str) else int(gi)) == 1
        test = (inside & intersect) | (~inside & (not intersect))
        if not test.any():
            continue
        d = ref_geo_distance(g, q0[test])
        dmin[test] = np.minimum(dmin[test], np.abs(d))
        if _gtype(g) == 0:
            new = d > 0.0
        else:
            out = d >= 0.0
            new = out if g.get("exterior", 0) else ~out
        inside[test] = new
    keep = inside
    disp = np.array([sg.get("mean_displacement", (0.0, 0.0, 0.0)) for sg in sites], dtype=np.float64)
    res = {"q0": q0[keep], "l": L[keep], "siteid": sid[keep]}
    res["q"] = res["q0"] + disp[res["siteid"]]
    res["matid"] = np.array([sites[s].get("materialid", 0) for s in res["siteid"]], dtype=np.int32)
    res["tag"] = np.array([sites[s].get("tag", 0) for s in res["siteid"]], dtype=np.int32)
    res["sigma"] = np.array([sites[s].get("atomic_frequency", -1.0) for s in res["siteid"]])
    res["x"] = np.array([sites[s].get("x", -1.0e-3) for s in res["siteid"]])
    res["dist_min"] = dmin[keep]
    res["dist_min_all"] = dmin
    res["inside_all"] = inside
    res["l_all"] = L
    return res


def ref_apply_region(sites: dict, region: dict) -> dict:
    """A regional initial condition as the reference applies it, restated:
    SpaceInitializer::ApplyRegionalICOnOneLattice (SpaceInitializer.cpp:
    883-1040) with the reference's own signed distances, on a copy."""
    out = {k: np.array(v, copy=True) for k, v in sites.items()}
    sel = (out["matid"] == region.get("materialid", -1)) & (out["siteid"] == region.get("siteid", -1))
    idx = np.nonzero(sel)[0]
    geoms = region.get("geoms", [])
    inside = np.ones(len(idx), dtype=bool)
    inc = {"intersection": 1, "union": 2}
    for k in sorted(range(len(geoms)), key=lambda k: geoms[k]["order"]):
        g = geoms[k]
        gi = g["inclusion"]
        intersect = (inc[gi] if isinstance(gi, str) else int(gi)) == 1
        test = (inside & intersect) | (~inside & (not intersect))
        if not test.any():
            continue
        d = ref_geo_distance(g, out["q"][idx[test]])
        if _gtype(g) == 0:
            new = d > 0.0
        else:
            o = d >= 0.0
            new = o if g.get("exterior", 0) else ~o
        inside[test] = new
    hit = idx[inside]
    out["q"][hit] += np.asarray(region.get("mean_displacement", (0.0, 0.0, 0.0)), dtype=np.float64)
    out["sigma"][hit] = region.get("atomic_frequency", -1.0)
    out["tag"][hit] = region.get("tag", 0)
    if region.get("x", -1.0e-3) >= 0.0:
        out["x"][hit] = region["x"]
    return out
