"""a2c_gb300: GB300-native (sm_103a) GPP-EAM evaluator for a2c's diffusive
molecular dynamics hot path.

The product is the CUDA library behind the C ABI in include/a2c_gpp.h.
This module is a thin Python view of that ABI (for tests, benchmarks and
scripting); the reference-facing C++ host API is include/a2c_host.hpp.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N
from ._native import A2CError, A2C_ERR_LISTS_STALE, A2C_FP64, A2C_MIXED, A2C_PAIRS_BOTH_SIDES, A2C_PAIRS_ONCE  # noqa: F401
from ._native import (CONVERGED_GATOL, CONVERGED_STALLED, DIVERGED_LS_FAILURE, DIVERGED_MAXFCN,  # noqa: F401
                      DIVERGED_MAXITS, DIVERGED_NAN)

__all__ = ["Gpp", "Batch", "BatchResult", "batch_workload", "lattice_fcc", "peak_flops", "restart_write",
           "restart_read", "A2CError", "A2C_FP64", "A2C_MIXED", "A2C_PAIRS_BOTH_SIDES", "A2C_PAIRS_ONCE", "LbfgsResult"]


@dataclass
class LbfgsResult:
    X: np.ndarray
    fmin: float
    iters: int
    nfev: int
    gnorm: float
    reason: int
    mixed_iters: int = 0
    fp64_iters: int = 0
    mixed_gnorm: float = 0.0


def _f64(a, n=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float64)
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def _i32(a, n=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.int32)
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


class Gpp:
    """One evaluator context (Minimizer + AppCtx of the reference)."""

    def __init__(self, nPd: int, nH: int, *, T: float = 300.0, QWp: float = 1.0 / 12.0, eps: float = 1e-5,
                 rc: float = 5.35, a_Pd: float = 3.89, box=(0.0, 0.0, 0.0), periodic=(0, 0, 0),
                 coe_Pd=(0.0, 0.0, 0.0, 0.0), coe_H=(0.0, 0.0, 0.0, 0.0), precision: int | str = A2C_FP64,
                 device: int = 0):
        L = N.lib()
        p = N.GppParams()
        L.a2c_gpp_default_params(C.byref(p))
        p.nPd, p.nH = int(nPd), int(nH)
        p.T, p.QWp, p.eps, p.rc, p.a_Pd = T, QWp, eps, rc, a_Pd
        for d in range(3):
            p.box[d] = float(box[d])
            p.periodic[d] = int(bool(periodic[d]))
        for k in range(4):
            p.coe_Pd[k] = float(coe_Pd[k])
            p.coe_H[k] = float(coe_H[k])
        if isinstance(precision, str):
            precision = {"fp64": A2C_FP64, "mixed": A2C_MIXED}[precision]
        p.precision = int(precision)
        p.device = int(device)
        self.params = p
        self.nPd, self.nH = int(nPd), int(nH)
        self.N = self.nPd + self.nH
        h = C.c_void_p()
        N.check(L.a2c_gpp_create(C.byref(p), C.byref(h)), "a2c_gpp_create")
        self._h = h
        self._L = L

    # -- lifecycle -----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.a2c_gpp_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    @property
    def stream(self) -> int:
        return int(self._L.a2c_gpp_stream(self._h) or 0)

    def set_threads_per_site(self, tps: int) -> None:
        N.check(self._L.a2c_gpp_set_threads_per_site(self._h, int(tps)), "a2c_gpp_set_threads_per_site")

    def set_pair_mode(self, mode: int | str) -> None:
        """Mixed-precision pass 2: "once" (A2C_PAIRS_ONCE, default; each pair
        evaluated by one of its sites) or "both" (A2C_PAIRS_BOTH_SIDES)."""
        if isinstance(mode, str):
            mode = {"both": A2C_PAIRS_BOTH_SIDES, "once": A2C_PAIRS_ONCE}[mode]
        N.check(self._L.a2c_gpp_set_pair_mode(self._h, int(mode)), "a2c_gpp_set_pair_mode")

    @property
    def pair_mode(self) -> int:
        """The pass 2 mode the current lists run with."""
        m = C.c_int(0)
        N.check(self._L.a2c_gpp_get_pair_mode(self._h, C.byref(m)), "a2c_gpp_get_pair_mode")
        return m.value

    def synchronize(self) -> None:
        N.check(self._L.a2c_gpp_synchronize(self._h), "a2c_gpp_synchronize")

    def set_precision(self, precision: int | str) -> None:
        if isinstance(precision, str):
            precision = {"fp64": A2C_FP64, "mixed": A2C_MIXED}[precision]
        N.check(self._L.a2c_gpp_set_precision(self._h, int(precision)), "a2c_gpp_set_precision")

    # -- state ---------------------------------------------------------------
    def set_occupancy(self, xH) -> None:
        x = _f64(xH, self.nH)
        N.check(self._L.a2c_gpp_set_occupancy(self._h, N.ptr(x)), "a2c_gpp_set_occupancy")

    def occupancy(self) -> np.ndarray:
        x = np.empty(self.nH)
        N.check(self._L.a2c_gpp_get_occupancy(self._h, N.ptr(x)), "a2c_gpp_get_occupancy")
        return x

    def set_state(self, X) -> None:
        X = _f64(X, 4 * self.N)
        N.check(self._L.a2c_gpp_set_state(self._h, N.ptr(X)), "a2c_gpp_set_state")

    def state(self) -> np.ndarray:
        X = np.empty(4 * self.N)
        N.check(self._L.a2c_gpp_get_state(self._h, N.ptr(X)), "a2c_gpp_get_state")
        return X

    # -- neighbors -----------------------------------------------------------
    def build_neighbors(self, X) -> int:
        X = _f64(X, 4 * self.N)
        m = C.c_int(0)
        N.check(self._L.a2c_gpp_build_neighbors(self._h, N.ptr(X), C.byref(m)), "a2c_gpp_build_neighbors")
        return m.value

    def neighbors(self, list_id: int) -> tuple[np.ndarray, np.ndarray]:
        tot = C.c_int64(0)
        N.check(self._L.a2c_gpp_neighbor_total(self._h, list_id, C.byref(tot)), "a2c_gpp_neighbor_total")
        nsite = self.nPd if list_id in (N.LIST_PDPD, N.LIST_PDH) else self.nH
        off = np.zeros(nsite + 1, dtype=np.int64)
        idx = np.zeros(max(tot.value, 1), dtype=np.int32)
        N.check(self._L.a2c_gpp_get_neighbors(self._h, list_id, N.ptr(off), N.ptr(idx)), "a2c_gpp_get_neighbors")
        return off, idx[: tot.value]

    def set_neighbor_lists(self, X, lists: dict, PdPdnum=None) -> None:
        """Lists in the reference's form (a2c_gpp_set_neighbor_lists): `lists`
        maps LIST_PDPD, LIST_PDH, LIST_HPD, LIST_HH, LIST_HH1 to (offsets,
        local indices); X (4N) fixes periodic images."""
        arrs = []
        for lid in (N.LIST_PDPD, N.LIST_PDH, N.LIST_HPD, N.LIST_HH, N.LIST_HH1):
            o, i = lists[lid]
            arrs += [np.ascontiguousarray(o, dtype=np.int64), np.ascontiguousarray(i, dtype=np.int32)]
        Xa = None if X is None else np.ascontiguousarray(X, dtype=np.float64)
        sh = None if PdPdnum is None else np.ascontiguousarray(PdPdnum, dtype=np.int32)
        N.check(self._L.a2c_gpp_set_neighbor_lists(self._h, N.ptr(Xa), *[N.ptr(a) for a in arrs], N.ptr(sh)),
                "a2c_gpp_set_neighbor_lists")

    def shell_counts(self) -> np.ndarray:
        s = np.zeros(3 * max(self.nPd, 1), dtype=np.int32)
        N.check(self._L.a2c_gpp_get_shell_counts(self._h, N.ptr(s)), "a2c_gpp_get_shell_counts")
        return s[: 3 * self.nPd].reshape(self.nPd, 3)

    # -- evaluation ----------------------------------------------------------
    def eval(self, X) -> tuple[float, np.ndarray]:
        X = _f64(X, 4 * self.N)
        G = np.empty(4 * self.N)
        f = C.c_double(0.0)
        N.check(self._L.a2c_gpp_eval(self._h, N.ptr(X), C.byref(f), N.ptr(G)), "a2c_gpp_eval")
        return f.value, G

    def eval_device(self, dX: int, df: int, dG: int) -> None:
        """Stream-ordered evaluation on device pointers (ints)."""
        N.check(self._L.a2c_gpp_eval_device(self._h, C.c_void_p(dX), C.c_void_p(df), C.c_void_p(dG)),
                "a2c_gpp_eval_device")

    def profile_eval(self, dX: int, df: int, dG: int) -> np.ndarray:
        """Stage durations [ms] of one evaluation: prep, pass 1, pass 2, reduce."""
        ms = np.zeros(4, dtype=np.float32)
        N.check(self._L.a2c_gpp_profile_eval(self._h, C.c_void_p(dX), C.c_void_p(df), C.c_void_p(dG), N.ptr(ms)),
                "a2c_gpp_profile_eval")
        return ms

    def density(self) -> np.ndarray:
        r = np.empty(self.N)
        N.check(self._L.a2c_gpp_get_density(self._h, N.ptr(r)), "a2c_gpp_get_density")
        return r

    def eam(self, which: int, x) -> np.ndarray:
        """Device FP64 EAM function `which` (0..13, as a2c_gpp_eam_eval)."""
        x = _f64(x)
        out = np.empty_like(x)
        N.check(self._L.a2c_gpp_eam_eval(self._h, int(which), N.ptr(x), x.size, N.ptr(out)), "a2c_gpp_eam_eval")
        return out

    def bounds(self) -> tuple[np.ndarray, np.ndarray]:
        lb, ub = np.empty(4 * self.N), np.empty(4 * self.N)
        N.check(self._L.a2c_gpp_bounds(self._h, N.ptr(lb), N.ptr(ub)), "a2c_gpp_bounds")
        return lb, ub

    def autotune(self, reps: int = 3) -> tuple[int, dict]:
        """Threads per site chosen by the library's autotuner at the current
        state, and the mean milliseconds per evaluation of each candidate."""
        t = C.c_int()
        ms = (C.c_float * 4)()
        N.check(self._L.a2c_gpp_autotune(self._h, int(reps), C.byref(t), ms), "a2c_gpp_autotune")
        return t.value, {k: float(v) for k, v in zip((1, 2, 4, 8), ms)}

    def set_tile(self, tps: int = 0, rho_block: int = 0, grad_block: int = 0) -> None:
        """Tile of the mixed pair kernels (a2c_gpp_set_tile; 0 = the library's choice)."""
        N.check(self._L.a2c_gpp_set_tile(self._h, int(tps), int(rho_block), int(grad_block)), "a2c_gpp_set_tile")

    def tile(self) -> tuple[int, int, int]:
        """(threads per site, pass-1 block, pass-2 block) in use (a2c_gpp_get_tile)."""
        t = (C.c_int * 3)()
        N.check(self._L.a2c_gpp_get_tile(self._h, t), "a2c_gpp_get_tile")
        return tuple(int(v) for v in t)

    def autotune_tile(self, reps: int = 3) -> tuple[tuple[int, int, int], list]:
        """Tile chosen by the library's tuner at the current state (set on
        the context) and the candidates as (tile, ms) in the order timed."""
        t = (C.c_int * 3)()
        ms = (C.c_float * 10)()
        N.check(self._L.a2c_gpp_autotune_tile(self._h, int(reps), t, ms), "a2c_gpp_autotune_tile")
        return tuple(int(v) for v in t), _tile_candidates(ms)

    def snapshot_async(self, desc, frame: int, time: float, X0=None, gamma=None, siteid=None, tag=None) -> None:
        """Writes the context's current state (a2c_gpp_snapshot_async)."""
        X0, gamma = _opt(X0, np.float64, 4 * self.N), _opt(gamma, np.float64, self.nH)
        siteid, tag = _opt(siteid, np.int8, self.N), _opt(tag, np.int8, self.N)
        self._snap_desc = desc
        N.check(self._L.a2c_gpp_snapshot_async(self._h, C.byref(desc), int(frame), float(time),
                                               N.ptr(X0) if X0 is not None else None,
                                               N.ptr(gamma) if gamma is not None else None,
                                               N.ptr(siteid) if siteid is not None else None,
                                               N.ptr(tag) if tag is not None else None), "a2c_gpp_snapshot_async")

    def snapshot_wait(self) -> None:
        N.check(self._L.a2c_gpp_snapshot_wait(self._h), "a2c_gpp_snapshot_wait")

    def set_minimizer(self, mode) -> None:
        """L-BFGS driver (a2c_gpp_set_minimizer): "default" (mixed precision
        device-driven, FP64 host-driven), "host" (True) or "device" (the
        engine for both forms)."""
        m = {"default": 0, False: 0, "host": 1, True: 1, "device": 2}[mode]
        N.check(self._L.a2c_gpp_set_minimizer(self._h, m), "a2c_gpp_set_minimizer")

    def set_neighbor_skin(self, skin: float) -> None:
        N.check(self._L.a2c_gpp_set_neighbor_skin(self._h, float(skin)), "a2c_gpp_set_neighbor_skin")

    def update_neighbors(self, X) -> tuple[int, bool]:
        """Lists at X through the skin path: (max neighbors, whether the
        candidate lists were rebuilt)."""
        m, r = C.c_int(), C.c_int()
        N.check(self._L.a2c_gpp_update_neighbors(self._h, N.ptr(_f64(X, 4 * self.N)), C.byref(m), C.byref(r)),
                "a2c_gpp_update_neighbors")
        return m.value, bool(r.value)

    def minimize(self, X, **kw) -> LbfgsResult:
        lp = N.LbfgsParams()
        self._L.a2c_lbfgs_default_params(C.byref(lp))
        for k, v in kw.items():
            setattr(lp, k, v)
        X = _f64(X, 4 * self.N).copy()
        f, it, nfev, gn, why = C.c_double(), C.c_int(), C.c_int(), C.c_double(), C.c_int()
        N.check(self._L.a2c_gpp_minimize(self._h, N.ptr(X), C.byref(lp), C.byref(f), C.byref(it), C.byref(nfev),
                                         C.byref(gn), C.byref(why)), "a2c_gpp_minimize")
        mi, fi, mg = C.c_int(), C.c_int(), C.c_double()
        N.check(self._L.a2c_gpp_minimize_stats(self._h, C.byref(mi), C.byref(fi), C.byref(mg)), "a2c_gpp_minimize_stats")
        return LbfgsResult(X, f.value, it.value, nfev.value, gn.value, why.value, mi.value, fi.value, mg.value)

    # -- occupancy dynamics --------------------------------------------------
    def chem_potential(self, gamma_bd: float, gamma, full_H) -> tuple[np.ndarray, np.ndarray]:
        g = _f64(gamma, self.nH).copy()
        fh = _i32(full_H, self.nH).copy()
        N.check(self._L.a2c_gpp_chem_potential(self._h, float(gamma_bd), N.ptr(g), N.ptr(fh)),
                "a2c_gpp_chem_potential")
        return g, fh

    def apply_dirichlet(self, sites, gamma_bd: float, xUb: float, gamma, full_H) -> tuple[np.ndarray, np.ndarray]:
        s = _i32(sites)
        g = _f64(gamma, self.nH).copy()
        fh = _i32(full_H, self.nH).copy()
        N.check(self._L.a2c_gpp_apply_dirichlet(self._h, N.ptr(s), int(s.size), float(gamma_bd), float(xUb),
                                                N.ptr(g), N.ptr(fh)), "a2c_gpp_apply_dirichlet")
        return g, fh

    def diffuse(self, dt, nu, Qm, xLb, xUb, gamma, full_H, x) -> np.ndarray:
        g = _f64(gamma, self.nH)
        fh = _i32(full_H, self.nH)
        xo = _f64(x, self.nH).copy()
        N.check(self._L.a2c_gpp_diffuse(self._h, dt, nu, Qm, xLb, xUb, N.ptr(g), N.ptr(fh), N.ptr(xo)),
                "a2c_gpp_diffuse")
        return xo

    def dmd_run(self, X, xH, gamma, full_H, bd_sites, surf_sites, nsteps: int, *, dt: float, nu: float, Qm: float,
                x_bd: float, gamma_bd: float, xLb: float = 1e-3, xUb: float = 1.0 - 1e-16,
                neighbor_update: bool = False, host_steps: bool = False, **lbfgs) -> dict:
        """nsteps DMD outer steps on the device (a2c_gpp_dmd_run); host_steps
        sequences every step from the host instead of one CUDA graph."""
        dp = N.DmdParams()
        self._L.a2c_lbfgs_default_params(C.byref(dp.lbfgs))
        for k, v in lbfgs.items():
            setattr(dp.lbfgs, k, v)
        dp.dt, dp.nu, dp.Qm, dp.xLb, dp.xUb, dp.x_bd, dp.gamma_bd = dt, nu, Qm, xLb, xUb, x_bd, gamma_bd
        dp.neighbor_update = int(bool(neighbor_update))
        dp.host_steps = int(bool(host_steps))
        X = _f64(X, 4 * self.N).copy()
        xH = _f64(xH, self.nH).copy()
        g = _f64(gamma, self.nH).copy()
        fh = _i32(full_H, self.nH).copy()
        bd = _i32(bd_sites)
        sf = _i32(surf_sites)
        out = {k: np.zeros(max(nsteps, 1)) for k in ("xH_mean", "xH_interior", "fmin")}
        its = np.zeros(max(nsteps, 1), dtype=np.int32)
        N.check(self._L.a2c_gpp_dmd_run(self._h, N.ptr(X), N.ptr(xH), N.ptr(g), N.ptr(fh),
                                        N.ptr(bd) if bd.size else None, int(bd.size),
                                        N.ptr(sf) if sf.size else None, int(sf.size), C.byref(dp), int(nsteps),
                                        N.ptr(out["xH_mean"]), N.ptr(out["xH_interior"]), N.ptr(out["fmin"]),
                                        N.ptr(its)), "a2c_gpp_dmd_run")
        res = {k: v[:nsteps] for k, v in out.items()}
        res.update(X=X, xH=xH, gamma=g, full_H=fh, iters=its[:nsteps])
        return res

    def macro_results(self, x, HSurf) -> tuple[float, float]:
        x = _f64(x, self.nH)
        hs = _i32(HSurf)
        a, b = C.c_double(), C.c_double()
        N.check(self._L.a2c_gpp_macro_results(self._h, N.ptr(x), N.ptr(hs) if hs.size else None, int(hs.size),
                                              C.byref(a), C.byref(b)), "a2c_gpp_macro_results")
        return a.value, b.value


@dataclass
class BatchResult:
    X: np.ndarray         # concatenated minima
    fmin: np.ndarray      # per instance
    iters: np.ndarray
    nfev: np.ndarray
    gnorm: np.ndarray
    reason: np.ndarray
    mixed_iters: np.ndarray
    fp64_iters: np.ndarray
    ticks: int            # evaluations of every live instance
    seconds: float        # device time of the minimization


class Batch:
    """Many independent lattices evaluated and minimized together
    (a2c_gpp_batch_*).  `instances` is a sequence of dicts with keys nPd, nH
    and optionally T, box, periodic; the remaining parameters are shared.
    Arrays are the instances' arrays concatenated in instance order."""

    def __init__(self, instances, *, QWp: float = 1.0 / 12.0, eps: float = 1e-5, rc: float = 5.35,
                 a_Pd: float = 3.89, precision: int | str = A2C_FP64, device: int = 0):
        L = N.lib()
        if isinstance(precision, str):
            precision = {"fp64": A2C_FP64, "mixed": A2C_MIXED}[precision]
        arr = (N.GppParams * len(instances))()
        self.sizes = []
        for k, inst in enumerate(instances):
            p = arr[k]
            L.a2c_gpp_default_params(C.byref(p))
            p.nPd, p.nH = int(inst["nPd"]), int(inst["nH"])
            p.T = float(inst.get("T", 300.0))
            p.QWp, p.eps, p.rc, p.a_Pd = QWp, eps, rc, a_Pd
            box, per = inst.get("box", (0.0, 0.0, 0.0)), inst.get("periodic", (0, 0, 0))
            for d in range(3):
                p.box[d] = float(box[d])
                p.periodic[d] = int(bool(per[d]))
            p.precision = int(precision)
            p.device = int(device)
            self.sizes.append((p.nPd, p.nH))
        self.B = len(instances)
        self.N = sum(a + b for a, b in self.sizes)
        self.nH = sum(b for _, b in self.sizes)
        self.offsets = np.cumsum([0] + [a + b for a, b in self.sizes])
        h = C.c_void_p()
        N.check(L.a2c_gpp_batch_create(arr, self.B, C.byref(h)), "a2c_gpp_batch_create")
        self._h = h
        self._L = L

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.check(self._L.a2c_gpp_batch_destroy(self._h), "a2c_gpp_batch_destroy")
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_occupancy(self, xH) -> None:
        N.check(self._L.a2c_gpp_batch_set_occupancy(self._h, N.ptr(_f64(xH, self.nH))), "a2c_gpp_batch_set_occupancy")

    def build_neighbors(self, X) -> int:
        m = C.c_int()
        N.check(self._L.a2c_gpp_batch_build_neighbors(self._h, N.ptr(_f64(X, 4 * self.N)), C.byref(m)),
                "a2c_gpp_batch_build_neighbors")
        return m.value

    def set_threads_per_site(self, tps: int) -> None:
        N.check(self._L.a2c_gpp_batch_set_threads_per_site(self._h, int(tps)), "a2c_gpp_batch_set_threads_per_site")

    def set_graphs(self, on: bool) -> None:
        N.check(self._L.a2c_gpp_batch_set_graphs(self._h, int(bool(on))), "a2c_gpp_batch_set_graphs")

    def eval(self, X) -> tuple[np.ndarray, np.ndarray]:
        f = np.empty(self.B)
        G = np.empty(4 * self.N)
        N.check(self._L.a2c_gpp_batch_eval(self._h, N.ptr(_f64(X, 4 * self.N)), N.ptr(f), N.ptr(G)),
                "a2c_gpp_batch_eval")
        return f, G

    def minimize(self, X, **kw) -> BatchResult:
        lp = N.LbfgsParams()
        self._L.a2c_lbfgs_default_params(C.byref(lp))
        for k, v in kw.items():
            setattr(lp, k, v)
        X = _f64(X, 4 * self.N).copy()
        B = self.B
        fmin, gn = np.empty(B), np.empty(B)
        it, nf, why, mi, fi = (np.empty(B, dtype=np.int32) for _ in range(5))
        N.check(self._L.a2c_gpp_batch_minimize(self._h, N.ptr(X), C.byref(lp), N.ptr(fmin), N.ptr(it), N.ptr(nf),
                                               N.ptr(gn), N.ptr(why), N.ptr(mi), N.ptr(fi)), "a2c_gpp_batch_minimize")
        t, sec = C.c_int(), C.c_double()
        N.check(self._L.a2c_gpp_batch_stats(self._h, C.byref(t), C.byref(sec)), "a2c_gpp_batch_stats")
        return BatchResult(X, fmin, it, nf, gn, why, mi, fi, t.value, sec.value)

    def autotune(self, X, reps: int = 3) -> tuple[int, dict]:
        """Threads per site chosen by the library's autotuner, and the mean
        milliseconds per evaluation of each candidate."""
        t = C.c_int()
        ms = (C.c_float * 4)()
        N.check(self._L.a2c_gpp_batch_autotune(self._h, N.ptr(_f64(X, 4 * self.N)), int(reps), C.byref(t), ms),
                "a2c_gpp_batch_autotune")
        return t.value, {k: float(v) for k, v in zip((1, 2, 4, 8), ms)}

    def set_tile(self, tps: int = 0, rho_block: int = 0, grad_block: int = 0) -> None:
        N.check(self._L.a2c_gpp_batch_set_tile(self._h, int(tps), int(rho_block), int(grad_block)),
                "a2c_gpp_batch_set_tile")

    def tile(self) -> tuple[int, int, int]:
        t = (C.c_int * 3)()
        N.check(self._L.a2c_gpp_batch_get_tile(self._h, t), "a2c_gpp_batch_get_tile")
        return tuple(int(v) for v in t)

    def autotune_tile(self, X, reps: int = 3) -> tuple[tuple[int, int, int], list]:
        """Tile chosen by the library's tuner on the whole batch at X, and the
        candidates as (tile, ms) in the order timed."""
        t = (C.c_int * 3)()
        ms = (C.c_float * 10)()
        N.check(self._L.a2c_gpp_batch_autotune_tile(self._h, N.ptr(_f64(X, 4 * self.N)), int(reps), t, ms),
                "a2c_gpp_batch_autotune_tile")
        return tuple(int(v) for v in t), _tile_candidates(ms)

    def split(self, X) -> list[np.ndarray]:
        """Per-instance views of a concatenated 4N array."""
        X = np.asarray(X)
        return [X[4 * self.offsets[k]:4 * self.offsets[k + 1]] for k in range(self.B)]


def read_input(path: str) -> dict:
    """An input file in the reference's syntax (a2c_input_read): the fields
    the evaluator, the DMD loop and the snapshots use, with the reference's
    defaults.  Raises A2CError with the parser's message on a bad file."""
    inp = N.Input()
    msg = C.create_string_buffer(256)
    st = N.lib().a2c_input_read(str(path).encode(), C.byref(inp), msg, 256)
    if st != N.A2C_OK:
        raise A2CError(st, "a2c_input_read: " + msg.value.decode())
    out = {}
    for name, _ in N.Input._fields_:
        v = getattr(inp, name)
        if isinstance(v, bytes):
            v = v.decode()
        elif hasattr(v, "__len__"):
            v = list(v)
        out[name] = v
    return out


GEOMETRY_TYPES = {"plane": 0, "cylinder_cone": 1, "cylinder_sphere": 2, "sphere": 3, "parallelepiped": 4,
                  "spheroid": 5}
_INCLUSION = {"intersection": 1, "union": 2}
LATTICE_SITE_FIELDS = ("q", "q0", "l", "siteid", "matid", "tag", "sigma", "x")


def lattice_from_input(path: str, lattice_id: int = 0, max_sites: int = 256, max_geoms: int = 256) -> dict:
    """Lattice[lattice_id] of an input file (a2c_input_lattice) as a
    description dict: abc (9), origin, periodic, dmin, sites (list of dicts:
    l, materialid, tag, atomic_frequency, mean_displacement, x) and geoms
    (list of dicts: type, order, inclusion, exterior, p)."""
    desc = N.LatticeDesc()
    sites = (N.SiteGroup * max(max_sites, 1))()
    geoms = (N.Geometry * max(max_geoms, 1))()
    msg = C.create_string_buffer(256)
    st = N.lib().a2c_input_lattice(str(path).encode(), int(lattice_id), C.byref(desc), sites, max_sites, geoms,
                                   max_geoms, msg, 256)
    if st != N.A2C_OK:
        raise A2CError(st, "a2c_input_lattice: " + msg.value.decode())
    return {"abc": list(desc.abc), "origin": list(desc.origin), "periodic": list(desc.periodic), "dmin": desc.dmin,
            "sites": [{"l": list(g.l), "materialid": g.materialid, "tag": g.tag,
                       "atomic_frequency": g.atomic_frequency, "mean_displacement": list(g.mean_displacement),
                       "x": g.x} for g in sites[:desc.nsites]],
            "geoms": [{"type": g.type, "order": g.order, "inclusion": g.inclusion, "exterior": g.exterior,
                       "p": list(g.p)} for g in geoms[:desc.ngeom]]}


def _lattice_struct(desc: dict):
    d = N.LatticeDesc()
    for k in range(9):
        d.abc[k] = float(desc.get("abc", (1, 0, 0, 0, 1, 0, 0, 0, 1))[k])
    for k in range(3):
        d.origin[k] = float(desc.get("origin", (0, 0, 0))[k])
        d.periodic[k] = int(desc.get("periodic", (0, 0, 0))[k])
    d.dmin = float(desc.get("dmin", 0.0))
    sites = desc.get("sites", [])
    geoms = desc.get("geoms", [])
    sa = (N.SiteGroup * max(len(sites), 1))()
    for i, g in enumerate(sites):
        for k in range(3):
            sa[i].l[k] = float(g["l"][k])
            sa[i].mean_displacement[k] = float(g.get("mean_displacement", (0, 0, 0))[k])
        sa[i].materialid = int(g.get("materialid", 0))
        sa[i].tag = int(g.get("tag", 0))
        sa[i].atomic_frequency = float(g.get("atomic_frequency", -1.0))
        sa[i].x = float(g.get("x", -1.0e-3))
    ga = (N.Geometry * max(len(geoms), 1))()
    for i, g in enumerate(geoms):
        t = g["type"]
        ga[i].type = GEOMETRY_TYPES[t] if isinstance(t, str) else int(t)
        ga[i].order = int(g.get("order", i))
        inc = g.get("inclusion", "intersection")
        ga[i].inclusion = _INCLUSION[inc] if isinstance(inc, str) else int(inc)
        ga[i].exterior = int(bool(g.get("exterior", False)))
        for k, v in enumerate(g.get("p", ())):
            ga[i].p[k] = float(v)
    d.nsites, d.sites = len(sites), C.cast(sa, C.POINTER(N.SiteGroup))
    d.ngeom, d.geoms = len(geoms), C.cast(ga, C.POINTER(N.Geometry))
    return d, (sa, ga)


def build_lattice(desc: dict) -> dict:
    """The sites of one lattice (a2c_lattice_build): arrays q, q0, l (n x 3),
    siteid, matid, tag, sigma, x, in the reference's order."""
    d, keep = _lattice_struct(desc)
    msg = C.create_string_buffer(256)
    out = N.LatticeSites()
    st = N.lib().a2c_lattice_build(C.byref(d), C.byref(out), msg, 256)
    if st != N.A2C_OK:
        raise A2CError(st, "a2c_lattice_build: " + msg.value.decode())
    n = int(out.count)
    arr = {"q": np.zeros((n, 3)), "q0": np.zeros((n, 3)), "l": np.zeros((n, 3)),
           "siteid": np.zeros(n, np.int32), "matid": np.zeros(n, np.int32), "tag": np.zeros(n, np.int32),
           "sigma": np.zeros(n), "x": np.zeros(n)}
    if n:
        out.capacity = n
        for name in LATTICE_SITE_FIELDS:
            setattr(out, name, arr[name].ctypes.data)
        st = N.lib().a2c_lattice_build(C.byref(d), C.byref(out), msg, 256)
        if st != N.A2C_OK:
            raise A2CError(st, "a2c_lattice_build: " + msg.value.decode())
    del keep
    return arr


def _geoms_from(ga, n):
    return [{"type": g.type, "order": g.order, "inclusion": g.inclusion, "exterior": g.exterior,
             "p": list(g.p)} for g in ga[:n]]


def regions_from_input(path: str, max_regions: int = 64, max_geoms: int = 256) -> list:
    """The RegionalInitialCondition[k] blocks of an input file
    (a2c_input_regions) as dicts: lattice_id, materialid, siteid, tag,
    atomic_frequency, mean_displacement, x, geoms."""
    ra = (N.Region * max(max_regions, 1))()
    ga = (N.Geometry * max(max_geoms, 1))()
    n = C.c_int(0)
    msg = C.create_string_buffer(256)
    st = N.lib().a2c_input_regions(str(path).encode(), ra, max_regions, ga, max_geoms, C.byref(n), msg, 256)
    if st != N.A2C_OK:
        raise A2CError(st, "a2c_input_regions: " + msg.value.decode())
    base = C.addressof(ga)
    out = []
    for r in ra[: n.value]:
        first = (C.cast(r.geoms, C.c_void_p).value - base) // C.sizeof(N.Geometry) if r.ngeom else 0
        out.append({"lattice_id": r.lattice_id, "materialid": r.materialid, "siteid": r.siteid, "tag": r.tag,
                    "atomic_frequency": r.atomic_frequency, "mean_displacement": list(r.mean_displacement),
                    "x": r.x, "geoms": _geoms_from(ga[first:first + r.ngeom], r.ngeom)})
    return out


def material_names_from_input(path: str, max_materials: int = 64) -> list:
    """Material[m].MaterialName of an input file (a2c_input_material_names)."""
    L = 256
    buf = C.create_string_buffer(max_materials * L)
    n = C.c_int(0)
    msg = C.create_string_buffer(256)
    st = N.lib().a2c_input_material_names(str(path).encode(), buf, max_materials, L, C.byref(n), msg, 256)
    if st != N.A2C_OK:
        raise A2CError(st, "a2c_input_material_names: " + msg.value.decode())
    raw = buf.raw
    return [raw[k * L:(k + 1) * L].split(b"\0", 1)[0].decode() for k in range(n.value)]


def apply_region(sites: dict, region: dict) -> dict:
    """A regional initial condition (a2c_lattice_apply_region) applied to a
    copy of build_lattice's arrays."""
    out = {k: np.array(v, copy=True) for k, v in sites.items()}
    d, keep = _lattice_struct({"sites": [], "geoms": region.get("geoms", [])})
    r = N.Region()
    r.lattice_id = int(region.get("lattice_id", -1))
    r.materialid = int(region.get("materialid", -1))
    r.siteid = int(region.get("siteid", -1))
    r.tag = int(region.get("tag", 0))
    r.atomic_frequency = float(region.get("atomic_frequency", -1.0))
    for k in range(3):
        r.mean_displacement[k] = float(region.get("mean_displacement", (0, 0, 0))[k])
    r.x = float(region.get("x", -1.0e-3))
    r.ngeom, r.geoms = d.ngeom, d.geoms
    ls = N.LatticeSites()
    ls.capacity = ls.count = len(out["q"])
    for name in LATTICE_SITE_FIELDS:
        out[name] = np.ascontiguousarray(out[name])
        setattr(ls, name, out[name].ctypes.data)
    msg = C.create_string_buffer(256)
    st = N.lib().a2c_lattice_apply_region(C.byref(r), C.byref(ls), msg, 256)
    if st != N.A2C_OK:
        raise A2CError(st, "a2c_lattice_apply_region: " + msg.value.decode())
    del keep
    return out


def lattice_conflicts(q, q_other, dmin: float) -> np.ndarray:
    """Mask of the sites of q that stay (a2c_lattice_conflicts): False where
    a site of q_other lies within dmin in every coordinate."""
    q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 3)
    qo = np.ascontiguousarray(q_other, dtype=np.float64).reshape(-1, 3)
    keep = np.ones(len(q), dtype=np.uint8)
    nrem = C.c_int64(0)
    N.check(N.lib().a2c_lattice_conflicts(N.ptr(q), len(q), N.ptr(qo), len(qo), float(dmin), N.ptr(keep),
                                          C.byref(nrem)), "a2c_lattice_conflicts")
    return keep.astype(bool)


def build_lattices(descs: list, regions: list | None = None) -> list:
    """All lattices of an input (SpaceInitializer::SetupLatticeVariables,
    SpaceInitializer.cpp:41-116): each built; the regional initial
    conditions applied in index order (lattice_id < 0: to every lattice);
    then lattice i loses its sites within its dmin (MinDistance, or its
    shortest lattice vector) of lattice j's sites, for every j != i except
    j < i with a dmin not above i's (already resolved)."""
    out = [build_lattice(d) for d in descs]
    for r in regions or []:
        lid = int(r.get("lattice_id", -1))
        if lid >= len(out):
            raise A2CError(N.A2C_ERR_INVALID, f"RegionalInitialCondition: unknown lattice id {lid}")
        for k in (range(len(out)) if lid < 0 else [lid]):
            out[k] = apply_region(out[k], r)
    dm = []
    for d in descs:
        v = float(d.get("dmin", 0.0))
        if v <= 0.0:
            abc = np.asarray(d.get("abc", (1, 0, 0, 0, 1, 0, 0, 0, 1)), dtype=np.float64).reshape(3, 3)
            v = float(np.min(np.sqrt((abc * abc).sum(axis=1))))
        dm.append(v)
    for i in range(len(out)):
        for j in range(len(out)):
            if j == i or (j < i and dm[j] <= dm[i]):
                continue
            keep = lattice_conflicts(out[i]["q"], out[j]["q"], dm[i])
            if not keep.all():
                out[i] = {k: v[keep] for k, v in out[i].items()}
    return out


def snapshot_desc(prefix: str, *, fmt: str = "both", precision: int = 2, box=(0.0, 0.0, 0.0), origin=(0.0, 0.0, 0.0),
                  periodic=(0, 0, 0), lattice_id: int = 0):
    """Descriptor of a snapshot series (a2c_snapshot_desc): files
    <prefix>_L<lattice_id>_<frame>.vtp / .xyz and <prefix>_L<lattice_id>.pvd."""
    d = N.SnapshotDesc()
    d.lattice_id = int(lattice_id)
    d._prefix = str(prefix).encode()  # keeps the bytes alive with the descriptor
    d.prefix = d._prefix
    d.format = {"vtp": 1, "xyz": 2, "both": 3}[fmt]
    d.precision = int(precision)
    for k in range(3):
        d.axes[4 * k] = float(box[k])
        d.origin[k] = float(origin[k])
        d.periodic[k] = int(bool(periodic[k]))
    return d


def snapshot_begin(desc) -> None:
    N.check(N.lib().a2c_snapshot_begin(C.byref(desc)), "a2c_snapshot_begin")


def _opt(a, dtype, n):
    return None if a is None else np.ascontiguousarray(a, dtype=dtype).reshape(-1)[:n].copy()


def snapshot_write(desc, frame: int, time: float, nPd: int, nH: int, X, xH, X0=None, gamma=None, siteid=None,
                   tag=None) -> None:
    n = nPd + nH
    X = _f64(X, 4 * n)
    xH = _f64(xH, nH)
    X0, gamma = _opt(X0, np.float64, 4 * n), _opt(gamma, np.float64, nH)
    siteid, tag = _opt(siteid, np.int8, n), _opt(tag, np.int8, n)
    N.check(N.lib().a2c_snapshot_write(C.byref(desc), int(frame), float(time), int(nPd), int(nH), N.ptr(X),
                                       N.ptr(X0) if X0 is not None else None, N.ptr(xH),
                                       N.ptr(gamma) if gamma is not None else None,
                                       N.ptr(siteid) if siteid is not None else None,
                                       N.ptr(tag) if tag is not None else None), "a2c_snapshot_write")


def snapshot_write_lattice(desc, frame: int, time: float, sites: dict, gamma=None, material_names=None) -> None:
    """Snapshot of a set-up lattice (build_lattice's arrays) with its own
    site groups, materials, tags, widths and occupancies
    (a2c_snapshot_write_lattice); material_names label the XYZ species."""
    n = len(sites["q"])
    arr = {k: np.ascontiguousarray(sites[k]) for k in LATTICE_SITE_FIELDS}
    ls = N.LatticeSites()
    ls.capacity = ls.count = n
    for name in LATTICE_SITE_FIELDS:
        setattr(ls, name, arr[name].ctypes.data)
    g = None if gamma is None else np.ascontiguousarray(gamma, dtype=np.float64)
    names = list(material_names or [])
    cn = (C.c_char_p * max(len(names), 1))(*[str(m).encode() for m in names])
    N.check(N.lib().a2c_snapshot_write_lattice(C.byref(desc), int(frame), float(time), C.byref(ls),
                                               N.ptr(g) if g is not None else None, cn, len(names)),
            "a2c_snapshot_write_lattice")


def restart_write(path: str, nPd: int, nH: int, X, xH, gamma, full_H, step: int = 0, time: float = 0.0) -> None:
    """Restart file in the format the reference's readResults reads."""
    N.check(N.lib().a2c_restart_write(str(path).encode(), nPd, nH, N.ptr(_f64(X, 4 * (nPd + nH))),
                                      N.ptr(_f64(xH, nH)), N.ptr(_f64(gamma, nH)), N.ptr(_i32(full_H, nH)),
                                      int(step), float(time)), "a2c_restart_write")


def restart_read(path: str, nPd: int, nH: int, xLb: float = 1e-3, xUb: float = 1.0 - 1e-16):
    """(X, xH, gamma, full_H) from a restart file (x clamped to [xLb, xUb])."""
    X, xH, g = np.empty(4 * (nPd + nH)), np.empty(nH), np.empty(nH)
    fh = np.empty(nH, dtype=np.int32)
    N.check(N.lib().a2c_restart_read(str(path).encode(), nPd, nH, xLb, xUb, N.ptr(X), N.ptr(xH), N.ptr(g), N.ptr(fh)),
            "a2c_restart_read")
    return X, xH, g, fh


def peak_flops(precision: int | str = A2C_MIXED, device: int = 0) -> float:
    """Measured FMA-pipe peak (flop/s) of FP32 ("mixed") or FP64 ("fp64")."""
    if isinstance(precision, str):
        precision = {"fp64": A2C_FP64, "mixed": A2C_MIXED, "fp32": A2C_MIXED}[precision]
    v = C.c_double()
    N.check(N.lib().a2c_gpp_peak_flops(int(device), int(precision), C.byref(v)), "a2c_gpp_peak_flops")
    return v.value


def lattice_fcc(ncell, *, a: float = 3.89, periodic=(1, 1, 1), pos_std: float = 0.0, sigma=(0.1, 0.1),
                x_mode: int = 0, x_center: float = 0.05, x_half: float = 0.0, x_matrix: float = 0.02,
                x_nucleus: float = 0.6, nucleus_radius: float = 80.0, interface_width: float = 5.0,
                xLb: float = 1e-3, xUb: float = 1.0 - 1e-16, seed: int = 1, device_out=None):
    """Seeded fcc Pd + octahedral H lattice (a2c_lattice_fcc).

    Returns (X, xH, surface, box, nPd, nH).  With device_out = (dX, dxH,
    dsurface, stream) -- device pointers, a stream handle -- the lattice is
    generated on the GPU instead (a2c_lattice_fcc_device) and None is
    returned."""
    if isinstance(ncell, int):
        ncell = (ncell, ncell, ncell)
    sp = N.LatticeSpec()
    for d in range(3):
        sp.ncell[d] = int(ncell[d])
        sp.periodic[d] = int(bool(periodic[d]))
    sp.a, sp.pos_std = a, pos_std
    sp.sigma_lo, sp.sigma_hi = float(sigma[0]), float(sigma[1])
    sp.x_mode, sp.x_center, sp.x_half = x_mode, x_center, x_half
    sp.x_matrix, sp.x_nucleus, sp.nucleus_radius, sp.interface_width = x_matrix, x_nucleus, nucleus_radius, \
        interface_width
    sp.xLb, sp.xUb, sp.seed = xLb, xUb, seed
    if device_out is not None:  # (dX, dxH, dsurface) device pointers, stream
        dX, dxH, dsf, stream = device_out
        N.check(N.lib().a2c_lattice_fcc_device(C.byref(sp), dX, dxH, dsf, stream), "a2c_lattice_fcc_device")
        return None
    nc = int(ncell[0]) * int(ncell[1]) * int(ncell[2])
    nPd = nH = 4 * nc
    X = np.empty(4 * (nPd + nH))
    xH = np.empty(nH)
    surf = np.empty(nH, dtype=np.int32)
    N.check(N.lib().a2c_lattice_fcc(C.byref(sp), N.ptr(X), N.ptr(xH), N.ptr(surf)), "a2c_lattice_fcc")
    box = tuple(float(ncell[d]) * a for d in range(3))
    return X, xH, surf, box, nPd, nH


def _tile_candidates(ms) -> list:
    """The tuner's ten candidates in the order it times them (threads per
    site at 256-thread blocks, then the pass-1 block, then the pass-2 block;
    the later stages at the earlier stages' winners) with their ms."""
    ms = [float(v) for v in ms]
    tps = (1, 2, 4, 8)
    t1 = tps[int(np.argmin(ms[0:4]))]
    best = min(range(4), key=lambda k: ms[k])
    cands = [(q, 256, 256) for q in tps]
    rb = (256, 512, 768)
    cands += [(t1, q, 256) for q in rb]
    b_ms = ms[best]
    r1 = 256
    for k, q in enumerate(rb):
        if ms[4 + k] < b_ms:
            b_ms, r1 = ms[4 + k], q
    cands += [(t1, r1, q) for q in (128, 256, 512)]
    return list(zip(cands, ms))


def batch_workload(n: int = 256, edge=(4, 16), T=(200.0, 600.0), x_mean=(0.01, 0.70), x_jitter: float = 0.02,
                   pos_std: float = 0.02, sigma: float = 0.10, seed: int = 4):
    """The batched-instances workload: n independent periodic fcc Pd + H
    lattices, instance k with edge ~ U{edge[0]..edge[1]} cells, T ~ U(T),
    mean occupancy ~ U(x_mean) with per-site jitter U(-x_jitter, x_jitter)
    (clamped to [1e-3, 1 - 1e-16]), N(0, pos_std) positions, sigma fixed.
    The per-instance draws come from numpy's PCG64 seeded with `seed`,
    instance after instance; instance k's lattice is a2c_lattice_fcc with
    seed 1000 * seed + k.

    Returns (instances, X, xH): the dicts Batch() takes and the concatenated
    state and occupancy."""
    rng = np.random.Generator(np.random.PCG64(seed))
    instances, Xs, xs = [], [], []
    for k in range(n):
        e = int(rng.integers(edge[0], edge[1] + 1))
        t = float(rng.uniform(T[0], T[1]))
        xm = float(rng.uniform(x_mean[0], x_mean[1]))
        X, xH, _, box, nPd, nH = lattice_fcc(e, periodic=(1, 1, 1), pos_std=pos_std, sigma=(sigma, sigma),
                                             x_center=xm, x_half=x_jitter, seed=1000 * seed + k)
        instances.append({"nPd": nPd, "nH": nH, "T": t, "box": box, "periodic": (1, 1, 1), "edge": e,
                          "x_mean": xm})
        Xs.append(X)
        xs.append(xH)
    return instances, np.concatenate(Xs), np.concatenate(xs)
