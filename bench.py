#!/usr/bin/env python
"""GPP-EAM objective+gradient throughput on GB300 (atom-evals/s).

Workload: the evaluator-throughput configuration -- an fcc Pd lattice of
32x32x32 cells with its octahedral H sites (131,072 Pd + 131,072 H =
262,144 sites), periodic in x, y, z, positions perturbed by N(0, 0.03 A),
sigma ~ U(0.08, 0.14) A, occupancy ~ U(0, 0.3) clamped to >= 1e-3, T = 300 K,
seeded synthetic data generated in-process.  One step = one objective +
gradient evaluation (both quadrature passes and the free-entropy reduction)
at a fixed state; one atom-eval = one site's contribution.

Headline `value`: the mixed-precision form (FP32 pair quadrature,
compensated per-site sums, FP64 per-site finish, the objective summed as
64.64 fixed point), device-resident inputs, CUDA
events on the evaluator's stream, L2 (129 MB) flushed by writing a 256 MB
buffer before every step.  Also reported: the FP64 plain form, the errors of
the mixed form against it, `e2e` through the public host-pointer entry
point a2c_gpp_eval (pinned host input and output copied every step), the
roofline of the dominant kernel (pass 2), the CPU oracle as a baseline, and
the SM clocks sampled during the timed region.

Multi-GPU (torchrun): every rank evaluates its own replica (weak scaling, no
data-path collective); `value` is the sum over ranks of atom-evals divided
by the slowest rank's device time.

--impl reference times the reference's CPU algorithm (the oracle port with
the reference's redundant finite-difference calls, all host threads) on the
same 262,144-site workload, without loading this repository's library.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GPP-EAM objective+grad atom-evals/s & time-to-minimum, mixed vs FP64 on GB300"
UNIT = "atom-evals/s"
WORKLOAD = dict(ncell=32, periodic=(1, 1, 1), pos_std=0.03, sigma=(0.08, 0.14), x_center=0.15, x_half=0.15, seed=2)


def config_dict(extra=None):
    c = {"workload": "evaluator throughput: fcc Pd 32x32x32 cells + octahedral H, periodic, 262,144 sites, "
                     "N(0,0.03 A) positions, sigma~U(0.08,0.14) A, x~U(0,0.3), T=300 K",
         "sites": 262144, "quadrature_points": 12, "cutoff_A": 5.35, "l2": "flushed (256 MB write) before each step"}
    if extra:
        c.update(extra)
    return c


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(v: float, world: int, device=None) -> float:
    """The slowest rank's value (device time) -- the only collective: it is
    timing bookkeeping, not part of the evaluator's data path."""
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(sites_per_rank: int, steps: int, world: int, max_time_s: float) -> float:
    """Replicas (weak scaling): every rank evaluates its own lattice of
    `sites_per_rank` sites `steps` times; atom-evals of all ranks divided by
    the slowest rank's time."""
    return world * sites_per_rank * steps / max_time_s


def replica_seed(base: int, rank: int) -> int:
    """Each rank draws an independent replica of the workload."""
    return base + rank


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"a2c_gb300_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        # sampling is live before the timed region starts (nvidia-smi takes
        # a moment to print its first sample)
        t0 = time.perf_counter()
        while self.proc and self.proc.poll() is None and time.perf_counter() - t0 < 3.0:
            self.fh.flush()
            if self.path.exists() and self.path.stat().st_size > 0:
                break
            time.sleep(0.01)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if not self.proc or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


# The sources that decide what the mixed kernels read and write: a traffic
# figure captured for other sources is stale.
KERNEL_SOURCES = ("k_mixed.cu", "internal.cuh", "tables.h", "tables.cpp")
TRAFFIC_FILE = ROOT / "profiles" / "traffic.json"


def kernel_source_sha() -> str:
    import hashlib

    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        h.update((ROOT / "a2c_gb300" / "csrc" / f).read_bytes())
    return h.hexdigest()[:16]


def traffic_from_ncu(csv_path: str, sites: int, bench_sites: int = 262144) -> dict:
    """Per-launch DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum)
    of every captured kernel in an ncu CSV (--csv --log-file), averaged over
    its launches and scaled from the captured case's `sites` to one
    `bench_sites` launch; keyed by the kernel's base name."""
    import csv

    per = {}
    with open(csv_path, newline="") as fh:
        rows = [r for r in csv.reader(fh) if r]
    head = next(i for i, r in enumerate(rows) if "Metric Name" in r)
    cols = rows[head]
    ki, mi, vi, ui = (cols.index(k) for k in ("Kernel Name", "Metric Name", "Metric Value", "Metric Unit"))
    idi = cols.index("ID")
    scale = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9}
    for r in rows[head + 1:]:
        if len(r) <= max(ki, mi, vi) or not r[mi].startswith("dram__bytes_"):
            continue
        name = r[ki].split("(")[0].split("<")[0].strip().split(" ")[-1].split("::")[-1]
        v = float(r[vi].replace(",", "")) * scale.get(r[ui], 1.0)
        per.setdefault(name, {}).setdefault(r[idi], 0.0)
        per[name][r[idi]] += v
    out = {}
    for name, launches in per.items():
        out[name] = sum(launches.values()) / len(launches) * bench_sites / sites
    return out


def write_traffic(csv_paths: str, sites: int) -> dict:
    """profiles/traffic.json from ncu captures of the profile case (one CSV
    per captured kernel, comma-separated paths), keyed by the hash of the
    kernel sources they were captured with."""
    k = {}
    for path in csv_paths.split(","):
        k.update(traffic_from_ncu(path, sites))
    doc = {"source_sha16": kernel_source_sha(), "captured_sites": sites, "scaled_to_sites": 262144,
           "bytes_per_launch": k,
           "note": "dram__bytes_read.sum + dram__bytes_write.sum per launch (ncu starts each launch with flushed "
                   "caches), averaged over the captured launches and scaled to a 262,144-site launch by the site "
                   "count"}
    TRAFFIC_FILE.write_text(json.dumps(doc, indent=1) + "\n")
    return doc


def measured_traffic(kernels):
    """DRAM bytes per 262,144-site launch of `kernels` summed, from
    profiles/traffic.json when it was captured for the current kernel
    sources; else (None, why)."""
    try:
        doc = json.loads(TRAFFIC_FILE.read_text())
    except Exception:
        return None, "no profiles/traffic.json"
    if doc.get("source_sha16") != kernel_source_sha():
        return None, f"stale: profiles/traffic.json was captured for kernel sources {doc.get('source_sha16')}, " \
                     f"these are {kernel_source_sha()}"
    b = doc.get("bytes_per_launch", {})
    if not all(k in b for k in kernels):
        return None, "profiles/traffic.json lacks " + ", ".join(k for k in kernels if k not in b)
    return sum(b[k] for k in kernels), "ncu capture of these kernel sources (profiles/traffic.json)"


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return json.loads(p.read_text())
    except Exception:
        return {}


def workload_lattice(ncell=None):
    """The evaluator-throughput lattice from the oracle's generator (the
    same values as the library's a2c_lattice_fcc, without loading the
    library): (X, xH, surface, box, nPd, nH)."""
    from oracle import oracle as O

    w = dict(WORKLOAD)
    if ncell:
        w["ncell"] = ncell
    return O.lattice_fcc(w["ncell"], periodic=w["periodic"], pos_std=w["pos_std"], sigma=w["sigma"],
                         x_center=w["x_center"], x_half=w["x_half"], seed=w["seed"])


def cpu_sample(threads: int, max_evals: int = 4, seconds: float = 20.0):
    """The oracle (reference arithmetic, the reference's redundant FD calls)
    on the full 262,144-site workload: `max_evals` evaluations, fewer when
    they would exceed `seconds`; returns (atom-evals/s, evals, sites)."""
    from oracle import oracle as O

    X, xH, _, box, nPd, nH = workload_lattice()
    pb = O.Problem(nPd, nH, box=box, periodic=WORKLOAD["periodic"])
    off, nbr, *_ = O.neighbors(pb, X)
    t0 = time.perf_counter()
    n = 0
    while n < max_evals and (n == 0 or (time.perf_counter() - t0) * (n + 1) / n < seconds):
        O.evaluate(pb, X, xH, off, nbr, mode=1, threads=threads)
        n += 1
    dt = time.perf_counter() - t0
    return (nPd + nH) * n / dt, n, nPd + nH


def nucleus_lattice(cells: int, seed: int = 3):
    """The mixed-minimization workload drawn at `cells`^3 cells: a spherical
    hydride nucleus (x = 0.60) with a 5 A tanh interface in an x = 0.02
    matrix, radius 80 A at 64^3 cells scaled with the box; N(0, 0.02 A)
    positions, sigma = 0.10 A, periodic, T = 300 K."""
    import a2c_gb300 as A

    return A.lattice_fcc(cells, periodic=(1, 1, 1), pos_std=0.02, sigma=(0.1, 0.1), x_mode=1, x_matrix=0.02,
                         x_nucleus=0.60, nucleus_radius=80.0 * cells / 64.0, interface_width=5.0, x_half=0.0,
                         seed=seed)


def time_to_minimum(cells: int, gatol: float, device: int, fp64_cap: int = 0, polish_cap: int = 0,
                    gatol_mixed: float = 1e-6):
    """Wall time of a2c_gpp_minimize to `gatol` in FP64 and in mixed
    precision on the hydride-nucleus lattice, and how far the mixed results
    are from the FP64 minimum.

    FP64 runs twice: host-driven (its sums in the single-system order) and
    device-driven by the batched engine (sums in chunks of 2048 terms).  The
    two are the same algorithm on the same objective; their distance
    (`fp64_vs_fp64_spread`) is how well `gatol` determines the minimum at
    all, and every mixed error is reported beside it.  The mixed form runs
    alone (gatol on its own gradient) and followed by the FP64 polish
    (gatol on the FP64 gradient), both to the same `gatol`, and alone to
    `gatol_mixed` (the configuration's 1e-6, below the FP64 form's
    finite-difference floor at this size).  With fp64_cap > 0 the FP64 runs
    stop after fp64_cap iterations and the FP64 time is extrapolated
    (labelled); polish_cap > 0 caps the polish iterations."""
    import numpy as np

    import a2c_gb300 as A

    X, xH, _, box, nPd, nH = nucleus_lattice(cells)
    out = {"cells": cells, "sites": nPd + nH, "gatol": gatol}
    kw = dict(gatol=gatol, max_it=20000, max_fev=40000)

    def state_err(Xa, Xb):
        a, b = Xa.reshape(-1, 4), Xb.reshape(-1, 4)
        return float(np.abs(a[:, :3] - b[:, :3]).max()), float(np.abs(a[:, 3] - b[:, 3]).max())

    with A.Gpp(nPd, nH, box=box, periodic=(1, 1, 1), device=device) as g:
        g.set_occupancy(xH)
        g.build_neighbors(X)
        g.eval(X)  # warm-up (lazy set-up of both forms)
        g.set_precision("mixed")
        g.eval(X)
        out["autotune_tile"] = list(g.autotune_tile()[0])
        g.set_precision("fp64")
        fp64 = {}
        for name, drv in (("fp64", "default"), ("fp64_device_engine", "device")):
            g.set_minimizer(drv)
            t0 = time.perf_counter()
            r = g.minimize(X, **(dict(kw, max_it=fp64_cap) if fp64_cap else kw))
            fp64[name] = (r, time.perf_counter() - t0)
        g.set_minimizer("default")
        g.set_precision("mixed")
        runs = {}
        for name, polish, gt in (("mixed_no_polish", 0, gatol), ("mixed", 1, gatol),
                                 ("mixed_no_polish_gatol_mixed", 0, gatol_mixed)):
            kwr = dict(kw, gatol=gt)
            if polish and polish_cap:
                kwr["max_it"] = runs["mixed_no_polish"][0].iters + polish_cap
            t0 = time.perf_counter()
            r = g.minimize(X, polish=polish, **kwr)
            runs[name] = (r, time.perf_counter() - t0)
        g.set_precision("fp64")
        f64_at, g64_at = {}, {}
        for name, (r, _) in runs.items():
            fv, gv = g.eval(r.X)
            f64_at[name] = fv
            g64_at[name] = float(np.linalg.norm(gv))
    r64, t64 = fp64["fp64"]
    for name, (r, t) in fp64.items():
        out[name] = {"seconds": t, "iters": r.iters, "nfev": r.nfev, "reason": r.reason, "gnorm": r.gnorm,
                     "sigma_range_A": [float(r.X[3::4].min()), float(r.X[3::4].max())], "f": r.fmin,
                     "seconds_per_iter": t / max(r.iters, 1)}
    r64e = fp64["fp64_device_engine"][0]
    dq, ds = state_err(r64.X, r64e.X)
    out["fp64_vs_fp64_spread"] = {"free_entropy_rel": abs(r64.fmin - r64e.fmin) / abs(r64.fmin),
                                  "max_position_A": dq, "max_sigma_A": ds,
                                  "what": "FP64 host-driven vs FP64 device-engine minimum (two summation orders)"}
    if fp64_cap:
        need = runs["mixed_no_polish"][0].iters
        out["fp64"].update(capped_at_iters=fp64_cap, extrapolated_seconds=t64 / max(r64.iters, 1) * need,
                           extrapolation="FP64 seconds per iteration x iterations of the mixed phase (a low "
                                         "estimate)")
    t64_ref = out["fp64"].get("extrapolated_seconds", t64)
    t64_best = min(t64_ref, fp64["fp64_device_engine"][1]) if not fp64_cap else t64_ref
    for name, (r, t) in runs.items():
        out[name] = {"seconds": t, "gatol": kw["gatol"] if name != "mixed_no_polish_gatol_mixed" else gatol_mixed,
                     "iters": r.iters, "mixed_iters": r.mixed_iters, "fp64_polish_iters": r.fp64_iters,
                     "sigma_range_A": [float(r.X[3::4].min()), float(r.X[3::4].max())],
                     "mixed_phase_gnorm": r.mixed_gnorm, "nfev": r.nfev, "reason": r.reason, "gnorm": r.gnorm,
                     "fp64_gnorm_at_result": g64_at[name], "speedup_vs_fp64": t64_ref / t,
                     "speedup_vs_fastest_fp64": t64_best / t}
        if not fp64_cap:
            dq, ds = state_err(r.X, r64.X)
            out[name]["vs_fp64_minimum"] = {"free_entropy_rel": abs(f64_at[name] - r64.fmin) / abs(r64.fmin),
                                            "max_position_A": dq, "max_sigma_A": ds,
                                            "fp64_vs_fp64_spread_position_A": out["fp64_vs_fp64_spread"][
                                                "max_position_A"]}
        else:
            out[name]["free_entropy_fp64_at_result"] = f64_at[name]
    return out


def dmd_slab(cells_xy: int, cells_z: int, seed: int = 5):
    """The coupled-DMD workload: fcc Pd + octahedral H, periodic in x and y,
    free surfaces in z, x = 0.01 everywhere, N(0, 0.02 A) positions, sigma =
    0.10 A; the H sites of the z = 0 layer are the Dirichlet sites."""
    import numpy as np

    import a2c_gb300 as A

    X, xH, surf, box, nPd, nH = A.lattice_fcc((cells_xy, cells_xy, cells_z), periodic=(1, 1, 0), pos_std=0.02,
                                             sigma=(0.1, 0.1), x_center=0.01, x_half=0.0, seed=seed)
    return X, xH, np.nonzero(surf)[0].astype(np.int32), box, nPd, nH


def dirichlet_gamma(T: float, x_bd: float, device: int) -> float:
    """gamma_bd: the mean chemical potential (gamma, with its +1.5 offset) of
    a periodic 4x4x4-cell crystal held at x = x_bd after minimization -- the
    value a bulk region at the Dirichlet occupancy has."""
    import numpy as np

    import a2c_gb300 as A

    X, xH, _, box, nPd, nH = A.lattice_fcc(4, periodic=(1, 1, 1), pos_std=0.0, sigma=(0.1, 0.1), x_center=x_bd,
                                           x_half=0.0, seed=1)
    with A.Gpp(nPd, nH, T=T, box=box, periodic=(1, 1, 1), device=device) as g:
        g.set_occupancy(xH)
        g.build_neighbors(X)
        r = g.minimize(X, gatol=1e-6)
        gam, _ = g.chem_potential(1e300, np.zeros(nH), np.zeros(nH, dtype=np.int32))
    return float(np.mean(gam))


def depth_profile(X, xH, nPd: int, a: float = 3.89):
    """Mean H occupancy per z-layer of octahedral sites (spacing a/2); X is
    the lattice state the layers are read from (the initial one: relaxed
    subsurface sites can move by more than a/4)."""
    import numpy as np

    z = X.reshape(-1, 4)[nPd:, 2]
    layer = np.rint(z / (0.5 * a)).astype(np.int64)
    layer -= layer.min()
    cnt = np.bincount(layer)
    return np.bincount(layer, weights=xH) / np.maximum(cnt, 1)


def run_dmd_case(args):
    """Coupled diffusive MD: `--dmd-steps` outer steps (minimization to
    gatol 1e-5 in the mixed form -- FP32 quadrature, FP64 L-BFGS, rates and
    occupancy update -- then one diffusion step) on a cells x cells x cells
    slab, T = 400 K, Dirichlet x = 0.80 on the z = 0 H layer, nu = 1e13 /s,
    Qm = 0.23 eV, dt = 1e-12 s (12 nu exp(-Qm/kT) dt = 0.15).  Reported: wall
    time per outer step, total H per step and the final depth profile; then
    the same protocol on a reduced 8x8x12-cell slab in FP64 and mixed, whose
    FP64 loop is bit-identical to the oracle's."""
    import numpy as np

    import a2c_gb300 as A

    dev = dist_env()[2]
    T, x_bd = 400.0, 0.80
    dmd = dict(dt=1e-12, nu=1e13, Qm=0.23, x_bd=x_bd, xLb=1e-3, xUb=1 - 1e-16)
    gbd = dirichlet_gamma(T, x_bd, dev)
    out = {"case": "coupled DMD", "T": T, "x_bd": x_bd, "gamma_bd": gbd, **{k: v for k, v in dmd.items()}}

    def run(cells_xy, cells_z, prec, steps):
        X, xH, bd, box, nPd, nH = dmd_slab(cells_xy, cells_z)
        with A.Gpp(nPd, nH, T=T, box=box, periodic=(1, 1, 0), precision=prec, device=dev) as g:
            g.set_occupancy(xH)
            g.build_neighbors(X)
            g.eval(X)  # lazy set-up outside the timed region
            g.synchronize()
            t0 = time.perf_counter()
            r = g.dmd_run(X, xH, np.zeros(nH), np.zeros(nH, dtype=np.int32), bd, bd, steps, gamma_bd=gbd,
                          gatol=1e-5, max_it=2000, polish=0, **dmd)
            dt = time.perf_counter() - t0
        return r, dt, nPd + nH, depth_profile(X, r["xH"], nPd)

    c = args.dmd_cells
    r, dt, n, prof = run(c, c, "mixed", args.dmd_steps)
    out["full"] = {"cells": [c, c, c], "sites": n, "steps": args.dmd_steps, "precision": "mixed",
                   "wall_s": dt, "wall_s_per_outer_step": dt / max(args.dmd_steps, 1),
                   "iters_per_step": r["iters"].tolist(), "xH_total": r["xH_mean"].tolist(),
                   "depth_profile_first_layers": prof[:12].tolist()}
    ks = args.dmd_ref_steps
    r64, t64, nr, p64 = run(8, 12, "fp64", ks)
    rmx, tmx, _, pmx = run(8, 12, "mixed", ks)
    out["reduced"] = {"cells": [8, 8, 12], "sites": nr, "steps": ks,
                      "fp64": {"wall_s_per_outer_step": t64 / ks, "xH_total": r64["xH_mean"].tolist(),
                               "iters_per_step": r64["iters"].tolist()},
                      "mixed": {"wall_s_per_outer_step": tmx / ks, "xH_total": rmx["xH_mean"].tolist(),
                                "iters_per_step": rmx["iters"].tolist()},
                      "xH_total_rel_err": float(np.max(np.abs(rmx["xH_mean"] - r64["xH_mean"]) / r64["xH_mean"])),
                      "profile_max_abs_err": float(np.max(np.abs(pmx - p64))),
                      "occupancy_max_abs_err": float(np.max(np.abs(rmx["xH"] - r64["xH"])))}
    print(json.dumps({"coupled_dmd": out}))
    return 0


def run_batch_case(args):
    """Batched uneven instances: `--batch-n` independent periodic lattices
    (edge ~ U{4..16} cells, T ~ U(200, 600) K, mean x ~ U(0.01, 0.70) +-
    0.02, N(0, 0.02 A) positions, sigma = 0.10 A; 256 lattices = 3,040,448
    sites) minimized to gatol 1e-6 as one batch, every L-BFGS tick a
    replayed CUDA graph, instances retiring as they converge, threads per
    site chosen by the library's autotuner.  Two mixed-precision runs: the
    mixed form alone (gatol on its gradient; FP32 quadrature, FP64 L-BFGS)
    and the mixed form followed by the FP64 polish (gatol on the FP64
    gradient).  Reported: time to finish the whole batch, aggregate
    atom-evals/s (sum over instances of sites x evaluations / device time).
    On every `--batch-stride`-th instance: the plain FP64 path looped
    instance by instance (a2c_gpp_minimize, the baseline), the mixed path
    looped, and one FP64 batch; loop times are scaled to the whole batch by
    sites (labelled extrapolated); the mixed results' distance to the FP64
    minima of the same instances."""
    import numpy as np

    import a2c_gb300 as A

    dev = dist_env()[2]
    inst, X, xH = A.batch_workload(n=args.batch_n)
    sizes = np.array([i["nPd"] + i["nH"] for i in inst])
    so = np.concatenate([[0], np.cumsum(sizes)])
    ho = np.concatenate([[0], np.cumsum([i["nH"] for i in inst])])
    kw = dict(gatol=1e-6, max_it=5000, max_fev=10000)
    out = {"case": "batched instances", "instances": len(inst), "sites": int(sizes.sum()),
           "edge_cells": [int(i["edge"]) for i in inst], "gatol": 1e-6}

    def reasons(r):
        return {int(k): int(v) for k, v in zip(*np.unique(r.reason, return_counts=True))}

    def by_reason(r):
        """Per stopping reason: instances, their sites and their atom-evals
        (so that the work of instances that stalled above gatol is told
        apart from that of converged ones)."""
        out = {}
        for k in np.unique(r.reason):
            sel = r.reason == k
            out[int(k)] = {"instances": int(sel.sum()), "sites": int(sizes[sel].sum()),
                           "atom_evals": float((sizes[sel] * r.nfev[sel]).sum())}
        return out

    res = {}
    with A.Batch(inst, precision="mixed", device=dev) as b:
        b.set_occupancy(xH)
        t0 = time.perf_counter()
        b.build_neighbors(X)
        out["neighbor_build_s"] = time.perf_counter() - t0
        tile, cands = b.autotune_tile(X)
        out["autotune"] = {"tile": {"threads_per_site": tile[0], "pass1_block": tile[1], "pass2_block": tile[2]},
                           "candidates_ms": {"x".join(map(str, t)): ms for t, ms in cands}}
        for name, polish in (("mixed_batch", 0), ("mixed_polish_batch", 1))[:1 if args.batch_mixed_only else 2]:
            t0 = time.perf_counter()
            r = b.minimize(X, polish=polish, **kw)
            wall = time.perf_counter() - t0
            evals = float((sizes * r.nfev).sum())
            res[name] = r
            out[name] = {"wall_s": wall, "device_s": r.seconds, "ticks": r.ticks, "atom_evals": evals,
                         "atom_evals_per_s": evals / r.seconds, "reasons": reasons(r), "by_reason": by_reason(r),
                         "mixed_iters_mean": float(r.mixed_iters.mean()),
                         "fp64_polish_iters_mean": float(r.fp64_iters.mean()),
                         "fp64_polish_iters_max": int(r.fp64_iters.max()), "nfev_max": int(r.nfev.max())}
            print(json.dumps({name: out[name]}), flush=True)
    if args.batch_mixed_only:  # the mixed batch alone (no polish run, no comparison loops)
        print(json.dumps(out))
        return 0
    sub = list(range(0, len(inst), args.batch_stride))
    sub_sites = int(sizes[sub].sum())
    scale = float(sizes.sum()) / sub_sites
    Xs = [X[4 * so[k]:4 * so[k + 1]] for k in range(len(inst))]
    hs = [xH[ho[k]:ho[k + 1]] for k in range(len(inst))]
    loops, loopX = {}, {}
    for prec, polish in (("fp64", 1), ("mixed", 0)):
        tot, ev = 0.0, 0.0
        for k in sub:
            it = inst[k]
            with A.Gpp(it["nPd"], it["nH"], T=it["T"], box=it["box"], periodic=it["periodic"], precision=prec,
                       device=dev) as g:
                g.set_occupancy(hs[k])
                g.build_neighbors(Xs[k])
                g.eval(Xs[k])
                t0 = time.perf_counter()
                rr = g.minimize(Xs[k], polish=polish, **kw)
                tot += time.perf_counter() - t0
                ev += (it["nPd"] + it["nH"]) * rr.nfev
                if prec == "fp64":
                    loopX[k] = (rr.X, rr.fmin)
        loops[prec] = {"subset_s": tot, "subset_atom_evals_per_s": ev / tot,
                       "extrapolated_whole_batch_s": tot * scale}
        print(json.dumps({prec + "_loop": loops[prec]}), flush=True)
    sub_inst = [inst[k] for k in sub]
    with A.Batch(sub_inst, precision="fp64", device=dev) as b:
        Xsub = np.concatenate([Xs[k] for k in sub])
        b.set_occupancy(np.concatenate([hs[k] for k in sub]))
        b.build_neighbors(Xsub)
        b.eval(Xsub)
        t0 = time.perf_counter()
        r64 = b.minimize(Xsub, **kw)
        t64 = time.perf_counter() - t0
        X64 = b.split(r64.X)
    acc = {}
    for name in ("mixed_batch", "mixed_polish_batch"):
        r = res[name]
        dq, df = 0.0, 0.0
        for j, k in enumerate(sub):
            a = r.X[4 * so[k]:4 * so[k + 1]].reshape(-1, 4)
            c = X64[j].reshape(-1, 4)
            dq = max(dq, float(np.abs(a[:, :3] - c[:, :3]).max()))
            df = max(df, abs(r.fmin[k] - r64.fmin[j]) / abs(r64.fmin[j]))
        acc[name] = {"max_position_A": dq, "max_free_entropy_rel": df}
    # the same FP64 minimization in two reduction orders (looped vs batched):
    # how well gatol 1e-6 determines the minimum at all
    dq, df = 0.0, 0.0
    for j, k in enumerate(sub):
        a = loopX[k][0].reshape(-1, 4)
        c = X64[j].reshape(-1, 4)
        dq = max(dq, float(np.abs(a[:, :3] - c[:, :3]).max()))
        df = max(df, abs(loopX[k][1] - r64.fmin[j]) / abs(r64.fmin[j]))
    acc["fp64_loop_vs_fp64_batch"] = {"max_position_A": dq, "max_free_entropy_rel": df}
    out["subset"] = {"instances": len(sub), "sites": sub_sites, "scale_to_batch": scale,
                     "fp64_loop": loops["fp64"], "mixed_loop": loops["mixed"],
                     "fp64_batch_s": t64, "fp64_batch_extrapolated_s": t64 * scale,
                     "fp64_batch_reasons": reasons(r64), "mixed_vs_fp64_minima": acc}
    base = loops["fp64"]["extrapolated_whole_batch_s"]
    out["speedup_vs_fp64_loop_extrapolated"] = {k: base / out[k]["wall_s"]
                                                for k in ("mixed_batch", "mixed_polish_batch")}
    print(json.dumps({"batched": out}))
    return 0


def run_reference(args):
    """The reference's CPU path on this host's cores: the oracle restatement
    (pinned bit for bit to the reference's own hot-path sources) with the
    reference's redundant finite-difference calls, OpenMP over sites, on the
    full 262,144-site workload; one objective+gradient evaluation per step.
    Loads no library of this repository: the lattice comes from the
    oracle's own generator."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O

    O.build(ref=False)
    threads = os.cpu_count() or 1
    X, xH, _, box, nPd, nH = workload_lattice()
    pb = O.Problem(nPd, nH, box=box, periodic=WORKLOAD["periodic"])
    t0 = time.perf_counter()
    off, nbr, *_ = O.neighbors(pb, X)
    nbr_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        O.evaluate(pb, X, xH, off, nbr, mode=1, threads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.evaluate(pb, X, xH, off, nbr, mode=1, threads=threads)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = (nPd + nH) * args.steps / tot
    sample = (f"the full workload ({nPd + nH} sites), one objective+gradient evaluation per step, "
              f"{threads} OpenMP threads")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict({"parallelism": "host cores", "same_workload": True}),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "neighbor_build_s": nbr_s,
            "note": "the reference's CPU path: the oracle restatement (bit-exact with the reference's own "
                    "sources where those compile) with its redundant FD calls, OpenMP over sites; the "
                    "reference itself needs PETSc and MPI, absent here"}
    print(json.dumps(line))
    return 0


def run_ours(args):
    import numpy as np
    import torch

    import a2c_gb300 as A
    from a2c_gb300 import flop_model
    from a2c_gb300 import _native as NATIVE

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = local
    w = WORKLOAD
    X, xH, _, box, nPd, nH = A.lattice_fcc(w["ncell"], periodic=w["periodic"], pos_std=w["pos_std"],
                                           sigma=w["sigma"], x_center=w["x_center"], x_half=w["x_half"],
                                           seed=replica_seed(w["seed"], rank))
    Ns = nPd + nH
    g = A.Gpp(nPd, nH, box=box, periodic=w["periodic"], precision="mixed", device=dev)
    g.set_occupancy(xH)
    g.build_neighbors(X)
    # neighbor lists: full cell-list build vs the skin refilter (0.5 A skin)
    nb = {}
    t0 = time.perf_counter()
    g.build_neighbors(X)
    nb["cell_build_ms"] = 1e3 * (time.perf_counter() - t0)
    g.set_neighbor_skin(0.5)
    t0 = time.perf_counter()
    g.update_neighbors(X)
    nb["skin_candidates_build_ms"] = 1e3 * (time.perf_counter() - t0)
    Xpin = torch.empty(4 * Ns, dtype=torch.float64, pin_memory=True)
    Xpin.copy_(torch.from_numpy(np.ascontiguousarray(X).reshape(-1)))

    def refilter_ms(src, reps=5):  # median over calls of a2c_gpp_update_neighbors
        ts, rb = [], 0
        for _ in range(reps):
            t0 = time.perf_counter()
            _, r = g.update_neighbors(src)
            ts.append(1e3 * (time.perf_counter() - t0))
            rb |= int(r)
        return float(np.median(ts)), rb

    # the caller's positions in pinned host memory (as the end-to-end
    # evaluation's), then in pageable memory
    nb["skin_refilter_ms"], rebuilt = refilter_ms(Xpin.numpy())
    nb["skin_refilter_pageable_ms"], rb2 = refilter_ms(X)
    nb["refilter_rebuilt"] = bool(rebuilt | rb2)
    g.set_neighbor_skin(0.0)
    g.build_neighbors(X)
    tot = {k: 0 for k in ("PdPd", "PdH", "HPd", "HH")}
    for lid, k in enumerate(tot):
        o, _ = g.neighbors(lid)
        tot[k] = int(o[-1])
    fl = flop_model.flops(tot["PdPd"], tot["PdH"], tot["HPd"], tot["HH"], Ns)
    fl_once = flop_model.flops_pairs_once(tot["PdPd"], tot["PdH"], tot["HPd"], tot["HH"], Ns)
    n_entries = sum(tot.values())

    stream = torch.cuda.ExternalStream(g.stream, device=dev)
    dX = torch.tensor(X, device=dev)
    dG = torch.empty_like(dX)
    df = torch.empty(1, dtype=torch.float64, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2
    torch.cuda.synchronize()

    def step_profiled():
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        return g.profile_eval(dX.data_ptr(), df.data_ptr(), dG.data_ptr())

    # the library's tile tuner (threads per site, pass-1 and pass-2 block
    # sizes) for each pass 2 pair mode (pairs once: each pair evaluated by
    # one of its sites; both: every site gathers over all its pairs), then
    # the faster mode at its tile
    g.set_state(X)
    tune, tiles = {}, {}
    for mode in (("once", "both") if args.pair_mode == "auto" else (args.pair_mode,)):
        g.set_pair_mode(mode)
        tiles[mode], cands = g.autotune_tile(reps=5)
        tune[mode] = {"x".join(map(str, t)): ms for t, ms in cands}
        step_profiled()
        tune[mode]["chosen_ms"] = min(float(np.sum(step_profiled())) for _ in range(3))
    mode = min(tiles, key=lambda m: tune[m]["chosen_ms"])
    g.set_pair_mode(mode)
    g.set_tile(*tiles[mode])
    best = tiles[mode][0]
    once = g.pair_mode == A.A2C_PAIRS_ONCE

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    def timed(nsteps, nwarm):
        for _ in range(nwarm):
            step_profiled()
        barrier()
        torch.cuda.synchronize()
        stages = []
        for _ in range(nsteps):
            stages.append(step_profiled())
        torch.cuda.synchronize()
        barrier()
        return np.array(stages)

    # clocks: sampled from before the headline's timed steps to the end of
    # the end-to-end steps (the other pair mode and the FP64 steps between)
    clk = ClockSampler(dev).__enter__()
    st_mixed = timed(args.steps, args.warmup)
    f_mixed = df.item()
    G_mixed = dG.cpu().numpy()

    # the other pair mode at its best mapping, for comparison (not the headline)
    modes = {mode: {"tile": list(tiles[mode]), "pass2_ms": float(np.mean(st_mixed[:, 2])),
                    "eval_ms": float(np.mean(st_mixed.sum(axis=1)))}}
    other = "both" if mode == "once" else "once"
    if other in tiles:
        g.set_pair_mode(other)
        g.set_tile(*tiles[other])
        st_other = timed(max(3, args.steps // 2), 2)
        modes[other] = {"tile": list(tiles[other]), "pass2_ms": float(np.mean(st_other[:, 2])),
                        "eval_ms": float(np.mean(st_other.sum(axis=1)))}
        g.set_pair_mode(mode)
        g.set_tile(*tiles[mode])

    # FP64 plain form on the same state
    g.set_precision("fp64")
    st_64 = timed(args.fp64_steps, 1)
    f_64 = df.item()
    G_64 = dG.cpu().numpy()
    g.set_precision("mixed")

    dev_time_mixed = max_over_ranks(float(st_mixed.sum()) * 1e-3, world, dev)
    dev_time_64 = max_over_ranks(float(st_64.sum()) * 1e-3, world, dev)
    value = whole_job_value(Ns, args.steps, world, dev_time_mixed)
    value_64 = whole_job_value(Ns, args.fp64_steps, world, dev_time_64)

    # end to end through the public host-pointer entry point
    Xp = torch.empty(4 * Ns, dtype=torch.float64, pin_memory=True)
    Xp.numpy()[:] = X
    Gp = torch.empty(4 * Ns, dtype=torch.float64, pin_memory=True)
    fbuf = np.zeros(1)
    L = NATIVE.lib()
    import ctypes as C

    fval = C.c_double()

    def e2e_step():
        NATIVE.check(L.a2c_gpp_eval(g.handle, C.c_void_p(Xp.data_ptr()), C.byref(fval), C.c_void_p(Gp.data_ptr())),
                     "a2c_gpp_eval")

    for _ in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e2e_step()
    e2e_t = []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_t.append(time.perf_counter() - t0)
    clk.__exit__(None, None, None)
    clocks = clk.summary()
    e2e_time = max_over_ranks(sum(e2e_t), world, dev)
    fbuf[0] = fval.value
    e2e_value = whole_job_value(Ns, args.steps, world, e2e_time)

    # roofline of the dominant kernel (pass 2) from the timed steps
    pass2_ms = float(np.mean(st_mixed[:, 2]))
    pass1_ms = float(np.mean(st_mixed[:, 1]))
    peak32 = A.peak_flops("fp32", dev)
    peak64 = A.peak_flops("fp64", dev)
    # achieved: the frozen per-atom-eval count (every site's full list) x the
    # sites of one launch; the executed count of the pairs-once kernels
    # (each pair's functions once) is reported beside it as pipe use
    exec2 = fl_once if once else fl["pass2"]
    ach = fl["pass2"] / (pass2_ms * 1e-3)
    pass2_64_ms = float(np.mean(st_64[:, 2]))
    traffic, traffic_src = measured_traffic(["k_grad_once", "k_grad_recv"] if once else ["k_grad_mixed"])
    if traffic is not None:
        traffic *= Ns / 262144.0
    kname = f"k_grad_once<{best}> + k_grad_recv<8> (pass 2, pairs once)" if once else \
        f"k_grad_mixed<{best}> (pass 2)"
    kname += f", {tiles[mode][2]} threads per block"
    roofline = {"bound": "fp32", "kernel": kname, "achieved": ach / 1e12,
                "peak": peak32 / 1e12, "unit": "TFLOP/s", "frac": ach / peak32,
                "peak_source": "measured in this run: FP32 FMA-chain kernel (a2c_gpp_peak_flops); "
                               "MEASURED_PEAKS.json holds only HBM and bf16-tensor peaks and no tensor core "
                               "is used here",
                "flops_per_launch": fl["pass2"], "flops_counted": "frozen model (flop_model.flops)",
                "executed_flops_per_launch": exec2,
                "executed_achieved": exec2 / (pass2_ms * 1e-3) / 1e12,
                "executed_frac": exec2 / (pass2_ms * 1e-3) / peak32, "traffic": traffic,
                "traffic_source": traffic_src,
                "algorithmic_bytes_per_launch": flop_model.algorithmic_bytes(Ns, n_entries),
                "hbm_frac": (flop_model.algorithmic_bytes(Ns, n_entries) / ((pass1_ms + pass2_ms) * 1e-3)) /
                            (measured_peaks().get("hbm_gbs", 6800.0) * 1e9),
                "pass1": {"ms": pass1_ms, "achieved_tflops": fl["pass1"] / (pass1_ms * 1e-3) / 1e12},
                "fp64_plain_pass2": {"ms": pass2_64_ms, "achieved_tflops": fl["pass2"] / (pass2_64_ms * 1e-3) / 1e12,
                                     "peak_tflops": peak64 / 1e12,
                                     "frac": fl["pass2"] / (pass2_64_ms * 1e-3) / peak64}}

    rel_f = abs(f_mixed - f_64) / abs(f_64)
    rel_g = float(np.linalg.norm(G_mixed - G_64) / np.linalg.norm(G_64))

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, n, sites = cpu_sample(threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{n} evaluations of the full workload ({sites} sites), oracle with the reference's "
                         f"arithmetic and redundant FD calls, OpenMP"}

    g.close()
    ttm = None
    if world == 1 and args.ttm_cells > 0:
        ttm = time_to_minimum(args.ttm_cells, args.ttm_gatol, dev)
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": dev_time_mixed * 1e3 / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
                "config": config_dict({"parallelism": f"replicas x{world}", "threads_per_site": best,
                                       "tile": {"threads_per_site": tiles[mode][0], "pass1_block": tiles[mode][1],
                                                "pass2_block": tiles[mode][2]},
                                       "pair_mode": mode, "autotune_ms": tune}),
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * 4 * Ns,
                        "d2h_bytes_per_step": 8 * 4 * Ns + 8},
                "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
                "gpu_launches": (5 if once else 4) * args.steps,  # k_prep, k_rho_mixed, pass 2 (1 or 2), k_objective
                "fp64_plain": {"value": value_64, "unit": UNIT, "steps": args.fp64_steps,
                               "ms_per_step": dev_time_64 * 1e3 / args.fp64_steps},
                "mixed_over_fp64": value / value_64,
                "mixed_error_vs_fp64": {"free_entropy_rel": rel_f, "gradient_rel_2norm": rel_g},
                "stages_ms_mixed": {"prep": float(np.mean(st_mixed[:, 0])), "pass1": pass1_ms, "pass2": pass2_ms,
                                    "reduce": float(np.mean(st_mixed[:, 3]))},
                "pass2_pair_modes": modes, "time_to_minimum": ttm, "neighbor_lists": nb}
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def run_profile_case(args):
    """A small case for ncu captures: a 40x40x40-cell lattice (512,000
    sites; neighbor lists ~165 MB, larger than the 129 MB L2), `--steps`
    mixed evaluations then one FP64 plain evaluation, untimed."""
    import torch

    import a2c_gb300 as A

    w = dict(WORKLOAD, ncell=args.case_cells)
    X, xH, _, box, nPd, nH = A.lattice_fcc(w["ncell"], periodic=w["periodic"], pos_std=w["pos_std"],
                                           sigma=w["sigma"], x_center=w["x_center"], x_half=w["x_half"],
                                           seed=w["seed"])
    with A.Gpp(nPd, nH, box=box, periodic=w["periodic"], precision="mixed") as g:
        g.set_occupancy(xH)
        g.build_neighbors(X)
        if args.case_tile:
            g.set_tile(*[int(v) for v in args.case_tile.split(",")])
        elif args.case_tps:
            g.set_threads_per_site(args.case_tps)
        g.set_pair_mode(args.case_pairs)
        dX = torch.tensor(X, device="cuda")
        dG = torch.empty_like(dX)
        df = torch.empty(1, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for _ in range(args.steps):
            g.eval_device(dX.data_ptr(), df.data_ptr(), dG.data_ptr())
        g.synchronize()
        if args.fp64_steps > 0:
            g.set_precision("fp64")
            g.eval_device(dX.data_ptr(), df.data_ptr(), dG.data_ptr())
            g.synchronize()
    print(json.dumps({"case": "profile", "sites": nPd + nH, "f": df.item()}))
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline sample")
    ap.add_argument("--ttm-cells", type=int, default=32,
                    help="time-to-minimum leg on a cells^3 nucleus lattice (0 = skip; 64 = the full 2,097,152 sites)")
    ap.add_argument("--ttm-gatol", type=float, default=2e-5,
                    help="gradient-norm tolerance both forms run to in the time-to-minimum leg: the tightest both "
                         "reach on their own gradients at 262,144 sites (the FP64 finite-difference gradient floors "
                         "near 5e-6, the mixed one near 1.5e-5 to 2.5e-5)")
    ap.add_argument("--case", choices=["bench", "profile", "ttm", "dmd", "batch"], default="bench",
                    help="profile: the small untimed case used for ncu captures")
    ap.add_argument("--case-cells", type=int, default=40)
    ap.add_argument("--case-tps", type=int, default=0, help="threads per site in the profile case (0 = library)")
    ap.add_argument("--case-tile", default="", help="tile of the profile case: threads per site, pass-1 block, "
                                                    "pass-2 block (e.g. 2,512,256; empty = library)")
    ap.add_argument("--case-pairs", choices=["once", "both"], default="once",
                    help="pass 2 pair mode of the profile case")
    ap.add_argument("--pair-mode", choices=["auto", "once", "both"], default="auto",
                    help="pass 2 pair mode of the evaluator workload (auto: the faster of the two, measured)")
    ap.add_argument("--ttm-fp64-cap", type=int, default=0,
                    help="stop the FP64 time-to-minimum run after this many iterations (0 = run to the end)")
    ap.add_argument("--ttm-polish-cap", type=int, default=0,
                    help="at most this many FP64 polish iterations after the mixed phase (0 = no cap)")
    ap.add_argument("--dmd-cells", type=int, default=48, help="coupled-DMD slab edge in cells")
    ap.add_argument("--dmd-steps", type=int, default=100, help="coupled-DMD outer steps")
    ap.add_argument("--dmd-ref-steps", type=int, default=10, help="outer steps of the reduced FP64/mixed comparison")
    ap.add_argument("--batch-n", type=int, default=256, help="instances of the batched case")
    ap.add_argument("--batch-stride", type=int, default=16, help="every k-th instance forms the looped subset")
    ap.add_argument("--batch-mixed-only", action="store_true",
                    help="batched case: only the mixed-precision batch minimization")
    ap.add_argument("--traffic-from", metavar="CSV[,CSV...]",
                    help="write profiles/traffic.json from ncu CSVs of the profile case (--case-cells cells) "
                         "and exit")
    args = ap.parse_args()
    if args.traffic_from:
        print(json.dumps(write_traffic(args.traffic_from, 8 * args.case_cells ** 3)))
        return 0
    if args.case == "profile":
        return run_profile_case(args)
    if args.case == "dmd":
        return run_dmd_case(args)
    if args.case == "batch":
        return run_batch_case(args)
    if args.case == "ttm":
        print(json.dumps({"time_to_minimum": time_to_minimum(args.ttm_cells, args.ttm_gatol, dist_env()[2],
                                                             args.ttm_fp64_cap, args.ttm_polish_cap)}))
        return 0
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
