"""Frozen algorithmic operation counts for one objective+gradient evaluation.

One atom-eval is one site's pass-1 + pass-2 contribution under the 12-point
quadrature rule.  Counting convention: add, sub, mul, min, max, select and
int<->float conversion = 1; FMA = 2; ex2 / rsqrt (the special-function
unit) = 1; loads = 0.  The counts are those of the closed-form evaluation
in a2c_gb300/csrc/k_mixed.cu (analytic derivatives, one evaluation of each
function per pair-point, F'(rho) once per site) and are used for BOTH
precisions, so the FP64 plain form's extra work -- the reference's
central differences -- is not counted as useful work.

Per neighbor pair (12 pair-points) of site species A and neighbor species B:
  pass 1: 46 (+1 for an H neighbor's occupancy) per pair overhead, plus per
          point 16 (f_Pd from the table) or 7 (f_H by ex2)
            -> Pd neighbor 238, H neighbor 131
  pass 2: 119 (+2 for an H neighbor) per pair overhead, plus per point
          33 (Pd-Pd: f_Pd', phi_Pd, phi_Pd' from the table),
          45 (Pd-H either way: table f_Pd', ex2 f_H', two-ex2 phi, phi'),
          30 (H-H: ex2 f_H', two-ex2 phi, phi')
            -> Pd-Pd 515, Pd-H / H-Pd 661, H-H 481
Per site: pass 1 finish 15 (embedding table), pass 2 finish 25.

Pass 2 with every pair evaluated once (A2C_PAIRS_ONCE): each unordered pair
costs its type's count above plus 28 for the neighbor's share (its width
sum, 18, and the scaled position share, 10); each received share costs 16
(four compensated adds) and each site 10 more to finish.  flops_pairs_once
gives these executed counts; flops() stays the frozen both-sides count.

Algorithmic bytes per atom-eval: the site's own state read twice (16 B),
its CSR bounds and Pd split (20 B) and neighbor entries (4 B each) read once
per pass, occupancy and F'(rho) (8 B), written F'/F (8 B), gradient (32 B)
and energy partials (16 B): 132 + 8 n_neighbors bytes.
"""
from __future__ import annotations

PASS1_PAIR = {"Pd": 238, "H": 131}  # by neighbor species
PASS2_PAIR = {"PdPd": 515, "PdH": 661, "HPd": 661, "HH": 481}
PASS1_SITE = 15
PASS2_SITE = 25


def flops(n_pdpd: int, n_pdh: int, n_hpd: int, n_hh: int, n_sites: int) -> dict:
    """FLOPs of pass 1, pass 2 and the total for one evaluation, from the
    numbers of ordered neighbor pairs of each type (site species first)."""
    p1 = (n_pdpd + n_hpd) * PASS1_PAIR["Pd"] + (n_pdh + n_hh) * PASS1_PAIR["H"] + n_sites * PASS1_SITE
    p2 = (n_pdpd * PASS2_PAIR["PdPd"] + n_pdh * PASS2_PAIR["PdH"] + n_hpd * PASS2_PAIR["HPd"] +
          n_hh * PASS2_PAIR["HH"] + n_sites * PASS2_SITE)
    return {"pass1": float(p1), "pass2": float(p2), "total": float(p1 + p2)}


def algorithmic_bytes(n_sites: int, n_entries: int) -> float:
    """Minimal HBM bytes of one evaluation (both passes)."""
    return float(132 * n_sites + 8 * n_entries)


PASS2_SHARE = 28  # neighbor's share of a pair evaluated once
PASS2_RECV = 16   # one received share, compensated
PASS2_RECV_SITE = 10


def flops_pairs_once(n_pdpd: int, n_pdh: int, n_hpd: int, n_hh: int, n_sites: int) -> float:
    """Executed FLOPs of pass 2 when every pair is evaluated once (by one of
    its sites) and the other site's share is stored and summed."""
    pairs = (n_pdpd // 2) * (PASS2_PAIR["PdPd"] + PASS2_SHARE) + n_hpd * (PASS2_PAIR["HPd"] + PASS2_SHARE) + \
        (n_hh // 2) * (PASS2_PAIR["HH"] + PASS2_SHARE)
    received = (n_pdpd // 2) + n_pdh + (n_hh // 2)
    return float(pairs + received * PASS2_RECV + n_sites * (PASS2_SITE + PASS2_RECV_SITE))
