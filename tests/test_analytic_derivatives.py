"""The mixed form's functions against the reference's (host only, no GPU):
the analytic FP64 derivatives its tables are built from, the reference's
central differences (step eps, potential.cpp:40-205) converging to them at
second order, and the FP32 tables' accuracy over the range the lattices
sample.

Measured along the way: the reference's f_Pd and phi_Pd are polynomials
whose terms cancel by orders of magnitude, so their values carry rounding
of ~1e-12 of their scale, and the reference's own central difference at
eps = 1e-5 amplifies it to 6e-7 (f_Pd) and 2e-7 (phi_Pd) of the
derivative's scale -- the source of the FP64 plain form's gradient noise
floor.  The other functions' FD derivatives are good to ~1e-9."""
import ctypes as C

import numpy as np
import pytest

import a2c_gb300 as A
from oracle import oracle as O

L = A._native.lib()
FUNCS = {0: "F_Pd", 2: "F_H", 4: "f_Pd", 6: "f_H", 8: "phi_Pd", 10: "phi_PdH", 12: "phi_H"}


def analytic(w, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    v, d = np.empty_like(x), np.empty_like(x)
    assert L.a2c_eam_analytic(w, x.ctypes.data, x.size, v.ctypes.data, d.ctypes.data) == 0
    return v, d


def table(w, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    v, d = np.empty_like(x), np.empty_like(x)
    assert L.a2c_mixed_table_eval(w, x.ctypes.data, x.size, v.ctypes.data, d.ctypes.data) == 0
    return v, d


def points(w):
    if w in (0, 2):
        return np.linspace(2.0, 40.0, 397)  # site densities of the lattices: 10-22
    r = np.linspace(1.3, 6.8, 551)
    # stay clear of the branch points, where a central difference straddles two forms
    for b in (5.0, 5.05, 5.35):
        r = r[np.abs(r - b) > 3e-3]
    return r


# values: the polynomial forms cancel, so operation order shows at ~1e-12
VALUE_TOL = {0: 1e-14, 2: 0.0, 4: 2e-11, 6: 0.0, 8: 2e-11, 10: 0.0, 12: 0.0}
# the reference's FD derivative at its own eps = 1e-5, relative to the scale
FD_TOL = {0: 1e-8, 2: 1e-8, 4: 2e-6, 6: 1e-9, 8: 1e-6, 10: 1e-8, 12: 1e-8}


@pytest.mark.parametrize("w", sorted(FUNCS))
def test_values_match_reference_form(w):
    x = points(w)
    v, _ = analytic(w, x)
    ref = O.eam(w, x)
    assert np.max(np.abs(v - ref)) <= VALUE_TOL[w] * np.abs(ref).max(), FUNCS[w]


@pytest.mark.parametrize("w", sorted(FUNCS))
def test_central_differences_converge_at_second_order(w):
    x = points(w)
    if w >= 4:  # the difference must not straddle a branch point
        x = x[np.all([np.abs(x - b) > 0.05 for b in (5.0, 5.05, 5.35)], axis=0)]
    _, d = analytic(w, x)
    err = {}
    for h in (2e-2, 1e-2):
        fd = (O.eam(w, x + h) - O.eam(w, x - h)) / (2 * h)
        err[h] = np.abs(fd - d)
    ratio = np.median(err[2e-2] / np.maximum(err[1e-2], 1e-300))
    assert 3.7 < ratio < 4.3, (FUNCS[w], ratio)
    # the reference's own step eps = 1e-5: O(eps^2) truncation plus rounding
    fd_ref = O.eam(w + 1, x)
    assert np.max(np.abs(fd_ref - d)) <= FD_TOL[w] * np.abs(d).max(), FUNCS[w]


@pytest.mark.parametrize("w,vtol,dtol", [(0, 3e-7, 3e-6), (2, 3e-7, 3e-6), (4, 3e-7, 3e-6), (8, 3e-7, 3e-6)])
def test_fp32_tables(w, vtol, dtol):
    x = points(w)
    v, d = analytic(w, x)
    tv, td = table(w, x)
    assert np.max(np.abs(tv - v)) <= vtol * np.abs(v).max(), FUNCS[w]
    assert np.max(np.abs(td - d)) <= dtol * np.abs(d).max(), FUNCS[w]
