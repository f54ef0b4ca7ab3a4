"""The C ABI library on a machine without a GPU: it loads, exports every
function include/a2c_gpp.h declares, validates parameters before touching
a device, and its host-side lattice generator is deterministic."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import a2c_gb300 as A
from a2c_gb300 import _native as N

ROOT = Path(__file__).resolve().parent.parent


def declared_functions() -> list[str]:
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        src = h.read_text()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[\w*]+\s+\**(a2c_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    L = N.lib()
    decl = declared_functions()
    assert len(decl) >= 25
    missing = [n for n in decl if not hasattr(L, n)]
    assert not missing, missing
    assert set(N.exported_symbols()) <= set(decl)


def test_status_strings_and_defaults():
    L = N.lib()
    for s in range(0, 9):
        assert L.a2c_status_string(s)
    p = N.GppParams()
    L.a2c_gpp_default_params(C.byref(p))
    assert (p.T, p.QWp, p.eps, p.rc, p.a_Pd, p.precision) == (300.0, 1.0 / 12.0, 1e-5, 5.35, 3.89, 0)
    lp = N.LbfgsParams()
    L.a2c_lbfgs_default_params(C.byref(lp))
    assert lp.m == 5 and lp.gatol == 1e-6 and lp.sigma_lb == 1e-6


def test_invalid_parameters_rejected_before_device():
    L = N.lib()
    p = N.GppParams()
    L.a2c_gpp_default_params(C.byref(p))
    h = C.c_void_p()
    for field, val in (("nPd", -1), ("T", 0.0), ("eps", -1.0), ("rc", 0.0), ("precision", 7)):
        q = N.GppParams.from_buffer_copy(p)
        setattr(q, field, val)
        assert L.a2c_gpp_create(C.byref(q), C.byref(h)) == N.A2C_ERR_INVALID, field
    q = N.GppParams.from_buffer_copy(p)
    q.periodic[0] = 1
    q.box[0] = 10.0  # not more than 2 rc
    assert L.a2c_gpp_create(C.byref(q), C.byref(h)) == N.A2C_ERR_INVALID
    q = N.GppParams.from_buffer_copy(p)
    q.nPd = 1 << 27
    assert L.a2c_gpp_create(C.byref(q), C.byref(h)) == N.A2C_ERR_INVALID


def test_no_device_is_a_status_not_a_crash():
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(A.A2CError) as e:
        A.Gpp(4, 4)
    assert e.value.status == N.A2C_ERR_NO_DEVICE


def test_lattice_generator():
    X, xH, surf, box, nPd, nH = A.lattice_fcc((2, 3, 4), periodic=(1, 1, 0), pos_std=0.0, sigma=(0.1, 0.1),
                                             x_center=0.05, x_half=0.0, seed=1)
    assert nPd == nH == 96 and X.size == 4 * 192 and box == (2 * 3.89, 3 * 3.89, 4 * 3.89)
    q = X.reshape(-1, 4)
    # first cell: Pd basis then (after all Pd) H basis, cells z, y, x
    assert np.allclose(q[:4, :3] / 3.89, [[0, 0, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0]])
    assert np.allclose(q[96:100, :3] / 3.89, [[0.5, 0, 0], [0, 0.5, 0], [0, 0, 0.5], [0.5, 0.5, 0.5]])
    assert np.allclose(q[4, :3] / 3.89, [1, 0, 0])
    assert np.all(q[:, 3] == 0.1) and np.all(xH == 0.05)
    # H sites with lattice z = 0: basis (0.5,0,0), (0,0.5,0), (0.5,0.5,0.5)? only z == 0 ones
    assert surf.sum() == 2 * 2 * 3
    X2, xH2, *_ = A.lattice_fcc((2, 3, 4), pos_std=0.03, sigma=(0.08, 0.14), x_center=0.15, x_half=0.15, seed=2)
    X3, xH3, *_ = A.lattice_fcc((2, 3, 4), pos_std=0.03, sigma=(0.08, 0.14), x_center=0.15, x_half=0.15, seed=2)
    assert np.array_equal(X2, X3) and np.array_equal(xH2, xH3)
    d = X2.reshape(-1, 4)[:, :3] - q[:, :3]
    assert 0.02 < d.std() < 0.04
    s = X2.reshape(-1, 4)[:, 3]
    assert s.min() >= 0.08 and s.max() <= 0.14
    assert xH2.min() >= 1e-3 and xH2.max() <= 0.3


def test_lattice_nucleus_profile():
    X, xH, *_ = A.lattice_fcc(8, x_mode=1, x_matrix=0.02, x_nucleus=0.6, nucleus_radius=8.0, interface_width=0.5,
                              x_half=0.0, seed=3)
    assert abs(xH.max() - 0.6) < 1e-3 and abs(xH.min() - 0.02) < 1e-6
