"""The device lattice generator (a2c_lattice_fcc_device): its deterministic
parts -- lattice positions, fixed widths, the nucleus occupancy profile,
surface flags -- equal the host generator's; its counter-based random draws
follow the same distributions, are reproducible, and depend on the seed."""
import numpy as np
import pytest
import torch

import a2c_gb300 as A

pytestmark = pytest.mark.gpu


def device(cells, **kw):
    nc = int(np.prod(cells)) if not isinstance(cells, int) else cells ** 3
    n = 8 * nc
    dX = torch.empty(4 * n, dtype=torch.float64, device="cuda")
    dx = torch.empty(n // 2, dtype=torch.float64, device="cuda")
    ds = torch.empty(n // 2, dtype=torch.int32, device="cuda")
    A.lattice_fcc(cells, device_out=(dX.data_ptr(), dx.data_ptr(), ds.data_ptr(), None), **kw)
    torch.cuda.synchronize()
    return dX.cpu().numpy(), dx.cpu().numpy(), ds.cpu().numpy()


def test_deterministic_parts_equal_host(gpu):
    for cells, per in ((5, (1, 1, 1)), ((3, 4, 6), (1, 1, 0))):
        kw = dict(periodic=per, pos_std=0.0, sigma=(0.1, 0.1), x_center=0.3, x_half=0.0, seed=4)
        X, xH, surf, *_ = A.lattice_fcc(cells, **kw)
        dX, dx, ds = device(cells, **kw)
        assert np.array_equal(dX, X) and np.array_equal(dx, xH) and np.array_equal(ds, surf)
    kw = dict(pos_std=0.0, sigma=(0.1, 0.1), x_mode=1, x_matrix=0.02, x_nucleus=0.6, nucleus_radius=8.0,
              interface_width=2.0, x_half=0.0, seed=4)
    X, xH, surf, *_ = A.lattice_fcc(6, **kw)
    dX, dx, ds = device(6, **kw)
    assert np.array_equal(dX, X) and np.max(np.abs(dx - xH)) < 1e-15


def test_random_parts(gpu):
    kw = dict(pos_std=0.02, sigma=(0.08, 0.14), x_center=0.15, x_half=0.15, seed=2)
    X0, *_ = A.lattice_fcc(24, **dict(kw, pos_std=0.0, sigma=(0.1, 0.1), x_half=0.0))
    dX, dx, _ = device(24, **kw)
    again, _, _ = device(24, **kw)
    other, _, _ = device(24, **dict(kw, seed=3))
    assert np.array_equal(dX, again) and not np.array_equal(dX, other)
    d = (dX.reshape(-1, 4)[:, :3] - X0.reshape(-1, 4)[:, :3]).ravel()
    n = d.size
    assert abs(d.mean()) < 5 * 0.02 / np.sqrt(n)
    assert abs(d.std() / 0.02 - 1) < 0.01
    sig = dX.reshape(-1, 4)[:, 3]
    assert sig.min() >= 0.08 and sig.max() < 0.14 and abs(sig.mean() - 0.11) < 1e-3
    assert dx.min() >= 1e-3 and dx.max() <= 0.3 and abs(dx.mean() - 0.15) < 2e-3
