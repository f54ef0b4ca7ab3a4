"""The oracle's lattice generator (orc_lattice_fcc, used by the CPU
baselines so that they never load the library) draws the same lattices as
the library's a2c_lattice_fcc, bit for bit, for every workload shape the
benchmark uses."""
import numpy as np
import pytest

import a2c_gb300 as A
from oracle import oracle as O

SPECS = {
    "throughput": dict(ncell=(5, 5, 5), periodic=(1, 1, 1), pos_std=0.03, sigma=(0.08, 0.14), x_center=0.15,
                       x_half=0.15, seed=2),
    "nucleus": dict(ncell=(6, 6, 6), periodic=(1, 1, 1), pos_std=0.02, sigma=(0.1, 0.1), x_mode=1, x_matrix=0.02,
                    x_nucleus=0.60, nucleus_radius=7.5, interface_width=5.0, x_half=0.0, seed=3),
    "slab": dict(ncell=(4, 3, 7), periodic=(1, 1, 0), pos_std=0.02, sigma=(0.1, 0.1), x_center=0.01, x_half=0.0,
                 seed=5),
    "clamped": dict(ncell=(2, 3, 4), pos_std=0.0, sigma=(0.1, 0.1), x_center=0.0, x_half=0.3, seed=11),
}


@pytest.mark.parametrize("name", list(SPECS))
def test_oracle_lattice_equals_library_lattice(name):
    a = A.lattice_fcc(**SPECS[name])
    b = O.lattice_fcc(**SPECS[name])
    for u, v in zip(a, b):
        if isinstance(u, np.ndarray):
            assert u.dtype == v.dtype and np.array_equal(u, v)
        else:
            assert u == v


def test_oracle_lattice_rejects_bad_sizes():
    with pytest.raises(ValueError):
        O.lattice_fcc((0, 2, 2))
