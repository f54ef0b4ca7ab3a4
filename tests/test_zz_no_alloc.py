"""The allocation-free mixed-precision entry point (a2c_gpp_eval_mixed_noalloc).

It serves callers that cannot allocate device memory while they evaluate
(a solver callback inside another framework's memory pool, or recording
under a driver that forbids allocation); its scratch is a fixed device
array inside the library.  Checked against the context path
(a2c_gpp_eval_device in mixed precision) on two calls in a row: within the
mixed form's tolerances (free entropy 1e-6 relative, gradient 1e-4 in the
2-norm), and, since both run the same pair kernels at the same tile, the
gradient bit for bit in either pair mode.  This file is collected last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import a2c_gb300 as A
from a2c_gb300 import _native as N

pytestmark = pytest.mark.gpu

TOL_F = 1e-6
TOL_G = 1e-4


def noalloc_fn():
    fn = N.lib().a2c_gpp_eval_mixed_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    return fn


# (cells, periodic): a small slab, and the largest lattice the fixed array
# holds (32 x 32 x 16 cells = 131,072 sites)
SIZES = {"slab_8x8x6": ((8, 8, 6), (1, 1, 0)), "max_32x32x16": ((32, 32, 16), (1, 1, 1))}


@pytest.mark.parametrize("size", list(SIZES))
def test_noalloc_matches_context_path_twice(gpu, size):
    import torch

    fn = noalloc_fn()
    cells, per = SIZES[size]
    X, xH, _, box, nPd, nH = A.lattice_fcc(cells, periodic=per, pos_std=0.03, sigma=(0.08, 0.14),
                                           x_center=0.15, x_half=0.15, seed=2)
    with A.Gpp(nPd, nH, box=box, periodic=per, precision="mixed") as g:
        g.set_occupancy(xH)
        g.build_neighbors(X)
        dX = torch.tensor(X, device="cuda")
        dG = torch.empty_like(dX)
        df = torch.empty(1, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        g.eval_device(dX.data_ptr(), df.data_ptr(), dG.data_ptr())
        g.synchronize()
        f_ref, G_ref = df.item(), dG.cpu().numpy()
        for _ in range(2):
            dG2 = torch.full_like(dX, float("nan"))
            df2 = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            assert fn(g.handle, dX.data_ptr(), df2.data_ptr(), dG2.data_ptr()) == N.A2C_OK
            g.synchronize()
            f2, G2 = df2.item(), dG2.cpu().numpy()
            assert abs(f2 - f_ref) <= TOL_F * abs(f_ref)
            assert np.linalg.norm(G2 - G_ref) <= TOL_G * np.linalg.norm(G_ref)
            # the same pair kernels as the context path (pairs once, same
            # tile): the same gradient bits; f differs only in how the
            # per-site terms are summed (FP64 tree here, exact fixed point there)
            assert np.array_equal(G2, G_ref)
            assert abs(f2 - f_ref) <= 1e-12 * abs(f_ref)
        # pairs from both sides: the both-sides pass 2 of the context path
        g.set_pair_mode("both")
        g.eval_device(dX.data_ptr(), df.data_ptr(), dG.data_ptr())
        g.synchronize()
        G_both = dG.cpu().numpy()
        assert fn(g.handle, dX.data_ptr(), df2.data_ptr(), dG2.data_ptr()) == N.A2C_OK
        g.synchronize()
        assert np.array_equal(dG2.cpu().numpy(), G_both)


def test_noalloc_rejects_problems_above_its_fixed_size(gpu):
    import torch

    fn = noalloc_fn()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    with A.Gpp(70000, 70000) as g:  # 140,000 sites > 131,072
        assert fn(g.handle, buf.data_ptr(), buf.data_ptr(), buf.data_ptr()) == N.A2C_ERR_INVALID
