"""The invariant the neighbor kernels' FP32 pass rests on (k_neighbors.cu:
prefilter, fp32_decides, pair_test), checked on the host with the same
single-precision operations (numpy float32 rounds every operation as the
kernels do: that translation unit is compiled with -fmad=false).

Whenever the FP32 pass settles a candidate -- inside rc + guard with every
coordinate difference at least guard inside rc and d^2 at least the guard
band away from rc^2, 0.75 a^2 and 1.25 a^2 -- the FP64 test of the reference
(minimum image fixed by the FP32 pass) must accept the pair too, and the
shell class taken from the FP32 values (below 0.75 a^2 / strictly between /
otherwise) must equal the FP64 class.  A candidate the FP32 pass rejects
must be rejected by the FP64 test.  Checked on a perturbed periodic fcc
lattice and on pairs placed at the thresholds within 1e-9..1e-1 A^2, in a
large box (coordinates up to ~120 A, where FP32 spacing is coarsest).
"""
import numpy as np

f32 = np.float32
RC, A = 5.35, 3.89
A75, A125 = 0.75 * A * A, 1.25 * A * A


def shell_class(d2, a75, a125):
    return np.where(d2 < a75, 0, np.where((d2 > a75) & (d2 < a125), 1, 2))


def fp32_pass(xi, xj, box):
    """Vectorised restatement of prefilter + fp32_decides for pairs (xi, xj):
    (inside rc + guard, decided, image m, d2f)."""
    fi, fj = xi.astype(f32), xj.astype(f32)
    boxf = box.astype(f32)
    invboxf = (1.0 / box).astype(f32)
    qmax = np.max(np.abs(np.concatenate([fi, fj])))
    qmax = np.nextafter(f32(qmax), f32(np.inf))  # k_positions_f32: one ulp up
    rcf = f32(RC)
    guard = f32(f32(1e-4) + f32(f32(1.9073486328125e-6) * f32(f32(qmax + f32(boxf.max())) + rcf)))
    lim = f32(rcf + guard)
    dd = fj - fi
    n = np.rint(f32(dd * invboxf[None, :]).astype(f32)).astype(f32)
    dd = f32(dd - f32(n * boxf[None, :]))
    m = -n.astype(np.int64)
    inside = np.all(np.abs(dd) <= lim, axis=1)
    d2f = f32(f32(f32(dd[:, 0] * dd[:, 0]) + f32(dd[:, 1] * dd[:, 1])) + f32(dd[:, 2] * dd[:, 2]))
    inside &= d2f <= f32(lim * lim)
    g = f32(lim - rcf)  # pair_test passes the guard as lim - rc
    band = f32(f32(f32(f32(2.0) * g) * f32(rcf + f32(1.0))) + f32(1e-5))
    inner = f32(rcf - g)
    decided = (inside & np.all(np.abs(dd) < inner, axis=1) & (d2f < f32(f32(RC * RC) - band))
               & (np.abs(f32(d2f - f32(A75))) > band) & (np.abs(f32(d2f - f32(A125))) > band)
               & np.all(np.abs(m) <= 1, axis=1))
    return inside, decided, m, d2f


def fp64_test(xi, xj, box, m):
    """exact_test: the reference's FP64 acceptance with the image m."""
    dd = (xj + m * box[None, :]) - xi
    ok = np.all(np.abs(dd) <= RC, axis=1)
    d2 = dd[:, 0] * dd[:, 0] + dd[:, 1] * dd[:, 1] + dd[:, 2] * dd[:, 2]
    return ok & (d2 <= RC * RC), d2


def check(xi, xj, box):
    inside, decided, m, d2f = fp32_pass(xi, xj, box)
    acc64, d2 = fp64_test(xi, xj, box, m)
    # a pair the FP32 pass rejects is never one the FP64 test accepts
    assert not np.any(acc64 & ~inside)
    # settled pairs: accepted by the FP64 test, in the same shell class
    assert np.all(acc64[decided])
    c32 = shell_class(d2f[decided], f32(A75), f32(A125))
    c64 = shell_class(d2[decided], A75, A125)
    assert np.array_equal(c32, c64)
    return int(decided.sum()), int((inside & ~decided).sum())


def test_lattice_pairs():
    rng = np.random.default_rng(7)
    ncell = 30  # box 116.7 A
    box = np.full(3, ncell * A)
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5], [0.5, 0.5, 0.5], [0.5, 0, 0],
                      [0, 0.5, 0], [0, 0, 0.5]]) * A
    cells = np.stack(np.meshgrid(*[np.arange(ncell)] * 3, indexing="ij"), -1).reshape(-1, 3) * A
    sel = rng.choice(len(cells), 300, replace=False)
    X = (cells[sel][:, None, :] + basis[None, :, :]).reshape(-1, 3) + rng.normal(0, 0.05, (300 * 8, 3))
    # every site against the sites of its neighborhood, through the box edges too
    centre = X[:400]
    offs = np.stack(np.meshgrid(*[np.arange(-2, 3)] * 3, indexing="ij"), -1).reshape(-1, 3) * (A / 2)
    xj = (centre[:, None, :] + offs[None, :, :] + rng.normal(0, 0.05, (400, len(offs), 3))).reshape(-1, 3)
    xj = np.mod(xj, box)  # wrapped into the box: the image is needed
    xi = np.repeat(centre, len(offs), axis=0)
    decided, undecided = check(xi, xj, box)
    assert decided > 10 * undecided > 0


def test_pairs_at_the_thresholds():
    rng = np.random.default_rng(11)
    box = np.full(3, 30 * A)
    n = 20000
    for t2 in (A75, A125, RC * RC):
        for delta in (1e-9, 1e-7, 1e-5, 1e-3, 1e-2, 1e-1):
            d2 = t2 + delta * rng.choice([-1.0, 1.0], n)
            u = rng.normal(size=(n, 3))
            u /= np.linalg.norm(u, axis=1)[:, None]
            xi = rng.uniform(0, box[0], (n, 3))
            xj = np.mod(xi + u * np.sqrt(d2)[:, None], box)
            check(xi, xj, box)
