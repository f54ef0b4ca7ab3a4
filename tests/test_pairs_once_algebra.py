"""The algebra behind evaluating each pair once (mixed pass 2, A2C_PAIRS_ONCE),
checked on the host in FP64 against the quadrature written out point by
point.

For a pair of sites a, b with D = q_a - q_b and u = sqrt(6) sigma, the
12-point rule (quadrature.cpp:43-76; electrondensity.cpp:23 for the point
vector) moves one coordinate m of one atom by +-u.  With any per-point
factor c(s) that is symmetric in the two sites (as (F'_a + F'_b) f'(s) +
phi'(s) is), site a's gradient terms are
    dPhi/dq_a     ~ sum_k c_k r_k
    dPhi/dsigma_a ~ sqrt(2) sum_k c_k (r_k . xi0_k)
(minimizer.cpp:172-284), and site b's are the same sums seen from b.  The
kernels fold them per coordinate into csum, e[m], sig (a's side) and sigj
(b's side): b's position share is -(D csum + e) and its width share sigj,
so one evaluation of the 12 factors serves both sites.
"""
import numpy as np

SQ3 = np.sqrt(3.0)


def points(D, ua, ub):
    """(r_k, xi0_k of the centre a, xi0_k seen from b) for the 12 points."""
    out = []
    for m in range(3):
        e = np.zeros(3)
        e[m] = 1.0
        for sgn in (+1.0, -1.0):
            # atom a moved by sgn*ua along m: r = D + sgn ua e; xi0(a) = sgn sqrt3 e
            out.append((D + sgn * ua * e, sgn * SQ3 * e, np.zeros(3)))
        for sgn in (+1.0, -1.0):
            # atom b moved by sgn*ub along m: r = D - sgn ub e; from b, xi0(b) = sgn sqrt3 e
            out.append((D - sgn * ub * e, np.zeros(3), sgn * SQ3 * e))
    return out


def g(s):
    """Any smooth symmetric per-point function (stands in for (F'_a+F'_b) f' + phi')."""
    return np.sin(1.3 * s) * np.exp(-0.4 * s) + 0.2 * s


def both_sides(D, ua, ub):
    """a's and b's gradient sums, each from its own frame, point by point."""
    qa, sa, qb, sb = np.zeros(3), 0.0, np.zeros(3), 0.0
    for r, xa, xb in points(D, ua, ub):
        s = np.linalg.norm(r)
        c = g(s) / s
        qa += c * r
        sa += np.sqrt(2.0) * c * (r @ xa)
        rb = -r  # the same point seen from b: q_b + ... - q_a - ...
        qb += c * rb
        sb += np.sqrt(2.0) * c * (rb @ xb)
    return qa, sa, qb, sb


def closed_form(D, ua, ub):
    """The kernels' per-coordinate folding (k_mixed.cu pair_terms)."""
    A_i, A_j = D @ D + ua * ua, D @ D + ub * ub
    csum, e, sig, sigj = 0.0, np.zeros(3), 0.0, 0.0
    for m in range(3):
        bi, bj = 2.0 * D[m] * ua, 2.0 * D[m] * ub
        s2 = [A_i + bi, A_i - bi, A_j - bj, A_j + bj]  # r = D+ua e, D-ua e, D-ub e, D+ub e
        cpi, cmi, cmj, cpj = [g(np.sqrt(v)) / np.sqrt(v) for v in s2]
        csum += cpi + cmi + cmj + cpj
        e[m] = ua * (cpi - cmi) + ub * (cpj - cmj)
        sig += D[m] * (cpi - cmi) + ua * (cpi + cmi)
        sigj += D[m] * (cpj - cmj) + ub * (cpj + cmj)
    own_q = D * csum + e
    return own_q, np.sqrt(6.0) * sig, -own_q, np.sqrt(6.0) * sigj


def test_share_algebra_matches_pointwise_quadrature():
    rng = np.random.default_rng(11)
    for _ in range(200):
        D = rng.normal(size=3) * 2.0
        D *= rng.uniform(1.8, 5.3) / np.linalg.norm(D)
        ua, ub = np.sqrt(6.0) * rng.uniform(0.05, 0.3, size=2)
        qa, sa, qb, sb = both_sides(D, ua, ub)
        cqa, csa, cqb, csb = closed_form(D, ua, ub)
        scale = max(np.abs(qa).max(), abs(sa), 1e-3)
        assert np.allclose(cqa, qa, rtol=0, atol=1e-12 * scale)
        assert abs(csa - sa) <= 1e-12 * scale
        assert np.allclose(cqb, qb, rtol=0, atol=1e-12 * scale)  # the neighbor's position share
        assert abs(csb - sb) <= 1e-12 * scale                    # the neighbor's width share


def test_pair_forces_cancel():
    """Newton's third law of the position shares (the reason the share can
    be the owner's vector negated)."""
    D = np.array([2.1, -1.3, 0.7])
    ua, ub = 0.4, 0.25
    qa, _, qb, _ = both_sides(D, ua, ub)
    assert np.allclose(qa + qb, 0.0, atol=1e-14 * np.abs(qa).max())
