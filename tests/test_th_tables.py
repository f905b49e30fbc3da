"""The Taylor-Hood reference tables that the FP64 element kernel contracts
with compile-time zero skipping (femx_gb300/csrc/th.cu, kRefX / tabNz): an
entry is left out when its magnitude is below 1e-14. That is only the same
element if every such entry is an exact zero of the integral (a rounding
residue of the quadrature sum) and every kept entry is far above the
threshold. The tables are rebuilt here from the same published 6-point
degree-4 rule (Dunavant) and P2 basis as the kernel's constexpr makeRef()."""
import numpy as np

A1, W1 = 0.445948490915964886, 0.223381589678011466 * 0.5
A2, W2 = 0.091576213509770743, 0.109951743655321868 * 0.5
POINTS = [(A1, A1, W1), (1 - 2 * A1, A1, W1), (A1, 1 - 2 * A1, W1),
          (A2, A2, W2), (1 - 2 * A2, A2, W2), (A2, 1 - 2 * A2, W2)]
THRESHOLD = 1e-14


def p2(r, s):
    l0, l1, l2 = 1 - r - s, r, s
    g0, g1, g2 = (-1.0, -1.0), (1.0, 0.0), (0.0, 1.0)
    n = [l0 * (2 * l0 - 1), l1 * (2 * l1 - 1), l2 * (2 * l2 - 1), 4 * l0 * l1, 4 * l1 * l2,
         4 * l2 * l0]
    dn = [[(4 * l0 - 1) * g0[d] for d in range(2)], [(4 * l1 - 1) * g1[d] for d in range(2)],
          [(4 * l2 - 1) * g2[d] for d in range(2)],
          [4 * (l1 * g0[d] + l0 * g1[d]) for d in range(2)],
          [4 * (l2 * g1[d] + l1 * g2[d]) for d in range(2)],
          [4 * (l0 * g2[d] + l2 * g0[d]) for d in range(2)]]
    return np.array(n), np.array(dn)


def tables():
    w = np.array([p[2] for p in POINTS])
    lam = np.array([(1 - p[0] - p[1], p[0], p[1]) for p in POINTS])
    dnr = np.array([p2(p[0], p[1])[1] for p in POINTS])            # [q][a][k]
    s00 = np.einsum("q,qa,qb->ab", w, dnr[:, :, 0], dnr[:, :, 0])
    s11 = np.einsum("q,qa,qb->ab", w, dnr[:, :, 1], dnr[:, :, 1])
    s01 = (np.einsum("q,qa,qb->ab", w, dnr[:, :, 0], dnr[:, :, 1])
           + np.einsum("q,qa,qb->ab", w, dnr[:, :, 1], dnr[:, :, 0]))
    c = np.einsum("q,qb,qak->kab", w, lam, dnr)                     # [k][a][b]
    dnv = np.array([p2(*v)[1] for v in [(0.0, 0.0), (1.0, 0.0), (0.0, 1.0)]])
    return {"dNv": dnv, "dNr": dnr, "S00": s00, "S11": s11, "S01": s01, "C": c}


# exact values with rational arithmetic where the integrand is polynomial of
# degree <= 4 (the rule integrates it exactly): S^kl (degree 2) and C (degree 2)
def exact_rational_zeros():
    from fractions import Fraction as F

    # integral over the reference triangle of r^i s^j = i! j! / (i + j + 2)!
    def mono(i, j):
        from math import factorial
        return F(factorial(i) * factorial(j), factorial(i + j + 2))

    # P2 gradients and P1 functions as polynomials {(i, j): coeff}
    def mul(p, q):
        out = {}
        for (a, b), x in p.items():
            for (c, d), y in q.items():
                out[(a + c, b + d)] = out.get((a + c, b + d), 0) + x * y
        return out

    def integ(p):
        return sum((x * mono(i, j) for (i, j), x in p.items()), F(0))

    l0 = {(0, 0): F(1), (1, 0): F(-1), (0, 1): F(-1)}
    l1 = {(1, 0): F(1)}
    l2 = {(0, 1): F(1)}
    lams = [l0, l1, l2]
    gl = [(-1, -1), (1, 0), (0, 1)]

    def scale(p, k):
        return {key: v * k for key, v in p.items()}

    def add(*ps):
        out = {}
        for p in ps:
            for key, v in p.items():
                out[key] = out.get(key, 0) + v
        return out

    # dN_a / dx_d for the six P2 functions
    grads = []
    for i in range(3):
        grads.append([add(scale(lams[i], 4 * gl[i][d]), {(0, 0): F(-gl[i][d])})
                      for d in range(2)])
    for i, j in [(0, 1), (1, 2), (2, 0)]:
        grads.append([add(scale(lams[j], 4 * gl[i][d]), scale(lams[i], 4 * gl[j][d]))
                      for d in range(2)])
    zeros = {}
    for name, (k, l) in {"S00": (0, 0), "S11": (1, 1)}.items():
        zeros[name] = np.array([[integ(mul(grads[a][k], grads[b][l])) == 0 for b in range(6)]
                                for a in range(6)])
    zeros["S01"] = np.array([[integ(add(mul(grads[a][0], grads[b][1]),
                                        mul(grads[a][1], grads[b][0]))) == 0
                              for b in range(6)] for a in range(6)])
    zeros["C"] = np.array([[[integ(mul(lams[b], grads[a][k])) == 0 for b in range(3)]
                            for a in range(6)] for k in range(2)])
    return zeros


def test_skipped_entries_are_exact_zeros_and_kept_entries_are_large():
    t = tables()
    for name, v in t.items():
        a = np.abs(v)
        small = a < THRESHOLD
        assert np.all(a[small] < 1e-15), name          # residues of exact zeros
        assert np.all(a[~small] > 1e-3), name          # kept entries: far above
        assert small.sum() > 0 or name == "dNr", name


def test_skipped_entries_match_the_exact_integrals():
    """S^kl and C are integrals of polynomials of degree 2, exact under the
    degree-4 rule: the entries skipped as zero are exactly the zero
    integrals (rational arithmetic)."""
    t = tables()
    z = exact_rational_zeros()
    for name in ("S00", "S11", "S01"):
        assert np.array_equal(np.abs(t[name]) < THRESHOLD, z[name]), name
    assert np.array_equal(np.abs(t["C"]) < THRESHOLD, z["C"])


def test_vertex_gradients_are_small_integers():
    t = tables()
    assert np.array_equal(t["dNv"], np.round(t["dNv"]))
    assert (np.abs(t["dNv"]) < THRESHOLD).sum() == 16
