"""Writes tests/golden/ref_tables.npz: libMesh's own QGauss rules and shape
functions (LAGRANGE, HIERARCHIC FIRST to THIRD, with element orientations)
evaluated by the reference sources compiled in oracle/_ref.  Run where the
reference tree is present:  python tests/golden/make_ref_golden.py"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import ref  # noqa: E402

HEX8, HEX27, TET4, TET10, TET14, PRISM6, PRISM18, PRISM20, PRISM21 = 10, 12, 8, 9, 34, 13, 15, 35, 36
# QGauss rules by element class (orders the configurations and tests use, and their neighbours)
QRULES = [(HEX8, o) for o in range(1, 10)] + [(TET4, o) for o in range(1, 7)] + [(PRISM6, o) for o in range(1, 8)]
# LAGRANGE (type, order, shapes) and HIERARCHIC (type, order, shapes, node count)
LAGRANGE = [(HEX8, 1, 8), (HEX27, 2, 27), (TET4, 1, 4), (TET10, 2, 10), (TET14, 3, 14), (PRISM6, 1, 6)]
HIER = [(HEX8, 1, 8, 8), (HEX27, 2, 27, 27), (HEX27, 3, 64, 27), (TET4, 1, 4, 4), (TET10, 2, 10, 10),
        (TET14, 3, 20, 14), (PRISM6, 1, 6, 6), (PRISM18, 2, 18, 18), (PRISM20, 3, 40, 20), (PRISM21, 3, 40, 21)]
Q_FOR = {HEX8: 3, HEX27: 7, TET4: 4, TET10: 4, TET14: 6, PRISM6: 3, PRISM18: 5, PRISM20: 5, PRISM21: 5}


def master(elem_type):
    """Master-element node points in libMesh's local node order."""
    hexv = [(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)]
    tetv = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)]
    priv = [(0, 0, -1), (1, 0, -1), (0, 1, -1), (0, 0, 1), (1, 0, 1), (0, 1, 1)]
    mid = lambda P, pairs: [tuple(np.mean([P[i] for i in g], 0)) for g in pairs]  # noqa: E731
    if elem_type == HEX8:
        return np.array(hexv, float)
    if elem_type == HEX27:
        e = [(0, 1), (1, 2), (2, 3), (3, 0), (0, 4), (1, 5), (2, 6), (3, 7), (4, 5), (5, 6), (6, 7), (7, 4)]
        f = [(0, 1, 2, 3), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7), (4, 5, 6, 7)]
        return np.array(hexv + mid(hexv, e) + mid(hexv, f) + [(0, 0, 0)], float)
    if elem_type in (TET4, TET10, TET14):
        e = [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]
        f = [(0, 1, 2), (0, 1, 3), (1, 2, 3), (0, 2, 3)]
        pts = tetv + (mid(tetv, e) if elem_type != TET4 else []) + (mid(tetv, f) if elem_type == TET14 else [])
        return np.array(pts, float)
    e = [(0, 1), (1, 2), (0, 2), (0, 3), (1, 4), (2, 5), (3, 4), (4, 5), (3, 5)]
    fq = [(0, 1, 4, 3), (1, 2, 5, 4), (0, 2, 5, 3)]
    ft = [(0, 1, 2), (3, 4, 5)]
    P = priv
    if elem_type == PRISM6:
        return np.array(P, float)
    pts = P + mid(P, e) + mid(P, fq)
    if elem_type == PRISM20:
        pts += mid(P, ft)
    if elem_type == PRISM21:
        pts += mid(P, ft) + [(1 / 3, 1 / 3, 0)]
    return np.array(pts, float)


def orientations(elem_type, X):
    """The master element and variants whose local frames differ: affine
    images under a rotation that reorders the points' lexicographic order
    (the edge and face orientation of HIERARCHIC shapes follows from it)."""
    rots = [np.eye(3), np.array([[0, 1, 0], [0, 0, 1], [1, 0, 0]], float),
            np.array([[-1, 0, 0], [0, 1, 0], [0, 0, -1]], float), np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]], float)]
    shift = np.array([0.3, -0.2, 0.1])
    return [X @ R.T + shift for R in rots]


def main():
    rng = np.random.default_rng(11)
    b = ref.Batch()
    keys = []
    for t, o in QRULES:
        b.qgauss(t, o)
        keys.append(("qgauss_%d_%d" % (t, o), None))
    # evaluation points: the rule the configurations use on the element, plus random interior points
    rule_pts = {}
    qb = ref.Batch()
    for t in sorted(set(k[0] for k in LAGRANGE + HIER)):
        cls = HEX8 if t in (HEX8, HEX27) else (TET4 if t in (TET4, TET10, TET14) else PRISM6)
        qb.qgauss(cls, Q_FOR[t])
    qres = qb.run()
    for t, (p, _) in zip(sorted(set(k[0] for k in LAGRANGE + HIER)), qres):
        if t in (HEX8, HEX27):
            extra = rng.uniform(-1, 1, (3, 3))
        elif t in (TET4, TET10, TET14):
            extra = rng.dirichlet(np.ones(4), 3)[:, :3]
        else:
            extra = np.column_stack([rng.dirichlet(np.ones(3), 3)[:, :2], rng.uniform(-1, 1, 3)])
        rule_pts[t] = np.vstack([p, extra])
    for t, o, n in LAGRANGE:
        b.lagrange(t, o, n, rule_pts[t])
        keys.append(("lagrange_%d_%d" % (t, o), rule_pts[t]))
    for t, o, n, nn in HIER:
        for v, X in enumerate(orientations(t, master(t))):
            b.hierarchic(t, o, n, X, rule_pts[t])
            keys.append(("hier_%d_%d_v%d" % (t, o, v), (X, rule_pts[t])))
    res = b.run()
    arrays = {}
    for (k, extra), r in zip(keys, res):
        if k.startswith("qgauss"):
            arrays[k + "_pts"], arrays[k + "_w"] = r
        elif k.startswith("lagrange"):
            arrays[k + "_at"], arrays[k + "_phi"], arrays[k + "_dphi"] = extra, r[0], r[1]
        else:
            arrays[k + "_X"], arrays[k + "_at"] = extra
            arrays[k + "_phi"], arrays[k + "_dphi"] = r
    out = os.path.join(HERE, "ref_tables.npz")
    np.savez_compressed(out, **arrays)
    print(out, len(arrays), "arrays")


if __name__ == "__main__":
    main()
