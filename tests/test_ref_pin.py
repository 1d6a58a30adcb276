"""The oracle's reference-element tables against libMesh's own code, bit for
bit: QGauss points and weights, LAGRANGE shapes and derivatives, HIERARCHIC
shapes and their central-difference derivatives (FIRST to THIRD, elements in
several orientations).  The reference values come from the reference sources
compiled in oracle/_ref (oracle/ref_build.py) and are committed as
tests/golden/ref_tables.npz (tests/golden/make_ref_golden.py); where the
reference tree is present the fixture is also regenerated and compared."""
import os
import sys
import tempfile

import numpy as np
import pytest

import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_ref_golden as mk  # noqa: E402

G = np.load(os.path.join(HERE, "golden", "ref_tables.npz"))


# prism rules above FIFTH are held for HIERARCHIC prisms of order 3
ORACLE_Q = [(t, o) for t, o in mk.QRULES if not (t == mk.PRISM6 and o > 5)]


@pytest.mark.parametrize("t,o", ORACLE_Q)
def test_qgauss_is_the_reference_rule(t, o):
    p, w = orc.qgauss(t, o)
    assert np.array_equal(p, G["qgauss_%d_%d_pts" % (t, o)])
    assert np.array_equal(w, G["qgauss_%d_%d_w" % (t, o)])


@pytest.mark.parametrize("t,o,n", mk.LAGRANGE)
def test_lagrange_shapes_are_the_reference_shapes(t, o, n):
    at = G["lagrange_%d_%d_at" % (t, o)]
    phi, dphi = orc.shapes(t, o, at)
    assert phi.shape[0] == n
    assert np.array_equal(phi, G["lagrange_%d_%d_phi" % (t, o)])
    assert np.array_equal(dphi, G["lagrange_%d_%d_dphi" % (t, o)])


ORACLE_HIER = list(mk.HIER)


@pytest.mark.parametrize("t,o,n,nn", ORACLE_HIER)
def test_hierarchic_shapes_are_the_reference_shapes(t, o, n, nn):
    for v in range(4):
        key = "hier_%d_%d_v%d" % (t, o, v)
        X, at = G[key + "_X"], G[key + "_at"]
        if o >= 2 and t == mk.HEX27:  # the face swaps change the rounding from SECOND on
            phi, dphi = orc.shapes_hier_hex(X, o, at)
        elif o == 3 and t == mk.TET14:
            phi, dphi = orc.shapes_tet3(X, at)
        elif o >= 2 and t in (mk.PRISM18, mk.PRISM20, mk.PRISM21):
            phi, dphi = orc.shapes_hier_prism(X, o, at)
        else:  # the other elements' shapes up to SECOND do not depend on the orientation
            phi, dphi = orc.shapes(t, o | 0x100, at)
        assert phi.shape[0] == n
        assert np.array_equal(phi, G[key + "_phi"]), key
        assert np.array_equal(dphi, G[key + "_dphi"]), key


@pytest.mark.skipif(not mk.ref.available(), reason="the reference source tree is not present")
def test_golden_tables_are_current():
    """Regenerates the fixture from the compiled reference and compares."""
    with tempfile.TemporaryDirectory() as d:
        old = mk.HERE
        mk.HERE = d
        try:
            mk.main()
        finally:
            mk.HERE = old
        fresh = np.load(os.path.join(d, "ref_tables.npz"))
        assert sorted(fresh.files) == sorted(G.files)
        for k in G.files:
            assert np.array_equal(fresh[k], G[k]), k
