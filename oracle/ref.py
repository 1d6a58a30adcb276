"""Front end of oracle/_ref/ref_tables: libMesh's own QGauss rules and
LAGRANGE / HIERARCHIC shape functions, compiled from the reference sources
by oracle/ref_build.py.  Test infrastructure: it pins the oracle's tables to
the reference (tests/golden/make_ref_golden.py writes them to a committed
fixture)."""
import os
import subprocess
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import ref_build  # noqa: E402


def available():
    return ref_build.available()


class Batch:
    """Collects requests, runs the reference driver once, returns the results
    in request order."""

    def __init__(self):
        self.lines, self.reqs = [], []

    @staticmethod
    def _pts(P):
        return ["%.17g %.17g %.17g" % tuple(p) for p in np.asarray(P, float).reshape(-1, 3)]

    def qgauss(self, elem_type, order):
        self.lines.append("qgauss %d %d" % (elem_type, order))
        self.reqs.append(("q", None))

    def lagrange(self, elem_type, order, n, pts):
        pts = np.asarray(pts, float).reshape(-1, 3)
        self.lines += ["lagrange %d %d %d %d" % (elem_type, order, n, len(pts))] + self._pts(pts)
        self.reqs.append(("s", (n, len(pts))))

    def hierarchic(self, elem_type, order, n, X, pts):
        X = np.asarray(X, float).reshape(-1, 3)
        pts = np.asarray(pts, float).reshape(-1, 3)
        self.lines += (["hierarchic %d %d %d %d" % (elem_type, order, n, len(X))] + self._pts(X) +
                       ["%d" % len(pts)] + self._pts(pts))
        self.reqs.append(("s", (n, len(pts))))

    def run(self):
        exe = ref_build.build()
        r = subprocess.run([exe], input="\n".join(self.lines) + "\n", capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("ref_tables failed:\n" + r.stdout[-2000:] + r.stderr[-2000:])
        tok = r.stdout.split()
        pos, out = 0, []
        for kind, shape in self.reqs:
            if kind == "q":
                n = int(tok[pos])
                v = np.array(tok[pos + 1:pos + 1 + 4 * n], float).reshape(n, 4)
                pos += 1 + 4 * n
                out.append((v[:, :3].copy(), v[:, 3].copy()))
            else:
                n, np_ = shape
                v = np.array(tok[pos:pos + 4 * n * np_], float)
                pos += 4 * n * np_
                out.append((v[:n * np_].reshape(n, np_), v[n * np_:].reshape(3, n, np_)))
        return out
