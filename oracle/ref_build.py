"""Build recipe for oracle/_ref/ref_tables (test infrastructure): libMesh's own
quadrature, LAGRANGE / HIERARCHIC shape-function and element sources,
compiled where they lie in the reference tree, linked with the driver and
shim of oracle/ref/.

The whole reference library cannot be built here (its parallel-library
submodule is absent, so configure and every file that includes it fail);
these leaf numerical files compile on their own against a hand-written
configuration header (oracle/ref/libmesh_config.h).  Symbols that only the
uncompiled files define are generated as stubs that abort with their name
if called: the driver's paths never reach them, and a stub that is reached
ends the run instead of returning a value.  Unresolved data symbols other
than type information of classes the driver never instantiates stop the
build, so no table is silently zero.

Compiled like the reference's optimised build: -O2 -DNDEBUG, and
-ffp-contract=off so that no multiply-add is fused (as in its x86-64 build).
Outputs go to oracle/_ref/ only.  Needs the reference tree (present where
the repository is developed; absent on machines that only run the tests,
which then use the committed golden tables under tests/golden/)."""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("LIBMESH_REFERENCE_DIR", "/root/reference")
OUT = os.path.join(HERE, "_ref")
EXE = os.path.join(OUT, "ref_tables")

SOURCES = (
    sorted(glob.glob(os.path.join(REF, "src", "quadrature", "*.C"))) +
    [os.path.join(REF, "src", p + ".C") for p in (
        "base/reference_counter", "base/libmesh_common", "base/dof_object",
        "fe/fe", "fe/fe_lagrange_shape_1D", "fe/fe_lagrange_shape_2D", "fe/fe_lagrange_shape_3D",
        "fe/fe_hierarchic_shape_1D", "fe/fe_hierarchic_shape_2D", "fe/fe_hierarchic_shape_3D",
        "geom/node", "geom/node_elem", "geom/edge", "geom/edge_edge2", "geom/edge_edge3",
        "geom/face", "geom/face_tri", "geom/face_tri3", "geom/face_tri6", "geom/face_tri7",
        "geom/face_quad", "geom/face_quad4", "geom/face_quad9", "geom/cell",
        "geom/cell_hex", "geom/cell_hex8", "geom/cell_hex27",
        "geom/cell_tet", "geom/cell_tet4", "geom/cell_tet10", "geom/cell_tet14",
        "geom/cell_prism", "geom/cell_prism6", "geom/cell_prism18", "geom/cell_prism20", "geom/cell_prism21",
        "numerics/type_vector", "utils/number_lookups")])
OWN = [os.path.join(HERE, "ref", "ref_shim.C"), os.path.join(HERE, "ref", "ref_tables.C")]
FLAGS = ["-std=c++17", "-O2", "-DNDEBUG", "-ffp-contract=off", "-fno-fast-math"]


def available():
    return os.path.isdir(os.path.join(REF, "src", "quadrature"))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout


def _include_dir():
    """oracle/_ref/include/libmesh/: a link to every reference header (they are
    included as "libmesh/<name>.h") and the configuration header."""
    inc = os.path.join(OUT, "include", "libmesh")
    os.makedirs(inc, exist_ok=True)
    for h in glob.glob(os.path.join(REF, "include", "**", "*.h"), recursive=True):
        dst = os.path.join(inc, os.path.basename(h))
        if not os.path.lexists(dst):
            os.symlink(h, dst)
    cfg = os.path.join(inc, "libmesh_config.h")
    if os.path.lexists(cfg):
        os.remove(cfg)
    os.symlink(os.path.join(HERE, "ref", "libmesh_config.h"), cfg)
    return os.path.dirname(inc)


def _stubs(objs):
    undef, defined = set(), set()
    for line in _run(["nm", "--undefined-only"] + objs).splitlines():
        p = line.split()
        if p and p[0] == "U":
            undef.add(p[-1])
    for line in _run(["nm", "--defined-only"] + objs).splitlines():
        p = line.split()
        if len(p) == 3:
            defined.add(p[2])
    need = sorted(s for s in undef - defined if "7libMesh" in s)
    names = _run(["c++filt"] + need).splitlines() if need else []
    out = ["#include <stdio.h>", "#include <stdlib.h>"]
    for s, dem in zip(need, names):
        if "(" not in dem:  # data
            if not s.startswith(("_ZTI", "_ZTS", "_ZTV")):
                raise RuntimeError("reference build: unresolved data symbol " + dem)
            out.append("char %s[64];" % s)
        elif "Singleton::Setup::Setup" in dem:  # static registration, nothing to register
            out.append("void %s(void) { }" % s)
        else:
            msg = dem.replace("\\", "\\\\").replace('"', '\\"').replace("%", "%%")
            out.append('void %s(void) { fprintf(stderr, "reference stub reached: %s\\n"); abort(); }' % (s, msg))
    path = os.path.join(OUT, "stubs.c")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    return path


def build(force=False):
    if not available():
        raise RuntimeError("the reference source tree is not present")
    deps = SOURCES + OWN + [os.path.join(HERE, "ref", "libmesh_config.h")]
    if not force and os.path.exists(EXE) and os.path.getmtime(EXE) >= max(os.path.getmtime(d) for d in deps):
        return EXE
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    inc = _include_dir()
    jobs, objs = [], []
    for src in SOURCES + OWN:
        rel = os.path.relpath(src, REF) if src.startswith(REF) else os.path.basename(src)
        obj = os.path.join(OUT, "obj", rel.replace(os.sep, "_") + ".o")
        objs.append(obj)
        jobs.append(["g++"] + FLAGS + ["-I" + inc, "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(2, min(16, os.cpu_count() or 2))) as ex:
        list(ex.map(_run, jobs))
    stub_c = _stubs(objs)
    stub_o = os.path.join(OUT, "obj", "stubs.o")
    _run(["gcc", "-c", stub_c, "-o", stub_o])
    tmp = EXE + ".tmp"
    _run(["g++", "-no-pie"] + objs + [stub_o, "-o", tmp])
    os.replace(tmp, EXE)
    return EXE


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
