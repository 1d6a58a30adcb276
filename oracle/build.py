"""Build recipe for the CPU oracle (test infrastructure): oracle/oracle.cpp,
oracle/oracle_constraints.cpp and oracle/oracle_mesh.cpp ->
oracle/_build/liboracle.so, compiled with -ffp-contract=off so that no
multiply-add is fused."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")


def build(force=False):
    srcs = [os.path.join(HERE, f) for f in ("oracle.cpp", "oracle_constraints.cpp", "oracle_mesh.cpp")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in srcs):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread"] + srcs + ["-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
