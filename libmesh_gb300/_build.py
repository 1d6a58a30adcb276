"""Build recipe for the native library: host C++ with g++, kernels with nvcc
for sm_103a, linked into libmesh_gb300/_lib/liblmg.so.  Translation units
compile in parallel; objects live in libmesh_gb300/_lib/obj."""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "liblmg.so")

CXX_SOURCES = ["host_mesh.cpp", "host_mesh_tri.cpp", "host_dofmap.cpp", "host_amr.cpp", "fe_tables.cpp",
               "hier3_tables.cpp"]
CU_SOURCES = ["elements.cu", "gather.cu", "context.cu", "context_general.cu", "general.cu", "batch.cu", "cg.cu",
              "vjp.cu", "probe.cu", "hier3.cu", "tc.cu", "amr_rows.cu", "dofs_device.cu", "batch_persistent.cu",
              "plan_device.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmesh_gb300")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose=False, force=False):
    """Compile every translation unit and link liblmg.so; returns its path."""
    nvcc = _nvcc()
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    srcs = [os.path.join(SRC, s) for s in CXX_SOURCES + CU_SOURCES]
    deps = srcs + [os.path.join(SRC, h) for h in os.listdir(SRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "libmesh_gb300.h"))
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps)):
        return LIB
    jobs = []
    objs = []
    for s in CXX_SOURCES:
        o = os.path.join(OUT, "obj", s + ".o")
        objs.append(o)
        # -ffp-contract=off: host tables (central-difference derivatives, refined
        # coordinates, constraint rows) round identically on x86-64 and aarch64,
        # where g++ would otherwise fuse multiply-adds
        jobs.append(["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fPIC", "-pthread", "-Wall", "-c",
                     os.path.join(SRC, s), "-o", o])
    for s in CU_SOURCES:
        o = os.path.join(OUT, "obj", s + ".o")
        objs.append(o)
        jobs.append([nvcc, "-std=c++17", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "--expt-relaxed-constexpr", "-c", os.path.join(SRC, s), "-o", o])
    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    cuda_lib = os.path.join(_cuda_home(nvcc), "lib64")
    tmp = LIB + ".tmp"
    _run([nvcc, "-shared", *ARCH, "-o", tmp, *objs, "-L" + cuda_lib, "-lcudart", "-Xcompiler",
          "-pthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force=True))
