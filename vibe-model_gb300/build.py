"""Build the GB300 library in-tree: vibe-model_gb300/libvibe_gb300.so.

nvcc compiles each CUDA translation unit for sm_103a in parallel, then links
one shared library. Host code is compiled without floating-point contraction
so the set-up arithmetic (grid metrics, reference state, initial state) gives
the same bits as the reference on x86 and Arm.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvibe_gb300.so")
# (source, object, extra flags)
SOURCES = [("step_fp64.cu", "step_fp64.o", []),
           ("step_fp64.cu", "step_fp64_exact.o", ["-DVGB_FP64_EXACT", "--fmad=false"]),
           ("step_mixed.cu", "step_mixed.o", []),
           ("model.cu", "model.o", []),
           ("ckern.cu", "ckern.o", []),
           ("helmholtz_ref.cu", "helmholtz_ref.o", ["--fmad=false"]),
           ("helmholtz_mg.cu", "helmholtz_mg.o", []),
           ("helmholtz_api.cu", "helmholtz_api.o", []),
           ("si_step.cu", "si_step.o", ["--fmad=false"]),
           ("nest.cu", "nest.o", ["--fmad=false"]),
           ("tlad.cu", "tlad.o", []),
           ("step_tlad.cu", "step_tlad.o", []),
           ("advect_tlad.cu", "advect_tlad.o", []),
           ("physics.cu", "physics.o", ["--fmad=false"]),
           ("diag.cu", "diag.o", ["--fmad=false"])]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libvibe_gb300.so")
    return exe


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    objs, jobs = [], []
    for src, obj, extra in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, obj)
        objs.append(o)
        if force or _stale(o, [s] + headers + [os.path.abspath(__file__)]):
            jobs.append([nvcc()] + _flags() + extra + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
