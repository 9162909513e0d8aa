"""Build of the in-tree native libraries.

``build()`` compiles ``csrc/*.cu`` into ``sudodem_gb300/libsqdem_gpu.so`` for sm_103a with
nvcc, the translation units in parallel.  Both are built with ``--fmad=false`` so that
products and sums keep the rounding sequence of the reference's x86-64 build (no fused
multiply-add), and so that the adjoint's dual-number replay takes the branches of its
forward run.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libsqdem_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsqdem_gpu.so")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".cu", ".cuh", ".h"))] + [
        os.path.join(HERE, "..", "include", "sqdem.h")
    ]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force=False, verbose=False):
    """Compile libsqdem_gpu.so in place; return its path."""
    if not force and up_to_date():
        return LIB
    nvcc = nvcc_path()
    objs = []
    tmp = os.path.join(HERE, "_obj")
    os.makedirs(tmp, exist_ok=True)
    units = [("sqdem_engine.cu", ["--fmad=false"]), ("sqdem_adjoint.cu", ["--fmad=false"]),
             ("sqdem_peaks.cu", ["--fmad=false"])]
    procs = []
    for src, extra in units:
        obj = os.path.join(tmp, src.replace(".cu", ".o"))
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
               "-Xcompiler", "-Wno-deprecated-declarations", "-diag-suppress", "1444",
               *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), cmd))
        objs.append(obj)
    for p, cmd in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + out.decode(errors="replace"))
        if verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    cmd = [nvcc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart"]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
