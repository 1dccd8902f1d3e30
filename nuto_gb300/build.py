"""Builds the in-tree CUDA library nuto_gb300/lib/libnuto_gb300.so for sm_103a (GB300).

Each translation unit under csrc/ is compiled by its own nvcc process (in parallel), then linked into one
shared library exposing the C ABI of include/nuto_gpu.h. No CMake; nvcc cross-compiles without a GPU.
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "lib")
VARIANTS = {
    # the product library
    "release": ("libnuto_gb300.so", []),
    # every kernel index range-checked and clamped, every launch synchronised and checked (debugging only)
    "checked": ("libnuto_gb300_checked.so", ["-DNUTO_GPU_CHECKED"]),
}
LIB_PATH = os.path.join(LIB_DIR, VARIANTS["release"][0])


ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cu", "assemble.cu", "fused.cu", "tc20.cu", "adjoint.cu", "krylov.cu", "newton.cu", "amg.cu"]


def lib_path(variant="release"):
    return os.path.join(LIB_DIR, VARIANTS[variant][0])


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _flags(extra=()):
    return ["-O3", "-std=c++17", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-fopenmp,-O3",
            "--expt-relaxed-constexpr", *extra]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, ptxas_info=False, variant="release"):
    out_name, defines = VARIANTS[variant]
    obj_dir = os.path.join(LIB_DIR, "obj_" + variant)
    out_path = os.path.join(LIB_DIR, out_name)
    os.makedirs(obj_dir, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "nuto_gpu.h"))
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(obj_dir, src.replace(".cu", ".o"))
        if force or _stale(o, [s] + headers):
            extra = (["-Xptxas", "-v"] if ptxas_info else []) + defines
            jobs.append((s, o, [nvcc(), *_flags(extra), "-c", s, "-o", o]))

    def run(job):
        s, o, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (s, r.stdout, r.stderr))
        return s, r.stderr

    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for s, err in ex.map(run, jobs):
                if verbose or ptxas_info:
                    sys.stderr.write("== %s\n%s" % (os.path.basename(s), err))
    objs = [os.path.join(obj_dir, src.replace(".cu", ".o")) for src in SOURCES]
    if jobs or _stale(out_path, objs):
        tmp = out_path + ".tmp.%d" % os.getpid()
        cmd = [nvcc(), "-shared", *ARCH, "-o", tmp, *objs, "-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, out_path)
    return out_path


if __name__ == "__main__":
    v = "checked" if "--checked" in sys.argv else "release"
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv, variant=v))
