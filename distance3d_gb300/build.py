"""Build libd3d_gb300.so (sm_103a) in-tree, under distance3d_gb300/_build/.

Each translation unit is compiled by nvcc in parallel, then linked into one
shared library with the static CUDA runtime.  Units whose results must be the
reference's bit for bit are compiled with -fmad=false (only the fma() calls
written in the source fuse); the mixed-precision unit contracts freely.

    python -m distance3d_gb300.build [--force] [--verbose]
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libd3d_gb300.so")
# FMA-throughput probe used by bench.py to measure the FP64/FP32 pipe peaks
PEAK_LIB = os.path.join(BUILD, "libd3d_peak.so")
PEAK_SRC = os.path.join(CSRC, "bench", "peak.cu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC,
          "-Xptxas", "-warn-spills"]

# (source, extra flags)
UNITS = [
    ("capi.cu", ["-fmad=false"]),
    ("store.cu", ["-fmad=false"]),
    ("gjk.cu", ["-fmad=false"]),
    ("epa.cu", ["-fmad=false"]),
    ("gjk_mixed.cu", ["-fmad=true"]),
    ("epa_mixed.cu", ["-fmad=true"]),
    ("epa_warp.cu", ["-fmad=true"]),
    ("schedule.cu", []),
    ("collide.cu", []),
    ("server.cu", []),
    ("tune.cu", []),
    ("robot.cu", ["-fmad=false"]),
    ("bvh.cu", []),
    ("mpr.cu", ["-fmad=false"]),
    ("mpr_mixed.cu", ["-fmad=true"]),
]


def nvcc():
    path = shutil.which("nvcc")
    if path is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        path = "/usr/local/cuda/bin/nvcc"
    if path is None:
        raise RuntimeError("nvcc not found: the CUDA toolkit is needed to build libd3d_gb300")
    return path


def _inputs_digest():
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE, os.path.join(CSRC, "bench")):
        for name in sorted(os.listdir(d)):
            if name.endswith((".cu", ".cuh", ".h")):
                with open(os.path.join(d, name), "rb") as f:
                    h.update(name.encode() + b"\0" + f.read())
    h.update(repr((ARCH, COMMON, UNITS)).encode())
    return h.hexdigest()


def build(force=False, verbose=False, ptxas_verbose=False):
    """Compile every unit and link the library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "inputs.sha256")
    digest = _inputs_digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return LIB
    cc = nvcc()
    jobs = []
    for src, flags in UNITS:
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *COMMON, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
        if ptxas_verbose:
            cmd += ["-Xptxas", "-v"]
        jobs.append((src, obj, cmd))

    def run(job):
        src, obj, cmd = job
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{p.stdout}\n{p.stderr}")
        return src, p.stderr

    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        for src, log in ex.map(run, jobs):
            if log.strip() and (verbose or ptxas_verbose):
                print(f"--- {src}\n{log}", file=sys.stderr)
    tmp = LIB + ".tmp"
    link = [cc, *ARCH, "-shared", "-cudart", "static", "-o", tmp] + [j[1] for j in jobs]
    if verbose:
        print(" ".join(link), file=sys.stderr)
    p = subprocess.run(link, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"link failed:\n{p.stdout}\n{p.stderr}")
    os.replace(tmp, LIB)
    p = subprocess.run([cc, *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-cudart", "static",
                        PEAK_SRC, "-o", PEAK_LIB + ".tmp"], capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"nvcc failed on {PEAK_SRC}:\n{p.stdout}\n{p.stderr}")
    os.replace(PEAK_LIB + ".tmp", PEAK_LIB)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv,
                ptxas_verbose="--ptxas" in sys.argv))
