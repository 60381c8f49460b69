"""Build the CUDA library in-tree: ``rascil_gb300/lib/librascil_gb300.so``.

Every translation unit is compiled by nvcc for sm_103a only, in parallel,
then linked against cuFFT and the CUDA runtime.  Host code is compiled
with FMA contraction off so the FP64 bucket coordinates are the same on
x86-64 and aarch64 hosts.

    python -m rascil_gb300.build            # build if sources changed
    python -m rascil_gb300.build --force    # always rebuild
"""

import argparse
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
BUILDDIR = os.path.join(HERE, "lib", "obj")
LIBNAME = "librascil_gb300.so"
SOURCES = ["gb_plan.cu", "gb_invert.cu", "gb_predict.cu", "gb_capi.cu", "gb_dft.cu", "gb_profile.cu",
           "gb_noalloc.cu", "gb_gains.cu", "gb_fft.cu", "gb_weight.cu",
           "gb_rotate.cu", "gb_batch.cu"]
HEADERS = ["gb_internal.cuh", "gb_plan.cuh", "gb_profile.cuh", "gb_fft.cuh", "gb_async.cuh", "es_table.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-Xptxas", "-O3"]


def nvcc():
    cand = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cand, "bin", "nvcc")
    if os.path.exists(path):
        return path
    found = shutil.which("nvcc")
    if not found:
        raise RuntimeError("nvcc not found (set CUDA_HOME)")
    return found


def lib_path():
    return os.path.join(LIBDIR, LIBNAME)


def _inputs():
    paths = [os.path.join(CSRC, s) for s in SOURCES + HEADERS]
    paths.append(os.path.join(HERE, "..", "include", "rascil_gb300.h"))
    paths.append(os.path.abspath(__file__))
    return paths


def up_to_date():
    out = lib_path()
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(p) <= t for p in _inputs())


def _compile(src, extra):
    obj = os.path.join(BUILDDIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), res.stderr))
    return obj, res.stderr


def build(force=False, verbose=False, ptxas_info=False):
    """Compile and link; returns the library path."""
    if not force and up_to_date():
        return lib_path()
    os.makedirs(BUILDDIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    objs = [r[0] for r in results]
    if verbose or ptxas_info:
        for _, err in results:
            if err:
                sys.stderr.write(err)
    tmp = lib_path() + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcufft", "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), res.stderr))
    os.replace(tmp, lib_path())
    return lib_path()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true")
    args = ap.parse_args()
    print(build(force=args.force, verbose=True, ptxas_info=args.ptxas_info))


if __name__ == "__main__":
    main()
