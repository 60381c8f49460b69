"""Recipe: build the reference's own CUDA component-DFT kernel so the GPU
DFT here can be timed against it on the same GPU.

The reference ships that kernel as a source string, ``cuda_kernel_source``
in ``rascil/processing_components/imaging/dft.py:181-258``, compiled at run
time through CuPy (``dft.py:284-332``).  CuPy is not installed, so:

* ``extract(ref_root)`` (runs where the reference tree is present; its root
  is an argument, or RASCIL_REFERENCE_ROOT for the command line) copies
  the string into ``oracle/_ref/dft_kernel_ref.cu`` -- an untracked build
  output, never committed;
* ``build()`` (runs anywhere nvcc is) compiles that file together with
  ``launch_ref_dft.cu`` (this directory; the launcher and the small
  ``complex<T>`` stand-in for CuPy's header are this project's code) into
  ``oracle/_ref/libref_dft.so``.

The launch shape mirrors ``dft_gpu_raw_kernel`` (``dft.py:313-331``): blocks
of (128, 2, 2) over (baseline, channel, time).
"""
import ast
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "..", "_ref")
KERNEL = os.path.join(REF_DIR, "dft_kernel_ref.cu")
LIB = os.path.join(REF_DIR, "libref_dft.so")


def extract(ref_root):
    """Copy the kernel string out of the reference tree rooted at
    ``ref_root`` (None or a missing tree: nothing to do, returns None)."""
    if not ref_root:
        return None
    path = os.path.join(ref_root, "rascil", "processing_components", "imaging", "dft.py")
    if not os.path.exists(path):
        return None
    tree = ast.parse(open(path).read())
    for node in tree.body:
        if isinstance(node, ast.Assign) and any(
                isinstance(t, ast.Name) and t.id == "cuda_kernel_source" for t in node.targets):
            os.makedirs(REF_DIR, exist_ok=True)
            with open(KERNEL, "w") as f:
                f.write(node.value.value)
            return KERNEL
    return None


def build(force=False):
    if not os.path.exists(KERNEL):
        return None
    srcs = [os.path.join(HERE, "launch_ref_dft.cu"), KERNEL]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s)
                                                 for s in srcs):
        return LIB
    cmd = ["nvcc", "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
           "-Xcompiler", "-fPIC", "-shared", "-I", os.path.join(HERE, "include"),
           os.path.join(HERE, "launch_ref_dft.cu"), "-o", LIB + ".tmp"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference DFT build failed:\n" + res.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RASCIL_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_ref_dft.py REFERENCE_ROOT (or set RASCIL_REFERENCE_ROOT)")
    print(extract(root), build(force=True))
