"""Build recipe for the oracle libraries (test infrastructure only).

* ``oracle/liboracle.so``  -- the C restatement in oracle.c (gcc).
* ``oracle/_ref/libscsref.so`` -- the reference's own CPU code (loader, core
  decomposition, BFS, heuristics) compiled from its sources in place through
  ``oracle/ref_driver.cu``.
* ``oracle/_ref/scs_ref_server`` -- the reference's own GPU server, its
  ``main.cu`` compiled unchanged for sm_103a (``nvcc -std=c++17``; the file
  includes the rest of its sources).  It is run only by
  ``tests/golden/make_ref_gpu.py`` to record the reference's answers.

Each is built only where the reference tree exists (``SCS_REF_DIR``); the
output directory is git-ignored and nothing is copied out of the reference.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# where this recipe looks for the reference tree unless SCS_REF_DIR says
# otherwise (the tree is absent on the GPU machine: every step skips then)
DEFAULT_REF = "/root/reference"


def ref_dir():
    """The reference tree to build from, or None when it is not present."""
    d = os.path.abspath(os.environ.get("SCS_REF_DIR", DEFAULT_REF))
    return d if os.path.isdir(d) else None


def build_oracle(verbose=False):
    out = os.path.join(HERE, "liboracle.so")
    src = os.path.join(HERE, "oracle.c")
    if os.path.exists(out) and os.path.getmtime(out) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "oracle.h"))):
        return out
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-Wall", "-o", out, src]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return out


def build_ref(src=None, verbose=False):
    """Compile the reference's CPU code; returns the .so path or None."""
    src = src or ref_dir()
    if not src:
        return None
    heur = os.path.join(src, "inc", "heuristic.h")
    if not os.path.exists(heur):
        return None
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libscsref.so")
    drv = os.path.join(HERE, "ref_driver.cu")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(drv):
        return out
    cmd = [nvcc, "-std=c++17", "-O2", "-Xcompiler", "-fPIC", "-shared",
           '-DSCS_REF_HEURISTIC_H="%s"' % heur, "-o", out, drv]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return out


def build_ref_server(src=None, verbose=False):
    """Compile the reference's main.cu unchanged into oracle/_ref; returns
    the executable's path or None when the tree or nvcc is absent."""
    src = os.path.abspath(src) if src else ref_dir()
    if not src or not os.path.exists(os.path.join(src, "main.cu")):
        return None
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "scs_ref_server")
    main = os.path.join(src, "main.cu")
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(main):
        return out
    cmd = [nvcc, "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a",
           "-o", out, main, "-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd, cwd=src)
    return out


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_ref(sys.argv[1] if len(sys.argv) > 1 else None, verbose=True))
    if "--server" in sys.argv:
        print(build_ref_server(verbose=True))
