"""Build recipe for the oracle libraries (test infrastructure only).

* ``oracle/liboracle.so``  -- the C restatement in oracle.c (gcc).
* ``oracle/_ref/libscsref.so`` -- the reference's own CPU code (loader, core
  decomposition, BFS, heuristics) compiled from its sources in place through
  ``oracle/ref_driver.cu``.  Built only where the reference tree exists; the
  output directory is git-ignored and nothing is copied out of the reference.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REF = "/root/reference"


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


def build_ref(ref_dir=None, verbose=False):
    """Compile the reference's CPU code; returns the .so path or None."""
    ref_dir = ref_dir or os.environ.get("SCS_REF_DIR", DEFAULT_REF)
    heur = os.path.join(ref_dir, "inc", "heuristic.h")
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


if __name__ == "__main__":
    print(build_oracle(verbose=True))
    print(build_ref(sys.argv[1] if len(sys.argv) > 1 else None, verbose=True))
