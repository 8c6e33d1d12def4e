"""Build the engine library in-tree: scs_gb300/_lib/libscs.so (sm_103a).

Each translation unit is compiled in parallel with nvcc (CUDA) or g++ (host
C++), then linked into one shared library exporting include/scs.h.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU = ["prep.cu", "bnb.cu", "engine.cu", "noalloc.cu", "core.cu", "mlp.cu", "propose.cu"]
CXX = ["host_graph.cpp", "host_api.cpp"]
LIB = "libscs.so"
EXES = {"scs_server": "server.cpp", "scs_client": "client.cpp", "scs_verify": "verify.cpp"}


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _deps_mtime():
    names = os.listdir(CSRC) + [os.path.join("..", "..", "include", "scs.h")]
    return max(os.path.getmtime(os.path.join(CSRC, f)) for f in names)


def lib_path():
    return os.environ.get("SCS_LIB") or os.path.join(OUT, LIB)


def build(verbose=False, force=False, out_dir=None, defines=()):
    """Build into out_dir (default scs_gb300/_lib) with extra -D defines."""
    global OUT
    saved = OUT
    if out_dir:
        OUT = out_dir
    try:
        return _build(verbose, force, list(defines))
    finally:
        OUT = saved


def _build(verbose, force, defines):
    os.makedirs(OUT, exist_ok=True)
    out = os.path.join(OUT, LIB)
    if not force and not defines and os.path.exists(out) and os.path.getmtime(out) >= _deps_mtime():
        return out
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    cmds = []
    for f in CU:
        cmds.append([nvcc(), *ARCH, "-O3", "-std=c++17", "-lineinfo", *defines,
                     "-Xcompiler", "-fPIC", "-c", os.path.join(CSRC, f),
                     "-o", os.path.join(objdir, f + ".o")])
    for f in CXX:
        cmds.append(["g++", "-O3", "-std=c++17", "-fPIC", "-Wall", "-c",
                     os.path.join(CSRC, f), "-o", os.path.join(objdir, f + ".o")])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        list(ex.map(run, cmds))
    objs = [os.path.join(objdir, f + ".o") for f in CU + CXX]
    run([nvcc(), *ARCH, "-shared", "-o", out, *objs, "-lcudart", "-lpthread"])
    # reference-compatible server and batch client, and the answer verifier,
    # linked to the library
    for exe, src in EXES.items():
        run(["g++", "-O2", "-std=c++17", "-Wall", "-o", os.path.join(OUT, exe),
             os.path.join(CSRC, src), "-L" + OUT, "-lscs", "-Wl,-rpath,$ORIGIN",
             "-lpthread"])
    return out


def exe_path(name):
    return os.path.join(OUT, name)


if __name__ == "__main__":
    print(build(verbose=True, force=True))
