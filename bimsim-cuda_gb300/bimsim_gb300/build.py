"""Build the CUDA library (libbimsim_gb300.so) and the `bimsim` CLI in-tree.

    python -m bimsim_gb300.build        (or bimsim_gb300.build.build())

Sources: bimsim-cuda_gb300/csrc (kernels, C ABI) and bimsim-cuda_gb300/cli.
Outputs: bimsim-cuda_gb300/lib/.  One -gencode (sm_103a), translation units
compiled in parallel; an output is rebuilt only when a source or header is
newer.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))  # bimsim-cuda_gb300/
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
CLI = os.path.join(PKG, "cli")
LIB = os.path.join(PKG, "lib")
OBJ = os.path.join(LIB, "obj")
INCLUDE = os.path.join(REPO, "include")
SO_NAME = "libbimsim_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    nvcc = nvcc_path()
    hdrs = _headers()
    jobs = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            # host code: no contraction, so that single-precision restatements of the reference round as written
            jobs.append([nvcc] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                                         "-Xptxas", "-warn-spills", "-I", INCLUDE, "-I", CSRC,
                                         "-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                         "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    so = os.path.join(LIB, SO_NAME)
    if force or _stale(so, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", so] + objs)
    cli_srcs = sorted(glob.glob(os.path.join(CLI, "*.cpp")))
    if cli_srcs:
        exe = os.path.join(LIB, "bimsim")
        if force or _stale(exe, cli_srcs + [so] + hdrs):
            _run(["g++", "-std=c++17", "-O2", "-I", INCLUDE, "-I", CSRC, "-o", exe] + cli_srcs +
                 ["-L" + LIB, "-lbimsim_gb300", "-Wl,-rpath,$ORIGIN"])
    return so


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
