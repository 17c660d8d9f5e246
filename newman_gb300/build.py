"""Builds the in-tree shared library newman_gb300/_lib/libnewman_gb300.so.

CUDA sources are compiled for sm_103a only; host C++ with g++.  Objects go to
newman_gb300/_build/.  Runs the compilers in parallel and skips the link when
every object is newer than its sources.
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libnewman_gb300.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# Per-file nvcc flags: the FP64 reference-order kernels never contract.
CU_FLAGS = {
    "render_fp64.cu": ["--fmad=false"],
    "render_mp.cu": ["--fmad=false"],
}


def _deps():
    return glob.glob(os.path.join(CSRC, "*.h*")) + glob.glob(os.path.join(CSRC, "*.cuh")) + [
        os.path.join(ROOT, "include", "newman_gb300.h")]


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + deps)


def build(force=False, verbose=False, ptxas_verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    deps = _deps()
    inc = ["-I", CSRC, "-I", os.path.join(ROOT, "include")]
    jobs, objs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        name = os.path.basename(src)
        obj = os.path.join(BUILD, name + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                   "-c", src, "-o", obj] + inc + CU_FLAGS.get(name, [])
            if ptxas_verbose:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread",
                         "-I", os.path.join(CUDA_HOME, "include"), "-c", src, "-o", obj] + inc)
    procs = []
    for cmd in jobs:
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if out and (verbose or p.returncode or ptxas_verbose):
            sys.stdout.write(out.decode(errors="replace"))
        if p.returncode:
            failed.append(cmd[-1] if cmd[0] == "g++" else cmd)
    if failed:
        raise RuntimeError("compilation failed: %s" % failed)
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-l:libgmp.so.10", "-lpthread"]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                ptxas_verbose="--ptxas" in sys.argv))
