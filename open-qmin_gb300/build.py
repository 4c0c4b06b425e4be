"""Build recipe for the qmin_gb300 native library (sm_103a only).

Compiles the CUDA translation units and the host set-up code in parallel with
nvcc / g++ and links ``_build/libqmin_gb300.so``.  Also builds the C++ host
drop-in example.  No CMake, no torch extension machinery: the library is a
plain C-ABI shared object.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libqmin_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build qmin_gb300")
    return cand


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "qmin_gb300.h"))
    units = ["qmin_kernels.cu", "qmin_fused.cu", "qmin_capi.cu", "qmin_batch.cu", "qmin_host_setup.cpp",
             "qmin_noalloc.cu", "qmin_warmnet.cu", "qmin_tiled.cu", "qmin_io.cpp", "qmin_split.cu",
             "qmin_geometry.cu"]
    objs, jobs = [], []
    for u in units:
        src = os.path.join(CSRC, u)
        obj = os.path.join(OUT, u.rsplit(".", 1)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
                                   "-ffp-contract=off", "-c", src, "-o", obj]
            if u.endswith(".cu"):
                cmd += ["-Xptxas", "-v"] if verbose else []
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                print(out)
    if force or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    # C++ host drop-in example (compile check + GPU example run)
    ex_src = os.path.join(HERE, "host", "example_fire.cpp")
    ex_bin = os.path.join(OUT, "example_fire")
    if os.path.exists(ex_src) and (force or _stale(ex_bin, [ex_src, LIB, os.path.join(HERE, "host", "qmin_gb300.hpp")])):
        _run(["g++", "-std=c++17", "-O2", "-I", os.path.join(HERE, "..", "include"), "-I", os.path.join(HERE, "host"),
              ex_src, "-o", ex_bin, "-L", OUT, "-lqmin_gb300", "-Wl,-rpath," + OUT])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
