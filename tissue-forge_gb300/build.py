"""Build recipe of libtfg.so (CUDA kernels for sm_103a + host C++), in-tree.

Usage: python tissue-forge_gb300/build.py [--force]
Outputs tissue-forge_gb300/_build/libtfg.so.  Translation units compile in parallel.
Host code is compiled with -ffp-contract=off so that host-side float arithmetic
(cell origins, table construction) matches the reference's non-FMA x86 build on
every host architecture.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libtfg.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["csrc/tfg_engine.cu", "csrc/tfg_api.cu", "csrc/tfg_kernels.cu", "csrc/tfg_pair.cu",
              "csrc/tfg_pair_tile.cu", "csrc/tfg_pair_home.cu", "csrc/tfg_probe.cu", "csrc/tfg_noalloc.cu"]
CXX_SOURCES = ["host/tfg_potential.cpp", "host/tfg_server.cpp"]
HEADERS = ["csrc/tfg_device.cuh", "csrc/tfg_internal.h", "csrc/tfg_kernels.h", "csrc/tfg_engine_impl.h"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(HERE, "csrc")]
    hdrs = [os.path.join(HERE, h) for h in HEADERS] + [os.path.join(ROOT, "include", "tfg.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(HERE, src)
        o = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            cmd = [NVCC, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-Xptxas", "-v" if verbose else "-O3", *inc, "-c", s, "-o", o]
            jobs.append(cmd)
    for src in CXX_SOURCES:
        s = os.path.join(HERE, src)
        o = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                         "-fvisibility=hidden", *inc, "-c", s, "-o", o])
    procs = [(cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for cmd in jobs]
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append((cmd, out.decode(errors="replace")))
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("libtfg build failed:\n" + msg)
    if force or jobs or _newer(LIB, objs):
        subprocess.check_call([NVCC, "-shared", *ARCH, "-o", LIB, *objs, "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
