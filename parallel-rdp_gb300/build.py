"""Builds the native libraries of the package in-tree (csrc/_build/).

    librdp_cuda.so    - the RDP path: host command processor + sm_103a kernels
    librdp_cmdgen.so  - seeded synthetic command-stream generator (inputs)

Translation units are compiled in parallel; objects are rebuilt only when a
source or header is newer than the object.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(CSRC, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I" + INCLUDE]

CUDA_SOURCES = ["rdp_kernels.cu", "rdp_cp.cpp", "vi.cu", "sched.cu", "rdp_dump.cpp", "coherency.cu", "upscale.cu"]
HEADERS = ["rdp_types.h", "rdp_kernels.h", "blender_divider_runs.inc", "vi.h", "sched.h", "rdp_exec.h", "rdp_coherency.h", "rdp_upscale.h"]


def _newer(src_paths, target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(p) > t for p in src_paths if os.path.exists(p))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "rdp_cuda.h")]
    objs, jobs = [], []
    for src in CUDA_SOURCES:
        sp = os.path.join(CSRC, src)
        obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        if _newer([sp] + deps, obj):
            lang = [] if src.endswith(".cu") else ["-x", "cu"]
            jobs.append([NVCC] + NVCC_FLAGS + lang + ["-c", sp, "-o", obj])
    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                print(out)
    lib = os.path.join(OUT, "librdp_cuda.so")
    if _newer(objs, lib):
        _run([NVCC] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"])
    gen_src = os.path.join(CSRC, "cmdgen.cpp")
    gen_lib = os.path.join(OUT, "librdp_cmdgen.so")
    if _newer([gen_src, os.path.join(INCLUDE, "rdp_cmdgen.h")], gen_lib):
        _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I" + INCLUDE, "-o", gen_lib, gen_src])
    return lib, gen_lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
