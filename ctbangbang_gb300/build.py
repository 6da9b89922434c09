"""Builds libctbb_gb300.so in-tree: CUDA sources for sm_103a, host C++ with
-ffp-contract=off (the planner's float arithmetic must round like the
reference's), compiled in parallel and linked with the static CUDA runtime.

    python -m ctbangbang_gb300.build          # or __graft_entry__.build()
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(REPO, "_build")
LIB = os.path.join(HERE, "libctbb_gb300.so")

CUDA_SOURCES = [
    "abi.cu", "adaptive_filter.cu", "rebin.cu", "ramp_filter.cu", "ramp_tc.cu",
    "backproject.cu", "finalize.cu",
]
HOST_SOURCES = ["planner.cpp", "dicom.cpp", "server.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build ctbangbang_gb300")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, ptxas_info=False):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(REPO, "include", "ctbb_gb300.h"))
    common = ["-O3", "-std=c++17", "-I", os.path.join(REPO, "include"), "-I", CSRC]
    jobs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        cmd = [nvcc, *ARCH, "-lineinfo", *common, "-Xcompiler", "-fPIC,-ffp-contract=off",
               "--expt-relaxed-constexpr", "-c", s, "-o", o]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append((o, [s] + headers, cmd))
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        cmd = [nvcc, *common, "-x", "c++", "-Xcompiler", "-fPIC,-ffp-contract=off", "-c", s, "-o", o]
        jobs.append((o, [s] + headers, cmd))
    todo = [j for j in jobs if _stale(j[0], j[1]) or ptxas_info]
    logs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for out in ex.map(lambda j: _run(j[2]), todo):
            logs.append(out)
    objs = [j[0] for j in jobs]
    if todo or not os.path.exists(LIB) or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lpthread"])
        os.replace(LIB + ".tmp", LIB)
    if verbose or ptxas_info:
        sys.stdout.write("".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv))
