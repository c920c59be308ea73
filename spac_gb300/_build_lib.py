"""In-tree build of libspac_fk.so for sm_103a (nvcc + g++, no cmake).

Objects and the library go to spac_gb300/_build/.  Translation units compile
in parallel; a unit is rebuilt when its source or any header changed.
"""
import concurrent.futures as _cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INC = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(OUT, "libspac_fk.so")

CUDA_SOURCES = ["fk_paths.cu", "fk_paths_plain.cu", "fk_kernels.cu", "fk_api.cu", "fk_mlp.cu", "fk_noalloc.cu", "fk_disk.cu"]
CXX_SOURCES = ["fk_mesh.cpp", "fk_host.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + INC]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-I" + INC]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libspac_fk")


def _headers():
    return [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))] + \
        [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]


def _stale(obj, src, headers):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + headers)


def _compile(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose=False, extra_nvcc=()):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    jobs, objs = [], []
    for f in CUDA_SOURCES:
        src, obj = os.path.join(SRC, f), os.path.join(OUT, f + ".o")
        objs.append(obj)
        if _stale(obj, src, headers):
            jobs.append([nvcc] + ARCH + NVCC_FLAGS + list(extra_nvcc) + ["-c", src, "-o", obj])
    for f in CXX_SOURCES:
        src, obj = os.path.join(SRC, f), os.path.join(OUT, f + ".o")
        objs.append(obj)
        if _stale(obj, src, headers):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", obj])
    with _cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_compile, jobs):
            if verbose and out.strip():
                print(out)
    if jobs or not os.path.exists(LIB):
        _compile([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB
