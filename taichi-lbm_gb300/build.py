"""Build the CUDA library liblbm_gb300.so in-tree for sm_103a.

Each translation unit under csrc/ is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo`` and linked into
``taichi_lbm/_lib/liblbm_gb300.so`` (git-ignored; rebuilt on every machine).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "taichi_lbm", "_lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liblbm_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no implicit fma contraction, so a node computes bit for bit
# alike in every kernel that shares the source (fused multiply-adds are
# written out as fmaf where the hot paths want them)
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--use_fast_math=false", "-fmad=false"]


def _nvcc():
    nv = shutil.which("nvcc")
    if nv:
        return nv
    for cand in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbm_gb300.so")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    inc = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    inc.append(os.path.join(os.path.dirname(HERE), "include", "lbm_gb300.h"))
    return inc


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, ptxas_v=False):
    nvcc = _nvcc()
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    deps = _deps()
    srcs = sources()
    objs = [os.path.join(OBJ_DIR, os.path.basename(s)[:-3] + ".o") for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if force or _stale(o, s, deps)]
    extra = [s.replace("--use_fast_math=false", "") for s in FLAGS if s != "--use_fast_math=false"]
    if ptxas_v:
        extra = extra + ["-Xptxas", "-v"]

    def compile_one(so):
        s, o = so
        cmd = [nvcc] + ARCH + extra + ["-c", s, "-o", o + ".tmp"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(s)}:\n{r.stderr}")
        os.replace(o + ".tmp", o)
        return r.stderr

    logs = []
    if todo:
        with cf.ThreadPoolExecutor(max_workers=min(len(todo), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(compile_one, todo))
    if todo or force or not os.path.exists(LIB):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    if ptxas_v:
        return LIB, "\n".join(logs)
    return LIB


if __name__ == "__main__":
    res = build(force="--force" in sys.argv, verbose=True, ptxas_v="--ptxas-v" in sys.argv)
    if isinstance(res, tuple):
        print(res[1])
        res = res[0]
    print(res)
