"""Build libopenqp_gb300.so in-tree for sm_103a (GB300).

Each translation unit is compiled by its own nvcc process (they run in
parallel), then linked into one shared library with a C ABI
(include/openqp_gb300.h).  No cmake; the same recipe works on the x86 build
container (cross-compile) and on the Arm GPU hosts.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libopenqp_gb300.so")
SOURCES = ["oqpg_cls_%d.cu" % g for g in (17, 15, 14, 16, 2, 3, 4, 18, 13, 12, 11, 10, 9, 8, 7, 6, 5, 1, 0)] + \
    ["oqpg_grad_cls_f%d.cu" % g for g in range(5)] + \
    ["oqpg_grad_cls_a.cu", "oqpg_grad_cls_b.cu", "oqpg_host.cu", "oqpg_noalloc.cu", "oqpg_onee.cu", "oqpg_grad_host.cu",
     "oqpg_response.cu", "oqpg_sigma.cu", "oqpg_petite.cu", "oqpg_family.cu", "oqpg_family_df.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
         "-diag-suppress", "128,177,550"]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h", ".inc"))] + \
        [os.path.join(os.path.dirname(HERE), "include", "openqp_gb300.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        cmd = [cc] + ARCH + FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s" % (src, r.stderr))
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcublas", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
