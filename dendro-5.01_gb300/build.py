"""Build libdendro_gb300.so (sm_103a) in-tree: one nvcc/g++ job per source,
in parallel, then one link.  Usage: python build.py [--verbose]"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libdendro_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xptxas", "-v", "--expt-relaxed-constexpr"]
# extra nvcc flags for build experiments, e.g. DGB_NVCC_EXTRA="-DDGB_RHS_MIN_CTAS=1"
NVCC_FLAGS += os.environ.get("DGB_NVCC_EXTRA", "").split()
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-fopenmp", "-ffp-contract=off",
             "-Wall", "-Wno-unused-function"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def compile_one(src):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    if src.endswith(".cu"):
        cmd = [nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-I" + os.path.join(HERE, "..", "include"),
                                     "-I/usr/local/cuda/include", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, obj, r.returncode, r.stdout + r.stderr


def newer(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")))
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "dendro_gb300.h"))
    # a change of compiler flags rebuilds everything
    stamp = os.path.join(OUT, "flags.txt")
    flags = " ".join(NVCC_FLAGS + CXX_FLAGS)
    same_flags = os.path.exists(stamp) and open(stamp).read() == flags
    todo = [s for s in srcs
            if not same_flags or newer(os.path.join(OUT, os.path.basename(s) + ".o"), [s] + headers)]
    logs = {}
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 4))) as ex:
        for src, obj, rc, log in ex.map(compile_one, todo):
            logs[src] = log
            if verbose or rc != 0:
                sys.stderr.write(log)
            if rc != 0:
                raise RuntimeError(f"compile failed: {src}")
    with open(stamp, "w") as f:
        f.write(flags)
    objs = [os.path.join(OUT, os.path.basename(s) + ".o") for s in srcs]
    if todo or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    with open(os.path.join(OUT, "ptxas.log"), "a") as f:
        for src, log in logs.items():
            f.write(f"== {src}\n{log}\n")
    return LIB


if __name__ == "__main__":
    build(verbose="--verbose" in sys.argv)
    print(LIB)
