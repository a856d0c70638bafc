"""Build libgp103.so (the CUDA kernels behind the C ABI of include/gp103.h) in-tree, for sm_103a only.

    python -m autoplace_gb300.build          # or: import autoplace_gb300.build as b; b.build()

Each .cu file is compiled by nvcc in parallel (-gencode arch=compute_103a,code=sm_103a), then linked into
autoplace_gb300/_lib/libgp103.so with the static CUDA runtime (no dependency on torch's libraries)."""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libgp103.so")
SOURCES = ["wa.cu", "density.cu", "step.cu", "field.cu", "field_tc.cu", "api.cu", "eval.cu", "build.cu", "cluster.cu", "setup.cu", "noalloc.cu", "learn.cu", "batch.cu"]
# The density kernels flush float32 denormals as the reference's kernels do (they are built with --use_fast_math).
PER_FILE = {"density.cu": ["-ftz=true"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is needed to build libgp103")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(HERE), "include", "gp103.h"))
    return max(os.path.getmtime(f) for f in files)


def up_to_date():
    return os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps()


def build(force=False, verbose=False):
    """Compile and link libgp103.so unless it is newer than every source. -> path of the library."""
    if not force and up_to_date():
        return LIB
    os.makedirs(os.path.join(OUT_DIR, "obj"), exist_ok=True)
    cc = nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + CSRC]

    def one(src):
        obj = os.path.join(OUT_DIR, "obj", src.replace(".cu", ".o"))
        cmd = [cc] + common + PER_FILE.get(src, []) + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
