"""Build of the GB300 HEOM library: every CUDA/C++ source compiled for sm_103a with
nvcc (one -gencode, sources in parallel) and linked into heomq/_lib/libheom_gb300.so."""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUTDIR = os.path.join(HERE, "heomq", "_lib")
LIB = os.path.join(OUTDIR, "libheom_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3", "--expt-relaxed-constexpr"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def sources():
    return sorted(f for f in os.listdir(SRC) if f.endswith((".cu", ".cpp")))


def build(force=False, verbose=False, extra_flags=()):
    os.makedirs(os.path.join(OUTDIR, "obj"), exist_ok=True)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(HERE, "..", "include", "heom_gb300.h")]
    newest = max(os.path.getmtime(p) for p in deps)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    exe = nvcc()

    def compile_one(f):
        obj = os.path.join(OUTDIR, "obj", f + ".o")
        cmd = [exe, *ARCH, *FLAGS, *extra_flags, "-c", os.path.join(SRC, f), "-o", obj]
        if f.endswith(".cpp"):
            cmd = [exe, "-x", "cu", *cmd[1:]]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {f}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = LIB + ".tmp"
    r = subprocess.run([exe, *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
