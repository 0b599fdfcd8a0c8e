"""In-tree build of libmessi_gb300.so (sm_103a only).

    python -m messi_gb300.build        # or messi_gb300.build.build()

Each source compiles to an object in messi_gb300/_build/ in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo``; the objects link
into messi_gb300/libmessi_gb300.so with the CUDA runtime linked statically.
Rebuilds only when a source or header is newer than the library.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmessi_gb300.so")
SOURCES = ["api.cu", "prune.cu", "scfg.cu", "batch.cu", "decode.cu", "ingest.cu", "noalloc.cu", "mlp.cu", "host_model.cpp", "plan.cpp"]
HEADERS = [os.path.join(CSRC, "internal.h"), os.path.join(CSRC, "wave.cuh"),
           os.path.join(ROOT, "include", "messi_gb300.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build messi_gb300")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3,-fopenmp",
                   "-I" + os.path.join(ROOT, "include")]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0] + ".o")
    if not _stale(obj, [src] + HEADERS):
        return obj
    cmd = [nvcc()] + _flags() + ["-c", src, "-o", obj]
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-warn-spills"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)
    return obj


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    if not force and not _stale(LIB, srcs + HEADERS):
        return LIB
    if force:
        for f in os.listdir(BUILD):
            if f.endswith(".o"):
                os.remove(os.path.join(BUILD, f))
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs + ["-lgomp"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    # a shared library links with unresolved symbols; loading it resolves them
    chk = subprocess.run([sys.executable, "-c", f"import ctypes; ctypes.CDLL({tmp!r})"], capture_output=True,
                         text=True)
    if chk.returncode != 0:
        os.remove(tmp)
        raise RuntimeError(f"built library does not load:\n{chk.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
