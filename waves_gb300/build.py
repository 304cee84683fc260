"""Build recipe of the product library libwaves_gb300.so (in-tree, sm_103a only).

Every translation unit is compiled with -fmad=false (no implicit multiply-add contraction) and the
host code with -ffp-contract=off, so that each FP32 operation is the one the source spells out.
Objects compile in parallel; the result is waves_gb300/_build/libwaves_gb300.so.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libwaves_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                  "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fno-fast-math"]
SOURCES = ["waves_abi.cu", "k_pcg.cu", "k_motion.cu", "k_geom.cu", "k_mg.cu", "k_init.cu", "k_net.cu", "k_train.cu", "k_render.cu", "noalloc.cu", "config.cpp"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _compile(src, verbose=False):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + NVFLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def _stale(objs):
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "waves.h"),
                                                                 os.path.join(HERE, "harness", "waves_run.c")]
    if not os.path.exists(HARNESS):
        return True
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    if not force and not _stale(None):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if verbose:
        for _, err in results:
            sys.stderr.write(err)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_harness()
    return LIB


HARNESS = os.path.join(OUT, "waves_run")


def build_harness():
    """The headless C driver (harness/waves_run.c), linked against the library with an rpath."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler for the harness")
    cuda = os.path.dirname(os.path.dirname(nvcc()))
    cmd = [cc, "-std=c11", "-O2", "-Wall", "-I", os.path.join(HERE, "..", "include"),
           os.path.join(HERE, "harness", "waves_run.c"), "-o", HARNESS, "-L", OUT, "-lwaves_gb300",
           "-Wl,-rpath,$ORIGIN", "-L", os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(cuda, "lib64"), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"harness build failed:\n{r.stdout}\n{r.stderr}")
    return HARNESS


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
