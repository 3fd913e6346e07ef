"""Builds libhe4g.so (the sm_103a time step behind include/he4g.h) in-tree.

The translation units are compiled in parallel with nvcc for sm_103a only and
linked into he4gpu/_lib/libhe4g.so with the CUDA runtime linked statically,
so the library loads on a host without a GPU (it needs the driver only when a
call touches the device).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libhe4g.so")
DRIVER_SRC = os.path.join(ROOT, "host", "he4g_driver.cpp")
DRIVER = os.path.join(OUT_DIR, "he4g_driver")
SOURCES = ["fft_reg_df.cu", "fft_reg.cu", "fft_xy.cu", "api.cu", "field.cu", "fieldmp.cu", "fielddf.cu", "fft.cu", "setup.cpp", "setup_dev.cu", "noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhe4g.so")


def _compile(src, obj, extra):
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj, "-O3", "-std=c++17", "-lineinfo",
           "-Xcompiler", "-fPIC,-ffp-contract=off", *ARCH, *extra]
    if src.endswith(".cpp"):
        cmd[cmd.index("-lineinfo")] = "-x=c++"
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(ROOT), "include", "he4g.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_driver(force=False):
    """The native host driver (host/he4g_driver.cpp), linked against
    libhe4g.so with an rpath to its directory; returns its path."""
    if not force and os.path.exists(DRIVER) and os.path.getmtime(DRIVER) >= max(
            os.path.getmtime(DRIVER_SRC), os.path.getmtime(LIB)):
        return DRIVER
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("no C++ compiler for the host driver")
    inc = os.path.join(os.path.dirname(ROOT), "include")
    cmd = [cxx, "-O2", "-std=c++17", "-I", inc, DRIVER_SRC, "-o", DRIVER + ".tmp", "-L", OUT_DIR, "-lhe4g",
           "-Wl,-rpath,$ORIGIN", "-Wl,--allow-shlib-undefined"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"host driver build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(DRIVER + ".tmp", DRIVER)
    return DRIVER


def build(force=False, verbose=False):
    """Compiles and links libhe4g.so if any source is newer, then the host
    driver; returns the library's path."""
    if not force and not _stale():
        build_driver()
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    objdir = os.path.join(OUT_DIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose else []
    objs = [os.path.join(objdir, s + ".o") for s in SOURCES]
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        logs = list(ex.map(lambda a: _compile(a[0], a[1], extra), zip(SOURCES, objs)))
    if verbose:
        for log in logs:
            sys.stderr.write(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", *ARCH, "-o", tmp, *objs, "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_driver(force=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
