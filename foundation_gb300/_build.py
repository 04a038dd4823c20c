"""In-tree build of the native library (libfnd_rt.so) with nvcc for sm_103a.

Compiles every translation unit under csrc/ in parallel (one -gencode, no
cmake) and links one shared library into foundation_gb300/lib/. Objects go
to foundation_gb300/_build/ and are rebuilt when a source or any header is
newer than the object.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ_DIR = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libfnd_rt.so")
DEMO_PATH = os.path.join(LIB_DIR, "fnd_pass_demo")
RENDERER = os.path.join(PKG, "renderer")
# measurement kernels of the benchmark (not part of libfnd_rt.so)
PROBE_SRC = os.path.join(PKG, "probe", "l2_read.cu")
PROBE_PATH = os.path.join(LIB_DIR, "libfnd_probe.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++20", "-lineinfo", "-Xcompiler", "-fPIC,-O3,-pthread,-Wall",
          f"-I{os.path.join(ROOT, 'include')}"]
# host sources: contraction off so host float code matches its stated
# expression trees on both x86-64 and aarch64 hosts
HOST_FLAGS = ["-Xcompiler", "-ffp-contract=off"]
# path-tracing stages: the vertex logic (pt/shade.cuh) is inlined into the
# wavefront shade kernel, the tail megakernel and the training megakernel;
# without contraction the three evaluate it to the same bits, so a path gives
# the same result whichever kernel runs it. The raster pass likewise keeps
# the expression tree its scalar restatement evaluates.
PT_FLAGS = ["-fmad=false"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found (set NVCC or put the CUDA toolkit on PATH)")


def _sources():
    srcs = sorted(glob.glob(os.path.join(CSRC, "**", "*.cu"), recursive=True))
    srcs += sorted(glob.glob(os.path.join(CSRC, "**", "*.cpp"), recursive=True))
    return srcs


def _headers():
    hs = glob.glob(os.path.join(CSRC, "**", "*.h*"), recursive=True)
    hs += glob.glob(os.path.join(CSRC, "**", "*.cuh"), recursive=True)
    hs += glob.glob(os.path.join(ROOT, "include", "*.h"))
    return hs


def _obj_for(src: str) -> str:
    rel = os.path.relpath(src, CSRC).replace(os.sep, "__")
    return os.path.join(OBJ_DIR, rel + ".o")


def _compile(src: str, force: bool, newest_header: float) -> tuple[str, bool]:
    obj = _obj_for(src)
    if not force and os.path.exists(obj):
        t = os.path.getmtime(obj)
        if t >= os.path.getmtime(src) and t >= newest_header:
            return obj, False
    cmd = [nvcc(), *ARCH, *COMMON]
    if src.endswith(".cpp"):
        cmd += HOST_FLAGS
    elif os.path.basename(os.path.dirname(src)) in ("pt", "raster"):
        cmd += PT_FLAGS
    cmd += ["-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj, True


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    srcs = _sources()
    newest = max((os.path.getmtime(h) for h in _headers()), default=0.0)
    jobs = min(len(srcs), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, force, newest), srcs))
    objs = [o for o, _ in results]
    rebuilt = any(b for _, b in results)
    if rebuilt or force or not os.path.exists(LIB_PATH) or \
            any(os.path.getmtime(o) > os.path.getmtime(LIB_PATH) for o in objs):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
        if verbose:
            print(f"linked {LIB_PATH}", file=sys.stderr)
    _build_demo(force, verbose)
    _build_probe(force, verbose)
    return LIB_PATH


def _build_probe(force: bool, verbose: bool) -> None:
    """The benchmark's L2 read-bandwidth kernel (probe/l2_read.cu)."""
    if not force and os.path.exists(PROBE_PATH) and os.path.getmtime(PROBE_SRC) <= os.path.getmtime(PROBE_PATH):
        return
    tmp = PROBE_PATH + f".tmp{os.getpid()}"
    cmd = [nvcc(), *ARCH, *COMMON, "-shared", PROBE_SRC, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"probe build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, PROBE_PATH)
    if verbose:
        print(f"linked {PROBE_PATH}", file=sys.stderr)


def _build_demo(force: bool, verbose: bool) -> None:
    """The C++ path-tracer pass (renderer/) and its headless driver, linked
    against libfnd_rt.so with an $ORIGIN rpath."""
    srcs = sorted(glob.glob(os.path.join(RENDERER, "*.cpp")))
    deps = srcs + glob.glob(os.path.join(RENDERER, "*.hpp")) + _headers() + [LIB_PATH]
    if not force and os.path.exists(DEMO_PATH) and \
            all(os.path.getmtime(d) <= os.path.getmtime(DEMO_PATH) for d in deps):
        return
    cxx = os.environ.get("CXX", "g++")
    tmp = DEMO_PATH + f".tmp{os.getpid()}"
    cmd = [cxx, "-O2", "-std=c++20", "-pthread", f"-I{os.path.join(ROOT, 'include')}", "-I/usr/local/cuda/include",
           *srcs, "-o", tmp, f"-L{LIB_DIR}", "-lfnd_rt", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"demo build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, DEMO_PATH)
    if verbose:
        print(f"linked {DEMO_PATH}", file=sys.stderr)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
