"""C ABI surface on the CPU: the library loads, exports every function
include/*.h declares, and reports errors as status codes (no GPU needed:
only argument-validation paths and device discovery are exercised)."""
import ctypes as C
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"\b(fnd_\w+)\s*\(", src)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(built):
    from foundation_gb300 import rt
    lib = rt.load()
    names = declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", rt.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (fnd_\w+)", out))
    assert set(names) <= exported
    # the binding declares a signature for every symbol in the header
    assert set(names) <= set(rt.SIGNATURES)


def test_binding_constants_match_the_header():
    """The BVH flags (and the clustering radius field) of the Python binding
    are the header's."""
    from foundation_gb300 import rt
    src = open(os.path.join(ROOT, "include", "fnd_rt.h")).read()
    enums = {k: int(v) for k, v in re.findall(r"enum \{ (FND_\w+) = (\d+)u \};", src)}
    for name in ("BVH_SPATIAL_SPLITS", "BVH_GPU_BUILD", "BVH_SAH_COLLAPSE", "BVH_GPU_CLUSTER"):
        assert enums["FND_" + name] == getattr(rt, name), name
    shift = int(re.search(r"#define FND_BVH_CLUSTER_RADIUS\(r\) \(\(uint32_t\)\(r\) << (\d+)\)", src).group(1))
    assert rt.BVH_CLUSTER_RADIUS(5) == 5 << shift


def test_null_arguments_return_status(built):
    from foundation_gb300 import rt
    lib = rt.load()
    assert lib.fnd_rt_trace_closest(None, None, None, 0, None, 0) == -1
    assert lib.fnd_rt_trace_any(None, None, None, 0, None, 0) == -1
    assert lib.fnd_rt_destroy(None) == -1
    assert lib.fnd_rt_sync(None) == -1
    assert lib.fnd_rt_scene_destroy(None) == -1
    assert lib.fnd_rt_create(None, None) == -1
    assert lib.fnd_rt_last_error(None)


def test_bad_abi_version_rejected(built):
    from foundation_gb300 import rt
    d = rt._Desc(999, 0, None, 0)
    h = C.c_void_p()
    assert rt.load().fnd_rt_create(C.byref(d), C.byref(h)) == -1
    assert b"ABI version" in rt.load().fnd_rt_last_error(None)


def test_create_without_gpu_fails_cleanly(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from foundation_gb300 import rt
    with pytest.raises(rt.FndError) as e:
        rt.Context(0)
    assert e.value.code in (-3, -4)


def test_python_binding_fails_loudly_without_library(tmp_path):
    from foundation_gb300 import rt
    with pytest.raises(rt.FndError):
        rt.load(str(tmp_path / "missing.so"))
