"""The C++ pass as a Foundation application would build it.

CPU: the pass (renderer/PathTracerPass.cpp, renderer/FrameLoop.cpp) and a
minimal application around it (tests/native/foundation_link_check.cpp) are
compiled with FND_IN_FOUNDATION against Foundation's own src/Core headers
(Core.hpp, Allocator/Allocator.hpp) and linked with libfnd_rt.so. The pass
then takes Foundation's Core::Allocator, with its six virtual functions, and
its failures go through Foundation's BugCheck: run here without a GPU, the
program must reach BugCheck with the library's message. The library itself
defines no Foundation::Core symbol that could clash with the application's.

GPU: the same program built against the standalone declarations
(renderer/FoundationCore.hpp) draws a frame of a one-triangle scene under a
white sky: 0.5 on the Lambertian triangle (albedo 0.5), 1.0 on the sky, and
every host byte back in the allocator.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "foundation_gb300", "lib")
RENDERER = os.path.join(ROOT, "foundation_gb300", "renderer")
OUT = os.path.join(ROOT, "tests", "_build")
# Foundation's source tree (read-only); the CPU test is skipped where it is absent
FOUNDATION_SRC = os.environ.get("FOUNDATION_SRC", "/root/reference/src")


def _compile(out, *extra):
    os.makedirs(OUT, exist_ok=True)
    cmd = [os.environ.get("CXX", "g++"), "-std=c++20", "-O1", "-Wall", f"-I{os.path.join(ROOT, 'include')}",
           os.path.join(ROOT, "tests", "native", "foundation_link_check.cpp"),
           os.path.join(RENDERER, "FrameLoop.cpp"), os.path.join(RENDERER, "PathTracerPass.cpp"), *extra,
           f"-L{LIB}", "-lfnd_rt", f"-Wl,-rpath,{LIB}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, " ".join(cmd) + "\n" + r.stderr[-4000:]
    return out


@pytest.mark.skipif(not os.path.exists(os.path.join(FOUNDATION_SRC, "Core", "Allocator", "Allocator.hpp")),
                    reason="Foundation's source tree is not present")
def test_pass_builds_against_foundation_core(built):
    exe = _compile(os.path.join(OUT, "foundation_link_check_in_foundation"), "-DFND_IN_FOUNDATION",
                   f"-I{FOUNDATION_SRC}")
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")  # no device: the create call must fail through BugCheck
    r = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 3, r.stdout + r.stderr
    assert "ExceptionHandler: fnd_rt_create failed (" in r.stdout
    assert "BugCheck at" in r.stdout and "PathTracerPass.cpp" in r.stdout


def test_library_defines_no_foundation_core_symbols(built):
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    r = subprocess.run([nm, "-DC", "--defined-only", os.path.join(LIB, "libfnd_rt.so")], capture_output=True,
                       text=True, check=True)
    clashes = [ln for ln in r.stdout.splitlines() if "Foundation::Core::" in ln]
    assert not clashes, clashes[:10]


@pytest.mark.gpu
def test_pass_draws_a_frame_standalone(built):
    exe = _compile(os.path.join(OUT, "foundation_link_check_standalone"),
                   os.path.join(RENDERER, "FoundationCoreStandalone.cpp"))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "spp 8 centre 0.5000 0.5000 0.5000 corner 1.0000 1.0000 1.0000 used 0" in r.stdout
