"""In-tree build of libfcs_cuda.so for sm_103a.

Each CUDA translation unit is compiled by its own ``nvcc`` process (in
parallel), then linked into ``<package>/lib/libfcs_cuda.so``.  No CMake, no
Python extension machinery: the library is a plain C-ABI shared object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(PKG, "_build")
LIB = os.path.join(LIBDIR, "libfcs_cuda.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
           "--expt-relaxed-constexpr"]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _stale(obj, src_deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in src_deps)


def build(verbose: bool = False, force: bool = False, jobs: int | None = None) -> str:
    nvcc = _nvcc()
    home = _cuda_home(nvcc)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    cu, cpp = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(PKG), "include", "fcs.h"))
    cmds = []
    objs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJDIR, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmds.append([nvcc] + ARCH + CUFLAGS + ["-c", src, "-o", obj])
    for f in cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJDIR, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmds.append(["g++"] + CXXFLAGS + ["-I" + os.path.join(home, "include"), "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    if cmds:
        n = jobs or min(len(cmds), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            for cmd, r in ex.map(run, cmds):
                if verbose or r.returncode != 0:
                    sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError(f"compile failed: {cmd[-3]}")
    if force or cmds or not os.path.exists(LIB):
        link = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


PLUGIN = os.path.join(PKG, "plugin")
PLUGIN_BUILD = os.path.join(PLUGIN, "_build")
PLUGIN_LIB = os.path.join(PLUGIN_BUILD, "libFastChemistryModel.so")
STUB_LIB = os.path.join(PLUGIN_BUILD, "libfoamStub.so")


def build_plugin(verbose: bool = False) -> str:
    """libFastChemistryModel.so, the OpenFOAM-side plugin (plugin/), built
    against the OpenFOAM-10 stub of plugin/foam_stub (libfoamStub.so, which
    holds the chemistry-solver selection table) and libfcs_cuda.so.  With an
    OpenFOAM-10 installation the same sources are built by wmake (plugin/Make)."""
    lib = build(verbose=verbose)
    os.makedirs(PLUGIN_BUILD, exist_ok=True)
    inc = ["-I" + PLUGIN, "-I" + os.path.join(PLUGIN, "foam_stub"), "-I" + os.path.join(os.path.dirname(PKG), "include")]
    stub_src = os.path.join(PLUGIN, "foam_stub", "foamStub.C")
    srcs = [os.path.join(PLUGIN, f) for f in os.listdir(PLUGIN) if f.endswith((".C", ".H"))]
    srcs += [os.path.join(PLUGIN, "foam_stub", f) for f in os.listdir(os.path.join(PLUGIN, "foam_stub"))]
    cmds = []
    if _stale(STUB_LIB, [stub_src] + srcs):
        cmds.append(["g++"] + CXXFLAGS + inc + ["-shared", stub_src, "-o", STUB_LIB])
    if _stale(PLUGIN_LIB, srcs + [lib, os.path.join(os.path.dirname(PKG), "include", "fcs.h")]):
        cmds.append(["g++"] + CXXFLAGS + inc + ["-shared", os.path.join(PLUGIN, "odeChemistrySolvers.C"),
                                                "-o", PLUGIN_LIB, "-L" + LIBDIR, "-lfcs_cuda",
                                                "-L" + PLUGIN_BUILD, "-lfoamStub",
                                                "-Wl,-rpath," + LIBDIR, "-Wl,-rpath," + PLUGIN_BUILD])
    for cmd in cmds:
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("plugin build failed")
    return PLUGIN_LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
    print(build_plugin(verbose="-v" in sys.argv))
