"""Build the engine library ``libkpm_gb300.so`` in-tree for sm_103a.

Two translation units compiled in parallel: the CUDA kernels (nvcc, one
-gencode for sm_103a) and the host engine (g++), linked by nvcc with the
static CUDA runtime. Output goes to ``pybinding_gb300/_build/``.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libkpm_gb300.so")
INCLUDE = os.path.join(ROOT, "include")
GENCODE = "arch=compute_103a,code=sm_103a"


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


# the pybind11 module over the C ABI: its own extension, linked against LIB
MODULE_SRC = os.path.join(CSRC, "pykpm.cpp")
MODULE_NAME = "_kpm_gb300"


def module_path():
    import sysconfig
    return os.path.join(BUILD, MODULE_NAME + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))


def _pybind11_include():
    """pybind11's headers: the pybind11 package where installed, else the copy PyTorch ships."""
    try:
        import pybind11
        return pybind11.get_include()
    except ImportError:
        pass
    import importlib.util
    spec = importlib.util.find_spec("torch")
    if spec and spec.origin:
        inc = os.path.join(os.path.dirname(spec.origin), "include")
        if os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
            return inc
    raise RuntimeError("pybind11 headers not found (neither the pybind11 package nor PyTorch's copy)")


def sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))
            if f.endswith((".cu", ".cpp")) and os.path.join(CSRC, f) != MODULE_SRC]


def _deps():
    deps = sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    return deps + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]


def _stale():
    for out, deps in ((LIB, _deps()), (module_path(), [MODULE_SRC] + _deps())):
        if not os.path.exists(out):
            return True
        t = os.path.getmtime(out)
        if any(os.path.getmtime(d) > t for d in deps):
            return True
    return False


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    objs, cmds = [], []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if src.endswith(".cu"):
            cmd = [nvcc, "-gencode", GENCODE, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-psabi", "-I", INCLUDE, "-I", CSRC,
                   "-I", os.path.join(cuda, "include"), "-c", src, "-o", obj]
        cmds.append(cmd)

    import sysconfig
    mod_obj = os.path.join(BUILD, "pykpm.cpp.o")
    cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-Wall", "-Wno-psabi", "-I", INCLUDE,
                 "-I", _pybind11_include(), "-I", sysconfig.get_paths()["include"], "-c", MODULE_SRC, "-o", mod_obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        for cmd, r in ex.map(run, cmds):
            if verbose and r.stderr:
                sys.stderr.write(r.stderr)
            if r.returncode != 0:
                raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    tmp = LIB + ".%d.tmp" % os.getpid()
    link = [nvcc, "-shared", "-gencode", GENCODE, "-cudart", "static", "-o", tmp] + objs
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s%s" % (" ".join(link), r.stdout, r.stderr))
    os.replace(tmp, LIB)
    # the module finds libkpm_gb300.so next to itself
    mod = module_path()
    tmp = mod + ".%d.tmp" % os.getpid()
    link = ["g++", "-shared", "-o", tmp, mod_obj, "-L", BUILD, "-l:" + os.path.basename(LIB),
            "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s%s" % (" ".join(link), r.stdout, r.stderr))
    os.replace(tmp, mod)
    return LIB


def build_host_program(src, out=None):
    """Compile and link a C++ program that calls the engine through include/kpm_gb300.h
    (e.g. tests/cpp/host_caller.cpp) against libkpm_gb300.so; returns the executable's path."""
    lib = build()
    out = out or os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0])
    tmp = out + ".%d.tmp" % os.getpid()
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", INCLUDE, src, "-o", tmp, "-L", BUILD,
           "-l:" + os.path.basename(lib), "-Wl,-rpath," + BUILD]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("host program build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
