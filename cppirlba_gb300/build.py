"""In-tree build of the GB300 engine (sm_103a) and of the host data generator.

Outputs (git-ignored): cppirlba_gb300/_lib/libirlba_gb300.so and
cppirlba_gb300/_lib/libirlba_gb300_datagen.so. Translation units compile in
parallel; nothing here needs a GPU.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
BUILD = os.path.join(HERE, "_lib", "obj")

CUDA_SOURCES = ["engine.cu", "spmv.cu", "vec.cu", "svd.cu", "batch.cu", "batch_host.cu", "adjoint.cu",
                "adjoint_host.cu", "ingest.cu", "staging.cu", "rotate_tc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-O3", "-Xcompiler", "-pthread", "-Xcompiler", "-Wall",
              "-Xcompiler", "-Werror=infinite-recursion"] + ARCH


def _cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _run(cmd):
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), res.stdout))
    return res.stdout


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _torch_compile_cmd(src, obj):
    """g++ command compiling the libtorch extension source against the
    installed torch (no ninja needed)."""
    import sysconfig
    import torch
    from torch.utils import cpp_extension
    inc = []
    for d in cpp_extension.include_paths() + [sysconfig.get_paths()["include"], os.path.join(_cuda_home(), "include")]:
        inc += ["-I", d]
    abi = int(torch._C._GLIBCXX_USE_CXX11_ABI)
    return (["g++", "-O2", "-std=c++17", "-fPIC", "-w", "-c", src, "-o", obj,
             "-DTORCH_EXTENSION_NAME=_irlba_torch", "-DTORCH_API_INCLUDE_EXTENSION_H",
             "-D_GLIBCXX_USE_CXX11_ABI=%d" % abi] + inc)


def build(verbose=False, force=False, torch_ext=True):
    """Builds libirlba_gb300.so, the data generator and (torch_ext) the libtorch
    extension _irlba_torch.so; all translation units compile in parallel."""
    os.makedirs(BUILD, exist_ok=True)
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h", ".hpp"))]
    api = os.path.join(HERE, "..", "include", "irlba_gb300.h")
    headers.append(api)

    lib = os.path.join(OUT, "libirlba_gb300.so")
    objs = []
    jobs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", s, "-o", o])
    tsrc = os.path.join(CSRC, "torch_ops.cpp")
    tobj = os.path.join(BUILD, "torch_ops.o")
    if torch_ext and (force or _stale(tobj, [tsrc, api])):
        jobs.append(_torch_compile_cmd(tsrc, tobj))
    with ThreadPoolExecutor(max_workers=max(len(jobs), 1)) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or _stale(lib, objs):
        _run([nvcc] + ARCH + ["-shared", "-cudart", "shared", "-o", lib] + objs +
             ["-Xlinker", "-rpath," + os.path.join(cuda, "lib64")])

    dg = os.path.join(OUT, "libirlba_gb300_datagen.so")
    dsrc = os.path.join(CSRC, "datagen.cpp")
    if force or _stale(dg, [dsrc]):
        _run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread", dsrc, "-o", dg])

    if torch_ext:
        ext = os.path.join(OUT, "_irlba_torch.so")
        if force or _stale(ext, [tobj, lib]):
            from torch.utils import cpp_extension
            tlib = cpp_extension.library_paths()[0]
            _run(["g++", "-shared", tobj, "-o", ext, "-L", tlib, "-Wl,-rpath," + tlib, "-ltorch", "-ltorch_cpu",
                  "-ltorch_python", "-lc10", "-lc10_cuda", "-L", OUT, "-lirlba_gb300", "-Wl,-rpath,$ORIGIN",
                  "-L", os.path.join(cuda, "lib64"), "-lcudart"])
    return lib, dg


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
