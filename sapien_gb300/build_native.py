"""Build libsgdyn.so (CUDA kernels + C ABI + host model builder) in-tree for sm_103a.

Translation units compile in parallel with nvcc; objects go to sapien_gb300/_build/ and
the shared library to sapien_gb300/_lib/libsgdyn.so (both git-ignored). The CUDA runtime
is linked statically so the library only needs the driver at run time.
"""
from __future__ import annotations

import glob
import os
import platform
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libsgdyn.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# The host instantiation of the sweeps (single-configuration calls) calls fma() throughout:
# on x86-64 it needs the FMA instructions (every x86-64 CPU since 2013 has them) or each
# call goes to the C library; aarch64 always has them. fma rounds once either way, and the
# compiler is kept from fusing other products and sums, so host results stay what they were.
HOST_FLAGS = (["-Xcompiler", "-mfma", "-Xcompiler", "-ffp-contract=off"]
              if platform.machine() in ("x86_64", "AMD64") else [])
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                     "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC] + HOST_FLAGS


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.exists(cand) or cand == "nvcc"):
            return cand
    return "nvcc"


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers_mtime():
    hs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(
        os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _compile(src, hmt, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hmt):
        return obj, None
    cmd = [_nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, f"{src}:\n{r.stdout}\n{r.stderr}"
    return obj, None


JIT_HEADERS = ("device_model.h", "kernels.h", "spatial.cuh", "se3.cuh", "step_kernel.cuh", "diff_core.cuh",
               "diff_kernels.cuh", "team3.cuh")


def _write_jit_headers():
    """Embed the device headers the run-time compiler needs into a generated C++ file."""
    out = os.path.join(BUILD, "jit_headers.cpp")
    parts = ["// generated by build_native.py: device headers for run-time compilation",
             "namespace sgdyn {",
             "extern const char* const kJitHeaderNames[] = {" + ", ".join(f'"{h}"' for h in JIT_HEADERS) + "};",
             "extern const char* const kJitHeaderSources[] = {"]
    for h in JIT_HEADERS:
        text = open(os.path.join(CSRC, h)).read()
        assert ")SGJIT\"" not in text
        parts.append('R"SGJIT(' + text + ')SGJIT",')
    parts += ["};", f"extern const int kJitHeaderCount = {len(JIT_HEADERS)};", "}  // namespace sgdyn", ""]
    text = "\n".join(parts)
    if not os.path.exists(out) or open(out).read() != text:
        with open(out, "w") as f:
            f.write(text)
    return out


def build(verbose=False, jobs=None, force=False):
    """Compile all translation units and link libsgdyn.so; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    if force:
        for o in glob.glob(os.path.join(BUILD, "*.o")):
            os.remove(o)
    hmt = _headers_mtime()
    srcs = sources() + [_write_jit_headers()]
    jobs = jobs or min(len(srcs), max(2, os.cpu_count() or 2))
    with ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, hmt, verbose), srcs))
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
    objs = [o for o, _ in results]
    _link(objs, LIB, verbose)
    return LIB


def build_standalone(src, out, verbose=False):
    """Compile one .cu file into its own shared library `out` (same flags as libsgdyn.so)."""
    os.makedirs(os.path.dirname(out), exist_ok=True)
    obj = out + ".o"
    if not (os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)):
        cmd = [_nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{src}:\n{r.stdout}\n{r.stderr}")
    _link([obj], out, verbose)
    return out


def _link(objs, out, verbose):
    newest = max(os.path.getmtime(o) for o in objs)
    if os.path.exists(out) and os.path.getmtime(out) >= newest:
        return
    cmd = [_nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", out] + objs + ["-ldl"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
