"""Build the GB300 CUDA library in-tree: voxelhashmt_gb300/_lib/libvoxelhash_gb300.so.

One nvcc invocation per translation unit (run in parallel), one -gencode (sm_103a), then a shared link.
Device code is compiled with -fmad=false and host code with -ffp-contract=off so that every a*b+c of
the reference algorithm rounds twice, as the reference source is written; -prec-div / -prec-sqrt keep
their IEEE defaults.  The one exception is the second compile of vh_integrate.cu (VARIANTS): the opt-in
fast-math update pass, namespace vh::fast, built with -use_fast_math.

usage: python -m voxelhashmt_gb300.build [--force]
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libvoxelhash_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["vh_filter.cu", "vh_alloc.cu", "vh_integrate.cu", "vh_mesh.cu", "vh_misc.cu", "vh_render.cu",
           "vh_raycast.cu", "vh_static_scratch.cu", "vh_weld.cu", "vh_expf.cu", "vh_evict.cu", "vh_capi.cpp", "vh_png.cpp", "vh_dataset.cpp"]
# second compile of the update pass: the fast-math form (vh::fast), object name and extra device flags
VARIANTS = [("vh_integrate.cu", "vh_integrate_fast", ["-DVH_FAST_MATH", "-use_fast_math", "-fmad=true"]),
            # the denoiser's kernels: ordinary FP32 rounding (contraction allowed), no parity contract
            ("vh_nn.cu", "vh_nn", ["-fmad=true"])]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
         "-I", CSRC, "-I", INCLUDE]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "voxelhash_gb300.h"))
    files.append(os.path.abspath(__file__))
    return files


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed: %s\n%s\n%s" % (" ".join(cmd), res.stdout, res.stderr))
    return res


def build(force=False, verbose=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(f) for f in _deps()):
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    objs = []

    def compile_one(unit):
        src, name, extra = unit
        obj = os.path.join(LIBDIR, name + ".o")
        flags = [f for f in FLAGS if not (extra and f == "-fmad=false")]
        cmd = [nvcc(), *ARCH, *flags, *extra, "-x", "cu", "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = _run(cmd)
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    units = [(src, os.path.splitext(src)[0], []) for src in SOURCES] + VARIANTS
    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(compile_one, units))
    _run([nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs])
    os.replace(LIB + ".tmp", LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
