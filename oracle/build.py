"""Build recipes for the parity oracle (test infrastructure only).

* ``build_oracle()`` compiles oracle/vh_oracle.c into oracle/liboracle.so with gcc, and again with
  -DVO_FP64 (double arithmetic: the FP64 transcription) into oracle/liboracle64.so.
  ``-ffp-contract=off`` is mandatory: the restatement must round every a*b+c twice,
  exactly as the reference source is written (gcc on aarch64 contracts by default).
* ``build_ref()`` compiles the reference itself, from the read-only reference tree, into
  oracle/_ref/libref.so (x86 build host only; the tree does not exist elsewhere):
    - src/reconstruction_backend.cpp (CPU path + dispatcher, TSDFMC_HAVE_CUDA=1),
    - src/cuda_block_allocator.cu, src/cuda_tsdf_integrator.cu, src/cuda_mesh_extractor.cu
      compiled as host C++ under the CUDA emulation prelude in oracle/ref_emu/ (kernel launches
      ``k<<<g, b>>>(...)`` rewritten to ``vh_emu_launch(k, g, b, ...)`` on the fly),
  each followed in the same translation unit by a small C driver (oracle/ref_emu/driver_*.inc)
  so that internal functions are reachable.  The sources are streamed to g++ through stdin: no
  copy of the reference is written anywhere.

usage: python oracle/build.py [--ref]
"""
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
# the reference tree (read-only): VH_REFERENCE_ROOT, else the build container's mount point
REFERENCE = os.environ.get("VH_REFERENCE_ROOT", "/root/reference")
ORACLE_SO = os.path.join(HERE, "liboracle.so")
ORACLE64_SO = os.path.join(HERE, "liboracle64.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libref.so")

# no contraction, no fast-math; O2 like the reference's own CMake build (CMakeLists.txt:124-129)
FP_FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC"]


def _run(cmd, stdin_text=None):
    res = subprocess.run(cmd, input=stdin_text, text=True, capture_output=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), res.stdout, res.stderr))
    return res


def build_oracle(force=False):
    """oracle/liboracle.so (float arithmetic: the restatement) and oracle/liboracle64.so (the same source with
    -DVO_FP64: the FP64 transcription), compiled in parallel."""
    src = [os.path.join(HERE, "vh_oracle.c")]
    deps = src + [os.path.join(HERE, "vh_oracle.h"),
                  os.path.join(REPO, "voxelhashmt_gb300", "csrc", "vh_mc_tables.h")]
    newest = max(os.path.getmtime(d) for d in deps)
    jobs = []
    for so, defs in ((ORACLE_SO, []), (ORACLE64_SO, ["-DVO_FP64"])):
        if force or not os.path.exists(so) or os.path.getmtime(so) < newest:
            jobs.append((so, ["gcc", "-std=c11", *FP_FLAGS, *defs, "-shared", "-I",
                              os.path.join(REPO, "voxelhashmt_gb300", "csrc"), *src, "-o", so + ".tmp", "-lpthread",
                              "-lm"]))
    with ThreadPoolExecutor(max_workers=2) as ex:
        list(ex.map(lambda j: _run(j[1]), jobs))
    for so, _ in jobs:
        os.replace(so + ".tmp", so)
    return ORACLE_SO


def reference_available():
    return os.path.exists(os.path.join(REFERENCE, "src", "cuda_tsdf_integrator.cu"))


_PRELUDE = """
#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <unordered_set>
#include <vector>
#define private public
#include "tsdfmc/voxel_hash_tsdf.h"
#include "tsdfmc/reconstruction_backend.h"
#undef private
"""

_UNITS = [
    # (reference source, driver, emulated CUDA)
    ("src/reconstruction_backend.cpp", "driver_backend.inc", False),
    ("src/cuda_block_allocator.cu", "driver_allocator.inc", True),
    ("src/cuda_tsdf_integrator.cu", "driver_integrator.inc", True),
    ("src/cuda_mesh_extractor.cu", "driver_mesh.inc", True),
]


def _rewrite_launches(text):
    def repl(m):
        fn = "vh_emu_launch_sync" if m.group(1) == "compactifyActiveBlockHashKernel" else "vh_emu_launch"
        return "%s(%s, %s, %s, " % (fn, m.group(1), m.group(2).strip(), m.group(3).strip())
    out, n = re.subn(r"(\w+)<<<([^,>]+),\s*([^>]+)>>>\(", repl, text)
    return out, n


def _compile_unit(rel, driver, emulated, obj):
    path = os.path.join(REFERENCE, rel)
    text = open(path).read()
    if emulated:
        text, n = _rewrite_launches(text)
        if n == 0:
            raise RuntimeError("no kernel launches found in %s" % rel)
    prelude = ('#include "cuda_runtime.h"\n' if emulated else "") + _PRELUDE
    unit = (prelude + '#line 1 "%s"\n' % rel + text + '\n#line 1 "%s"\n' % driver +
            open(os.path.join(HERE, "ref_emu", driver)).read())
    cmd = ["g++", "-std=c++17", *FP_FLAGS, "-w", "-DTSDFMC_HAVE_CUDA=1",
           "-I", os.path.join(HERE, "ref_emu"), "-I", os.path.join(REFERENCE, "include"),
           "-iquote", os.path.join(REFERENCE, "src"), "-x", "c++", "-c", "-", "-o", obj]
    _run(cmd, unit)


def build_ref(force=False):
    if not reference_available():
        sys.stderr.write("reference not present at %s (set VH_REFERENCE_ROOT); oracle/_ref not built\n" % REFERENCE)
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    inputs = [os.path.join(REFERENCE, u[0]) for u in _UNITS]
    inputs += [os.path.join(HERE, "ref_emu", f) for f in os.listdir(os.path.join(HERE, "ref_emu"))]
    inputs.append(os.path.abspath(__file__))
    if not force and os.path.exists(REF_SO) and \
            os.path.getmtime(REF_SO) >= max(os.path.getmtime(p) for p in inputs):
        return REF_SO
    objs = []
    jobs = []
    with ThreadPoolExecutor(max_workers=5) as ex:
        for rel, driver, emulated in _UNITS:
            obj = os.path.join(REF_DIR, os.path.basename(rel) + ".o")
            objs.append(obj)
            jobs.append(ex.submit(_compile_unit, rel, driver, emulated, obj))
        rt = os.path.join(REF_DIR, "emu_runtime.o")
        objs.append(rt)
        jobs.append(ex.submit(_run, ["g++", "-std=c++17", *FP_FLAGS, "-I", os.path.join(HERE, "ref_emu"), "-c",
                                     os.path.join(HERE, "ref_emu", "emu_runtime.cpp"), "-o", rt]))
        for j in jobs:
            j.result()
    _run(["g++", "-shared", "-o", REF_SO + ".tmp", *objs, "-lm"])
    os.replace(REF_SO + ".tmp", REF_SO)
    for o in objs:
        os.remove(o)
    return REF_SO


REF_DATASET = os.path.join(REF_DIR, "ref_dataset_driver")


def build_ref_dataset(force=False):
    """oracle/ref_dataset_driver.cpp against the reference's include/tsdfmc/dataset_io.h (read in place)."""
    if not reference_available():
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    src = os.path.join(HERE, "ref_dataset_driver.cpp")
    inputs = [src, os.path.join(REFERENCE, "include", "tsdfmc", "dataset_io.h"),
              os.path.join(REFERENCE, "include", "tsdfmc", "math_types.h"), os.path.abspath(__file__)]
    if not force and os.path.exists(REF_DATASET) and \
            os.path.getmtime(REF_DATASET) >= max(os.path.getmtime(p) for p in inputs):
        return REF_DATASET
    _run(["g++", "-std=c++17", "-O2", *FP_FLAGS, "-I", os.path.join(REFERENCE, "include"), src, "-o",
          REF_DATASET + ".tmp"])
    os.replace(REF_DATASET + ".tmp", REF_DATASET)
    return REF_DATASET


if __name__ == "__main__":
    print(build_oracle(force=True))
    if "--ref" in sys.argv:
        print(build_ref(force=True))
        print(build_ref_dataset(force=True))
