"""Build the GB300 GGKS library: every csrc/*.cu unit is compiled for sm_103a
in parallel and linked into ggks-multiselect_gb300/libggks_gb300.so (CUDA
runtime linked statically).  No cmake; nvcc only.

    python ggks-multiselect_gb300/ggks_build.py [--verbose-ptxas]
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libggks_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# GGKS_BATCH_CHECKS=1: the batched kernel checks its data-dependent indices
# (a diagnostic build in its own object folder)
CHECKS = os.environ.get("GGKS_BATCH_CHECKS") == "1"
CHECK_FLAGS = ["-DGGKS_BATCH_CHECKS"] if CHECKS else []
# GGKS_BATCH_TIMING=1: the batched kernel reports per-problem cycles of its
# table phase (diagnostic build, own object folder)
if os.environ.get("GGKS_BATCH_TIMING") == "1":
    CHECKS = True
    CHECK_FLAGS.append("-DGGKS_BATCH_TIMING")
# GGKS_SMALL_TIMING=1: the small-vector kernel stamps its phase boundaries
# and the host prints them (diagnostic build, own object folder)
if os.environ.get("GGKS_SMALL_TIMING") == "1":
    CHECKS = True
    CHECK_FLAGS.append("-DGGKS_SMALL_TIMING")
if CHECKS:
    BUILD = os.path.join(HERE, "_build_" + "_".join(f[7:].lower() for f in CHECK_FLAGS))


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _compile(src, ptxas_verbose):
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    deps = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h")) + [src]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj, ""
    cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-c", src, "-o", obj, *CHECK_FLAGS]
    if ptxas_verbose:
        cmd[1:1] = ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(ptxas_verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, ptxas_verbose), srcs))
    objs = [o for o, _ in results]
    logs = "".join(l for _, l in results)
    stamp = os.path.join(HERE, "_build_kind")
    kind = " ".join(CHECK_FLAGS) if CHECKS else "release"
    same_kind = os.path.exists(stamp) and open(stamp).read() == kind
    if not same_kind or not os.path.exists(LIB) or \
            os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs,
               "-Xlinker", "--no-undefined", "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        with open(stamp, "w") as f:
            f.write(kind)
    return LIB, logs


if __name__ == "__main__":
    lib, logs = build(ptxas_verbose="--verbose-ptxas" in sys.argv)
    if logs:
        print(logs)
    print(lib)
