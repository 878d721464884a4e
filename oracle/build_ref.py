"""Builds oracle/_ref/libggks_ref.so: the reference's own bucket multiselect
path compiled for the host CPU (test infrastructure, used only to make the
golden fixtures that pin the oracle).

Sources, read in place from the reference tree (GGKS_REFERENCE, default
/root/reference), never copied into this repository:
  bucketMultiselect.cu            (bucketMultiselectWrapper, phaseOne, kernels)
  multiselectTimingFunctions.cu   (timeBucketMultiselect, timeBucketTopkselect,
                                   timeSortAndChooseMultiselect/-Topkselect)
The translation unit is assembled in memory and piped to g++:
  1. ref_host/cuda_host_emu.h -- the host stand-in for the CUDA runtime;
  2. each source after two mechanical rewrites that C++ needs and that change
     no statement of the algorithm:
       `kernel<<<grid, block[, smem]>>>(args);`
           -> `::ggks_host_emu::launch(dim3(grid), dim3(block), smem,
                                       [&] { kernel(args); });`
       `extern __shared__ T name[];`
           -> `T *name = (T *) ::ggks_host_emu::dynamic_shared();`
     (`#line` directives keep diagnostics on the reference's own lines);
  3. ref_host/ref_entry.inc -- C entry points onto the timing adapters.
Thrust runs on its CPP back end; libcudart is not linked.

The output is an x86-64 host library: it runs where it is built, and the GPU
tests use only the committed fixtures it produced (tests/golden/ref_*.npz).
"""
import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT_DIR = HERE / "_ref"
OUT = OUT_DIR / "libggks_ref.so"
SOURCES = ("bucketMultiselect.cu", "multiselectTimingFunctions.cu")
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def reference_root():
    return Path(os.environ.get("GGKS_REFERENCE", "/root/reference"))


def _match_back(src, end, open_ch, close_ch):
    """Index of the `open_ch` that balances the `close_ch` at src[end]."""
    depth = 0
    i = end
    while i >= 0:
        if src[i] == close_ch:
            depth += 1
        elif src[i] == open_ch:
            depth -= 1
            if depth == 0:
                return i
        i -= 1
    raise ValueError("unbalanced " + close_ch)


def _match_fwd(src, start, open_ch, close_ch):
    depth = 0
    for i in range(start, len(src)):
        if src[i] == open_ch:
            depth += 1
        elif src[i] == close_ch:
            depth -= 1
            if depth == 0:
                return i
    raise ValueError("unbalanced " + open_ch)


def _split_top(s):
    parts, depth, cur = [], 0, []
    for ch in s:
        if ch in "([{<":
            depth += 1
        elif ch in ")]}>":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur))
    return [p.strip() for p in parts]


def rewrite_launches(src):
    out = []
    pos = 0
    while True:
        i = src.find("<<<", pos)
        if i < 0:
            out.append(src[pos:])
            return "".join(out)
        # callee: identifier, optionally with template arguments
        j = i - 1
        while src[j].isspace():
            j -= 1
        if src[j] == ">":
            j = _match_back(src, j, "<", ">") - 1
        k = j
        while k >= 0 and (src[k].isalnum() or src[k] in "_:"):
            k -= 1
        callee_start = k + 1
        cfg_end = src.find(">>>", i)
        cfg = _split_top(src[i + 3:cfg_end])
        a = cfg_end + 3
        while src[a].isspace():
            a += 1
        assert src[a] == "(", "launch without arguments"
        b = _match_fwd(src, a, "(", ")")
        semi = src.find(";", b)
        callee = src[callee_start:i].strip()
        grid, block = cfg[0], cfg[1]
        smem = cfg[2] if len(cfg) > 2 else "0"
        original = src[callee_start:semi + 1]
        call = (f"::ggks_host_emu::launch(dim3({grid}), dim3({block}), "
                f"(size_t)({smem}), [&] {{ {callee}{src[a:b + 1]}; }});")
        # keep the line count so #line stays exact
        call = call.replace("\n", " ") + "\n" * original.count("\n")
        out.append(src[pos:callee_start])
        out.append(call)
        pos = semi + 1


_DYN_SHARED = re.compile(r"extern\s+__shared__\s+(\w+)\s+(\w+)\s*\[\s*\]\s*;")


def rewrite_dynamic_shared(src):
    return _DYN_SHARED.sub(
        r"\1 *\2 = (\1 *) ::ggks_host_emu::dynamic_shared();", src)


# The reference compiles these sources inside compareMultiselect.hpp, whose
# includes (compareMultiselect.hpp:8-24) come first; bucketMultiselect.cu relies
# on them (thrust::minmax_element comes from <thrust/extrema.h>).
_HARNESS_INCLUDES = """#include <time.h>
#include <stdio.h>
#include <stdlib.h>
#include <iostream>
#include <fstream>
#include <sys/time.h>
#include <algorithm>
#include <thrust/reduce.h>
#include <thrust/functional.h>
#include <thrust/device_ptr.h>
#include <thrust/scan.h>
#include <thrust/extrema.h>
#include <thrust/pair.h>
#include <thrust/transform_reduce.h>
#include <thrust/random.h>
"""


def translation_unit(ref):
    parts = ['#include "cuda_host_emu.h"\n', _HARNESS_INCLUDES]
    for name in SOURCES:
        text = (ref / name).read_text()
        text = rewrite_dynamic_shared(rewrite_launches(text))
        parts.append(f'#line 1 "{ref / name}"\n')
        parts.append(text)
        parts.append("\n")
    parts.append('#line 1 "ref_entry.inc"\n#include "ref_entry.inc"\n')
    return "".join(parts)


def build(force=False, verbose=False):
    """Compiles the library if the reference tree is present; returns its path
    or None when the reference is absent."""
    ref = reference_root()
    if not all((ref / s).is_file() for s in SOURCES):
        return None
    deps = [ref / s for s in SOURCES] + [HERE / "ref_host" / "cuda_host_emu.h",
                                          HERE / "ref_host" / "ref_entry.inc",
                                          Path(__file__)]
    if (not force and OUT.exists()
            and OUT.stat().st_mtime >= max(p.stat().st_mtime for p in deps)):
        return OUT
    OUT_DIR.mkdir(exist_ok=True)
    tu = translation_unit(ref)
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-w",
           "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP",
           "-I", str(HERE / "ref_host"),
           "-I", str(CUDA / "include" / "cccl"), "-I", str(CUDA / "include"),
           "-x", "c++", "-", "-o", str(OUT)]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, input=tu, text=True, capture_output=True)
    if r.returncode != 0:
        raise RuntimeError("building the reference for the host failed:\n" + r.stderr[-6000:])
    return OUT


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose=True)
    print(p if p else "reference sources not found: nothing built")
