"""CPU tests of the C ABI: the library builds for sm_103a, loads, exports
every symbol include/ggks.h declares, and rejects invalid arguments before
touching the device (no compute call runs without a GPU)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "ggks.h")


@pytest.fixture(scope="module")
def lib():
    import ggks_build
    ggks_build.build()
    import ggks
    return ggks.lib()


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ggks_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared_functions()
    for t in ("f32", "f64", "u32"):
        for stem in ("ggks_multiselect_", "ggks_multiselect_host_", "ggks_topk_", "ggks_topk_host_"):
            assert stem + t in names


def test_library_exports_every_declared_symbol(lib):
    import ggks
    names = declared_functions()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(ggks.EXPORTS) | set(names)
    assert lib.ggks_version() == 10000


def test_binary_is_sm103a(lib):
    """The built library's fat binary holds device code for sm_103a only: the
    CUDA toolkit's listing of its embedded ELF images names one per
    translation unit, every one for sm_103a, and no PTX for a JIT to fall
    back on."""
    import shutil
    import subprocess

    import ggks
    tool = shutil.which("cuobjdump") or os.path.join(
        os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "cuobjdump")
    if not os.path.exists(tool):
        pytest.skip("cuobjdump not installed")
    r = subprocess.run([tool, "--list-elf", ggks.LIB_PATH], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    names = re.findall(r"ELF file\s+\d+:\s+(\S+)", r.stdout)
    units = {os.path.basename(p)[:-3] for p in
             __import__("glob").glob(os.path.join(ROOT, "ggks-multiselect_gb300", "csrc", "*.cu"))}
    assert names and all(n.endswith(".sm_103a.cubin") for n in names), names
    assert units <= {n.split(".")[0] for n in names}, (units, names)
    r = subprocess.run([tool, "--list-ptx", ggks.LIB_PATH], capture_output=True, text=True)
    assert not re.search(r"PTX file\s+\d+:", r.stdout + r.stderr), r.stdout


def test_status_strings(lib):
    import ggks
    assert ggks.status_string(0) == "ok"
    assert ggks.status_string(1) == "invalid argument"


@pytest.mark.parametrize("sfx,dt", [("f32", np.float32), ("f64", np.float64), ("u32", np.uint32)])
def test_invalid_arguments_rejected_without_device(lib, sfx, dt):
    import ggks
    f = getattr(lib, "ggks_multiselect_" + sfx)
    out = np.empty(4, dtype=dt)
    k = np.array([1, 2, 3, 4], dtype=np.uint32)
    fake = ctypes.c_void_p(1 << 20)  # never dereferenced: validation fails first
    o = ggks.Opts()
    # null vector, zero n, zero num_k, null k, null out
    assert f(None, 10, k.ctypes.data, 4, out.ctypes.data, ctypes.byref(o)) == ggks.INVALID_ARG
    assert f(fake, 0, k.ctypes.data, 4, out.ctypes.data, ctypes.byref(o)) == ggks.INVALID_ARG
    assert f(fake, 10, k.ctypes.data, 0, out.ctypes.data, ctypes.byref(o)) == ggks.INVALID_ARG
    assert f(fake, 10, None, 4, out.ctypes.data, ctypes.byref(o)) == ggks.INVALID_ARG
    assert f(fake, 10, k.ctypes.data, 4, None, ctypes.byref(o)) == ggks.INVALID_ARG
    # k outside [1, n] (generateKUniformRandom can emit k = 0)
    bad = np.array([0, 1, 2, 3], dtype=np.uint32)
    assert f(fake, 10, bad.ctypes.data, 4, out.ctypes.data, ctypes.byref(o)) == ggks.INVALID_ARG
    bad = np.array([1, 2, 3, 11], dtype=np.uint32)
    assert f(fake, 10, bad.ctypes.data, 4, out.ctypes.data, ctypes.byref(o)) == ggks.INVALID_ARG
    # n beyond 2^32 - 1
    assert f(fake, 1 << 32, k.ctypes.data, 4, out.ctypes.data, ctypes.byref(o)) == ggks.INVALID_ARG
    # misaligned device pointer
    if dt().itemsize > 1:
        mis = ctypes.c_void_p((1 << 20) + 1)
        assert f(mis, 10, k.ctypes.data, 4, out.ctypes.data, ctypes.byref(o)) == ggks.INVALID_ARG
    g = getattr(lib, "ggks_topk_" + sfx)
    assert g(fake, 10, 11, out.ctypes.data, ctypes.byref(o)) == ggks.INVALID_ARG
    assert g(fake, 10, 0, out.ctypes.data, ctypes.byref(o)) == ggks.INVALID_ARG
    assert g(None, 10, 3, out.ctypes.data, ctypes.byref(o)) == ggks.INVALID_ARG


def test_cpp_reference_mirror_header_compiles(lib, tmp_path):
    """The C++ mirror of the reference interface compiles against the C ABI
    (link only: nothing runs)."""
    import subprocess
    src = tmp_path / "mirror.cpp"
    src.write_text(
        '#include "ggks_bucket_multiselect.hpp"\n'
        "int main(int argc, char** argv) {\n"
        "  if (argc < 100) return 0;\n"
        "  float* d = nullptr; unsigned k[2] = {1, 2}; float out[2];\n"
        "  BucketMultiselect::bucketMultiselectWrapper(d, 10, k, 2, out, 152, 1024);\n"
        "  results_t<float>* r = timeBucketMultiselect(out, 2u, k, 2u);\n"
        "  results_t<float>* t = timeBucketTopkselect(out, 2u, 1u);\n"
        "  float* tk = randomizedTopkSelectWrapper(d, 10, 2);\n"
        "  float s1 = BucketSelect::bucketSelectWrapper(d, 10, 3, 152, 1024);\n"
        "  double* dd = nullptr; unsigned int* du = nullptr;\n"
        "  double s2 = RandomizedBucketSelect::randomizedBucketSelectWrapper(dd, 10, 3, 0, 0);\n"
        "  unsigned int s3 = BucketSelect::bucketSelectWrapper(du, 10, 3, 0, 0);\n"
        "  (void)s1; (void)s2; (void)s3;\n"
        "  free(tk); freeResults(r); freeResults(t);\n"
        "  return 0;\n}\n")
    import ggks
    exe = tmp_path / "mirror"
    r = subprocess.run(["g++", "-std=c++17", "-O1", str(src), "-I", os.path.join(ROOT, "include"),
                        ggks.LIB_PATH, "-o", str(exe), "-Wl,-rpath," + os.path.dirname(ggks.LIB_PATH)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("sfx,dt", [("f32", np.float32), ("f64", np.float64), ("u32", np.uint32)])
def test_batch_invalid_arguments_rejected_without_device(lib, sfx, dt):
    """The batched entry points validate every problem before touching a
    device."""
    import ggks
    f = getattr(lib, "ggks_multiselect_batch_" + sfx)
    t = getattr(lib, "ggks_topk_batch_" + sfx)
    o = ggks.Opts()
    fake = 4096  # never dereferenced: validation fails first
    ptrs = np.array([fake, fake], dtype=np.uint64)
    ns = np.array([10, 20], dtype=np.uint64)
    off = np.array([0, 2, 3], dtype=np.uint32)
    ks = np.array([1, 10, 20], dtype=np.uint32)
    out = np.zeros(3, dtype=dt)

    def call(p=ptrs, n=ns, o_=off, k=ks, num=2):
        return f(p.ctypes.data if p is not None else None, n.ctypes.data, num,
                 o_.ctypes.data if o_ is not None else None,
                 k.ctypes.data if k is not None else None, out.ctypes.data, ctypes.byref(o))

    assert call(num=0) == ggks.INVALID_ARG
    assert call(p=None) == ggks.INVALID_ARG
    assert call(o_=None) == ggks.INVALID_ARG
    assert call(k=None) == ggks.INVALID_ARG
    assert call(o_=np.array([1, 2, 3], dtype=np.uint32)) == ggks.INVALID_ARG   # k_offsets[0] != 0
    assert call(o_=np.array([0, 3, 2], dtype=np.uint32)) == ggks.INVALID_ARG   # decreasing
    assert call(k=np.array([0, 10, 20], dtype=np.uint32)) == ggks.INVALID_ARG  # k = 0
    assert call(k=np.array([1, 11, 20], dtype=np.uint32)) == ggks.INVALID_ARG  # k > n
    assert call(n=np.array([10, 0], dtype=np.uint64)) == ggks.INVALID_ARG      # n = 0 with k's
    assert call(p=np.array([fake, 0], dtype=np.uint64)) == ggks.INVALID_ARG    # null vector
    mis = np.array([fake + 1, fake], dtype=np.uint64)
    assert call(p=mis) == ggks.INVALID_ARG                                     # misaligned
    # no outputs at all: nothing to do
    assert call(o_=np.array([0, 0, 0], dtype=np.uint32)) == ggks.OK
    K = np.array([11, 3], dtype=np.uint32)                                    # K > n
    assert t(ptrs.ctypes.data, ns.ctypes.data, 2, K.ctypes.data, out.ctypes.data,
             ctypes.byref(o)) == ggks.INVALID_ARG
    assert t(ptrs.ctypes.data, ns.ctypes.data, 2, None, out.ctypes.data,
             ctypes.byref(o)) == ggks.INVALID_ARG


@pytest.mark.parametrize("sfx,dt", [("f32", np.float32), ("f64", np.float64), ("u32", np.uint32)])
def test_select_invalid_arguments_rejected_without_device(lib, sfx, dt):
    """Single-k select: null vector or output, n = 0, k outside [1, n]."""
    import ggks
    f = getattr(lib, "ggks_select_" + sfx)
    o = ggks.Opts()
    out = np.zeros(1, dtype=dt)
    fake = 4096
    assert f(None, 10, 1, out.ctypes.data, ctypes.byref(o)) == ggks.INVALID_ARG
    assert f(fake, 10, 1, None, ctypes.byref(o)) == ggks.INVALID_ARG
    assert f(fake, 0, 1, out.ctypes.data, ctypes.byref(o)) == ggks.INVALID_ARG
    assert f(fake, 10, 0, out.ctypes.data, ctypes.byref(o)) == ggks.INVALID_ARG
    assert f(fake, 10, 11, out.ctypes.data, ctypes.byref(o)) == ggks.INVALID_ARG


def test_python_structs_match_the_header(tmp_path):
    """The ctypes mirrors in ggks.py have the sizes and field offsets of the
    structs include/ggks.h declares (a C program compiled against the header
    prints them; nothing is called)."""
    import subprocess

    import ggks
    pairs = [("ggks_opts", ggks.Opts), ("ggks_stats", ggks.Stats),
             ("ggks_server_config", ggks.ServerConfig), ("ggks_request", ggks.Request),
             ("ggks_server_stats", ggks.ServerStats)]
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "ggks.h"', "int main(void) {"]
    for cname, cls in pairs:
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c11", str(src), "-I", os.path.join(ROOT, "include"), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n"):
        if line:
            name, field, val = line.split()
            got[(name, field)] = int(val)
    for cname, cls in pairs:
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)


def test_python_flags_match_the_header():
    """The option flags and status codes of ggks.py carry the values that
    include/ggks.h defines."""
    import re

    import ggks
    text = open(os.path.join(ROOT, "include", "ggks.h")).read()
    defs = dict(re.findall(r"#define\s+GGKS_FLAG_(\w+)\s+(\d+)u", text))
    assert {"OUT_DEVICE", "AUTOTUNE", "TOPK_PIPELINE", "NO_SMALL"} <= set(defs)
    for name, val in defs.items():
        assert getattr(ggks, "FLAG_" + name) == int(val), name


def test_rank_windows_host_logic(tmp_path):
    """The host's rank windows for speculative compaction (set_windows in the
    pipeline header), built into a host program with nvcc and run without a
    device: one window over all ranks, two split at the widest gap for up to
    64 requests, none when they span more than n / 16 ranks."""
    import shutil
    import subprocess
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    csrc = os.path.join(ROOT, "ggks-multiselect_gb300", "csrc")
    src = tmp_path / "windows.cu"
    src.write_text(r"""
#include <cstdio>
#include "ggks_pipeline.cuh"
using namespace ggks;
static void run(const char *name, const uint32_t *ranks, uint32_t m, uint64_t n) {
  Ctrl c = {};
  Req r[128];
  for (uint32_t i = 0; i < m; ++i) { r[i].rank = ranks[i]; r[i].out = i; }
  set_windows(&c, r, m, n);
  printf("%s %u", name, c.spec_nwin);
  for (uint32_t w = 0; w < c.spec_nwin; ++w)
    printf(" %llu %llu", (unsigned long long)c.spec_lo[w], (unsigned long long)c.spec_hi[w]);
  printf("\n");
}
int main() {
  const uint64_t n = 1 << 20;
  const uint32_t one[] = {5000};
  const uint32_t ends[] = {3, 1, 2, 1048575, 1048570, 0};
  const uint32_t close[] = {700000, 700010, 700005};
  const uint32_t spread[] = {0, 524288, 1048575};
  uint32_t many[100];
  for (int i = 0; i < 100; ++i) many[i] = 900000 + 7 * i;
  run("one", one, 1, n);
  run("ends", ends, 6, n);
  run("close", close, 3, n);
  run("spread", spread, 3, n);
  run("many", many, 100, n);
  return 0;
}
""")
    exe = tmp_path / "windows"
    r = subprocess.run([nvcc, "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                        "-I", csrc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True,
                               check=True).stdout.splitlines():
        name, *vals = line.split()
        out[name] = [int(v) for v in vals]
    assert out["one"] == [1, 5000, 5000]
    assert out["ends"] == [2, 0, 3, 1048570, 1048575]      # split at the widest gap
    assert out["close"] == [2, 700000, 700000, 700005, 700010]  # equal gaps: the first
    assert out["spread"] == [0]                              # spans more than n / 16
    assert out["many"] == [1, 900000, 900000 + 7 * 99]      # > 64 requests: one window
