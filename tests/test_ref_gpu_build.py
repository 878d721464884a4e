"""CPU tests of the tooling that runs the reference's own kernels on the GPU
(oracle/ref_gpu.py): where the reference's sources are, its kernels compile
for sm_103a into a cubin that holds every kernel the restated host driver
binds; without the sources an existing cubin is kept and nothing is built;
the driver reports why it cannot run when a part is missing.  Nothing here
needs a GPU: the cubin's kernel names come from ptxas's own report."""
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import ref_gpu  # noqa: E402

# the reference's kernels the host driver binds (ref_gpu_host.cu), as ptxas
# names them
BOUND = ["assignSmartBucket", "copyElements", "copyValuesInChunk", "enlargeIndexAndGetElements",
         "sumCounts", "reindexCounts", "copyInChunk", "ggks_ref_random_vector_f32",
         "ggks_ref_random_vector_f64"]


def _reference_present():
    root = ref_gpu._reference_root()
    return all(os.path.isfile(os.path.join(root, s)) for s in ref_gpu.REF_SOURCES)


@pytest.mark.skipif(not _reference_present(), reason="the reference's sources are not here")
def test_reference_kernels_compile_for_sm103a(tmp_path):
    nvcc = ref_gpu._nvcc()
    root = ref_gpu._reference_root()
    out = tmp_path / "k.cubin"
    cmd = [nvcc, "-cubin", *ref_gpu.ARCH, "-O3", "-std=c++17", "-w", "-Xptxas", "-v", "-I",
           ref_gpu.SRC_DIR,
           f'-DGGKS_REF_BUCKET_MULTISELECT="{os.path.join(root, ref_gpu.REF_SOURCES[0])}"',
           f'-DGGKS_REF_TIMING_FUNCTIONS="{os.path.join(root, ref_gpu.REF_SOURCES[1])}"',
           os.path.join(ref_gpu.SRC_DIR, "ref_kernels.cu"), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert out.read_bytes()[:4] == b"\x7fELF"
    entries = re.findall(r"Compiling entry function '([^']+)' for 'sm_103a'", r.stderr)
    for name in BOUND:
        assert any(name in e for e in entries), name
    # every launch of the reference's 1024-thread blocks fits the register file
    regs = [int(v) for v in re.findall(r"Used (\d+) registers", r.stderr)]
    assert regs and max(regs) <= 64, regs


def test_without_sources_an_existing_cubin_is_kept(tmp_path, monkeypatch):
    monkeypatch.setenv("GGKS_REFERENCE", str(tmp_path / "absent"))
    monkeypatch.setattr(ref_gpu, "CUBIN", str(tmp_path / "ref_kernels.cubin"))
    assert ref_gpu.build_cubin() is None
    (tmp_path / "ref_kernels.cubin").write_bytes(b"\x7fELF")
    assert ref_gpu.build_cubin() == str(tmp_path / "ref_kernels.cubin")


def test_unavailable_names_the_missing_part(tmp_path, monkeypatch):
    monkeypatch.setattr(ref_gpu, "CUBIN", str(tmp_path / "none.cubin"))
    monkeypatch.setattr(ref_gpu, "LIB", str(tmp_path / "none.so"))
    assert "cubin" in ref_gpu.unavailable()
    (tmp_path / "none.cubin").write_bytes(b"\x7fELF")
    assert "host driver" in ref_gpu.unavailable()
    (tmp_path / "none.so").write_bytes(b"")
    assert ref_gpu.unavailable() is None
