"""The C++ drop-in run on the GPU: a program written against the reference's
host interface (compareMultiselect.hpp:46-224 calls these names through
multiselectTimingFunctions.cu:113 and :222) is compiled against
include/ggks_bucket_multiselect.hpp alone, linked with the library, and run on
device data of every element type; every answer it writes is compared bit for
bit with the oracle (sort-and-choose)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from gpu_util import assert_same

pytestmark = pytest.mark.gpu

HARNESS = os.path.join(ROOT, "tests", "dropin", "dropin_harness.cpp")


def _cuda_home():
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ggks
    ggks.lib()
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = tmp_path_factory.mktemp("dropin") / "dropin_harness"
    cuda = _cuda_home()
    cmd = [cxx, "-std=c++17", "-O2", HARNESS, "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), ggks.LIB_PATH,
           "-L", os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath," + os.path.dirname(ggks.LIB_PATH),
           "-Wl,-rpath," + os.path.join(cuda, "lib64"), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(out)


@pytest.mark.parametrize("n,numk,K", [(1 << 20, 101, 1024), (300_007, 1001, 32),
                                      (4099, 50, 4099)])
def test_cpp_dropin_calls_match_oracle(exe, tmp_path, n, numk, K):
    import oracle

    import ggks_problems as gp
    oracle.build()
    vecs = {"f32": gp.generate("f32", "normal", n, 1), "f64": gp.generate("f64", "cauchy", n, 2),
            "u32": gp.generate("u32", "uniform16", n, 3)}
    k = gp.k_distinct(n, numk, 4)
    for t, v in vecs.items():
        v.tofile(tmp_path / f"vec_{t}.bin")
    k.tofile(tmp_path / "k.bin")
    r = subprocess.run([exe, str(tmp_path), str(n), str(k.size), str(K)], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    for t, v in vecs.items():
        want_ms = oracle.multiselect(v, k, 8)
        want_tk = oracle.topk(v, K, 8)
        rd = lambda nm, cnt: np.fromfile(tmp_path / f"{nm}_{t}.bin", dtype=v.dtype, count=cnt)
        assert_same(rd("ms", k.size), want_ms, f"bucketMultiselectWrapper {t}")
        assert_same(rd("tms", k.size), want_ms, f"timeBucketMultiselect {t}")
        assert_same(rd("ttk", K), want_tk, f"timeBucketTopkselect {t}")
        assert_same(rd("rtk", K), want_tk, f"randomizedTopkSelectWrapper {t}")
        want_sel = oracle.multiselect(v, k[np.arange(8) % k.size])
        assert_same(rd("sel", 8), want_sel, f"bucketSelectWrapper {t}")
        assert_same(rd("rsel", 8), want_sel, f"randomizedBucketSelectWrapper {t}")
