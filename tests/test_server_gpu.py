"""GPU tests of the serving loop (ggks_server_*): requests of mixed sizes,
element types and kinds are admitted under an HBM cap and the device's free
memory and coalesced into batched launches on several lanes; each result must
equal, bit for bit, the single-vector entry point on the same vector and k's
(the result "alone") and the oracle (sort-and-choose)."""
import os
import threading

import numpy as np
import pytest

from gpu_util import DeviceArray, assert_same

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ggks
    ggks.lib()
    return ggks


@pytest.fixture(scope="module")
def orc():
    import oracle
    oracle.build()
    return oracle


def _oracle(orc, x, kind, arg):
    thr = os.cpu_count() or 1
    return orc.multiselect(x, arg, thr) if kind == "ms" else orc.topk(x, arg, thr)


def _mixed_requests(seed, count, max_log2=22):
    """(dtype, dist, n, kind, ks or K) tuples: float32 / uint32 / float64 in
    ratio 6:3:1, 70% multiselect with 8-1024 k's, 30% top-k."""
    import ggks_problems as gp
    r = np.random.default_rng(seed)
    dists = {"f32": ("uniform", "normal", "cauchy", "uint_valued"),
             "u32": ("uniform", "uniform16", "sorted"),
             "f64": ("uniform", "normal", "cauchy", "uint_valued")}
    out = []
    for i in range(count):
        dt = ("f32",) * 6 + ("u32",) * 3 + ("f64",)
        dt = dt[int(r.integers(0, 10))]
        n = int(2 ** r.uniform(0, max_log2))
        dist = dists[dt][int(r.integers(0, len(dists[dt])))]
        x = gp.generate(dt, dist, n, seed=1000 * seed + i)
        if r.random() < 0.7:
            ks = r.integers(1, n + 1, int(r.integers(8, 1025))).astype(np.uint32)
            out.append((x, "ms", ks))
        else:
            out.append((x, "topk", int(r.integers(1, min(n, 4096) + 1))))
    return out


def _alone(g, d, x, kind, arg):
    if kind == "ms":
        return g.multiselect_ptr(d.ptr, x.size, x.dtype, arg)
    return g.topk_ptr(d.ptr, x.size, x.dtype, arg)


def test_server_results_same_alone_and_in_mix(g, orc):
    reqs = _mixed_requests(1, 80)
    devs = [DeviceArray(x) for x, _, _ in reqs]
    alone = [_alone(g, d, x, kind, arg) for d, (x, kind, arg) in zip(devs, reqs)]
    for i, (x, kind, arg) in enumerate(reqs):
        assert_same(alone[i], _oracle(orc, x, kind, arg), f"alone vs oracle {i}")
    srv = g.Server(0, hbm_cap_bytes=64 << 30)
    tickets = []
    for d, (x, kind, arg) in zip(devs, reqs):
        if kind == "ms":
            tickets.append(srv.submit(d.ptr, x.size, x.dtype, k=arg))
        else:
            tickets.append(srv.submit(d.ptr, x.size, x.dtype, K=arg))
    for i, t in enumerate(tickets):
        got, lat = srv.wait(t)
        assert lat >= 0.0
        assert_same(got, alone[i], f"request {i} ({reqs[i][0].dtype}, {reqs[i][1]}, "
                                   f"n={reqs[i][0].size})")
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs)
    assert st["batches"] < len(reqs)  # requests were coalesced
    assert st["max_batch_seen"] > 1


def test_server_host_vectors_under_a_small_cap(g, orc):
    """Host vectors are uploaded at admission; the admitted bytes never exceed
    the cap, so requests wait for earlier ones to finish."""
    import ggks_problems as gp
    cap = 48 << 20
    xs = [gp.generate("f32", "normal", (1 << 22) - i * 1000, seed=i) for i in range(10)]
    ks = [gp.k_distinct(x.size, 100, i) for i, x in enumerate(xs)]
    srv = g.Server(0, hbm_cap_bytes=cap)
    tickets = [srv.submit(x.ctypes.data, x.size, x.dtype, k=k, host=True) for x, k in zip(xs, ks)]
    res = [srv.wait(t)[0] for t in tickets]
    st = srv.stats()
    srv.close()
    for i, (x, k) in enumerate(zip(xs, ks)):
        d = DeviceArray(x)
        assert_same(res[i], g.multiselect_ptr(d.ptr, x.size, x.dtype, k), f"host request {i}")
        assert_same(res[i], orc.multiselect(x, k, 8), f"host request {i} vs oracle")
    assert st["uploads"] == len(xs)
    assert 0 < st["peak_bytes"] <= cap
    assert st["in_flight_bytes"] == 0


def test_server_concurrent_submitters(g, orc):
    reqs = _mixed_requests(2, 64, max_log2=20)
    devs = [DeviceArray(x) for x, _, _ in reqs]
    alone = [_oracle(orc, x, kind, arg) for x, kind, arg in reqs]
    srv = g.Server(0, hbm_cap_bytes=8 << 30, max_batch=16)
    results = [None] * len(reqs)

    def client(idx):
        for i in idx:
            x, kind, arg = reqs[i]
            t = srv.submit(devs[i].ptr, x.size, x.dtype,
                           k=arg if kind == "ms" else None, K=arg if kind == "topk" else None)
            results[i] = srv.wait(t)[0]

    threads = [threading.Thread(target=client, args=(range(c, len(reqs), 4),)) for c in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    st = srv.stats()
    srv.close()
    for i in range(len(reqs)):
        assert_same(results[i], alone[i], f"concurrent request {i}")
    assert st["completed"] == len(reqs)
    assert st["max_batch_seen"] <= 16


def test_server_lanes_overlap(g, orc):
    """With two lanes and small batches under load, one lane's kernel runs
    while the other lane plans, uploads and queues its own launch behind it
    on the device: the server counts launches queued behind a kernel still in
    flight, and the device time covered by batched kernels fits inside their
    span.  Every result equals the oracle's."""
    reqs = _mixed_requests(5, 160, max_log2=21)
    devs = [DeviceArray(x) for x, _, _ in reqs]
    srv = g.Server(0, hbm_cap_bytes=16 << 30, max_batch=6, lanes=2)
    tickets = [srv.submit(d.ptr, x.size, x.dtype, k=arg if kind == "ms" else None,
                          K=arg if kind == "topk" else None)
               for d, (x, kind, arg) in zip(devs, reqs)]
    res = [srv.wait(t)[0] for t in tickets]
    st = srv.stats()
    srv.close()
    for i, (x, kind, arg) in enumerate(reqs):
        assert_same(res[i], _oracle(orc, x, kind, arg), f"lanes request {i}")
    assert st["completed"] == len(reqs)
    assert st["batches"] >= len(reqs) // 6
    assert st["concurrent_launches"] > 0
    assert 0 < st["device_busy_ms"] <= st["device_span_ms"] + 1e-3


def test_server_admission_by_free_device_memory(g, orc):
    """The admission budget follows the device's free memory: with a reserve
    that leaves only 512 MB of it to the server, 16 host-vector requests of
    64 MB wait for earlier ones to finish (hbm_waits) although the
    cap would admit them all, and every result is exact.  The vectors are in
    pinned host memory, so an upload does not hold the admission thread: it
    reaches the eighth request (7 x 68 MB charged) while the first is still
    uploading, and that one must wait.  A request that could never fit -- the
    reserve larger than the free memory, nothing admitted -- fails with
    GGKS_OOM instead of waiting forever."""
    import torch

    import ggks_problems as gp
    xs = []
    for i in range(16):
        h = torch.empty(1 << 24, dtype=torch.float32, pin_memory=True).numpy()
        h[:] = gp.generate("f32", "uniform", 1 << 24, seed=40 + i)
        xs.append(h)
    ks = [gp.k_distinct(x.size, 64, i) for i, x in enumerate(xs)]
    torch.cuda.synchronize()
    free = torch.cuda.mem_get_info()[0]
    srv = g.Server(0, hbm_cap_bytes=64 << 30, hbm_reserve_bytes=free - (512 << 20))
    tickets = [srv.submit(x.ctypes.data, x.size, x.dtype, k=k, host=True) for x, k in zip(xs, ks)]
    res = [srv.wait(t)[0] for t in tickets]
    st = srv.stats()
    srv.close()
    for i, (x, k) in enumerate(zip(xs, ks)):
        assert_same(res[i], orc.multiselect(x, k, 8), f"budget request {i}")
    assert st["hbm_waits"] > 0
    # held back well below the 1 GB the requests add up to (the budget is
    # taken from the free memory when admitting, which moves a little as the
    # lanes' workspaces and the upload pool grow)
    assert st["peak_bytes"] <= (512 + 128) << 20
    assert 0 < st["admit_budget_bytes"] < 64 << 30
    assert st["in_flight_bytes"] == 0
    torch.cuda.synchronize()
    free = torch.cuda.mem_get_info()[0]
    srv = g.Server(0, hbm_cap_bytes=64 << 30, hbm_reserve_bytes=free + (1 << 30))
    t = srv.submit(xs[0].ctypes.data, xs[0].size, xs[0].dtype, k=ks[0], host=True)
    with pytest.raises(g.GgksError) as e:
        srv.wait(t)
    assert e.value.status == g.OOM
    srv.close()


def test_server_rejections(g):
    import ggks_problems as gp
    x = gp.generate("f32", "uniform", 1 << 20, seed=1)
    d = DeviceArray(x)
    srv = g.Server(0, hbm_cap_bytes=1 << 20)
    with pytest.raises(g.GgksError) as e:  # the request alone exceeds the cap
        srv.submit(x.ctypes.data, x.size, x.dtype, k=[1, 2], host=True)
    assert e.value.status == g.OOM
    with pytest.raises(g.GgksError) as e:  # k outside [1, n]
        srv.submit(d.ptr, x.size, x.dtype, k=[0])
    assert e.value.status == g.INVALID_ARG
    with pytest.raises(g.GgksError) as e:  # K > n
        srv.submit(d.ptr, 10, x.dtype, K=11)
    assert e.value.status == g.INVALID_ARG
    # a valid request still runs
    small = x[:1000].copy()
    ds = DeviceArray(small)
    t = srv.submit(ds.ptr, small.size, small.dtype, k=[1, 500, 1000])
    got, _ = srv.wait(t)
    assert_same(got, g.multiselect_ptr(ds.ptr, small.size, small.dtype, [1, 500, 1000]), "small")
    srv.close()
