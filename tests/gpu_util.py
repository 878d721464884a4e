"""Helpers shared by the GPU tests: device copies of numpy arrays (torch is
used only to own device memory) and bit-exact comparisons."""
import numpy as np


class DeviceArray:
    """A CUDA copy of a numpy array; uint32 data rides in an int32 tensor."""

    def __init__(self, arr, pad_front=0):
        import torch
        arr = np.ascontiguousarray(arr)
        self.dtype = arr.dtype
        self.n = arr.size
        carrier = {np.dtype(np.float32): np.float32, np.dtype(np.float64): np.float64,
                   np.dtype(np.uint32): np.int32}[arr.dtype]
        host = arr.view(carrier)
        if pad_front:
            host = np.concatenate([np.zeros(pad_front, dtype=carrier), host])
        self.t = torch.from_numpy(host).cuda()
        self.ptr = self.t.data_ptr() + pad_front * arr.itemsize


def bits(a):
    a = np.ascontiguousarray(a)
    if a.dtype == np.float32:
        return a.view(np.uint32)
    if a.dtype == np.float64:
        return a.view(np.uint64)
    return a


def assert_same(got, want, what=""):
    g, w = bits(got), bits(want)
    if not np.array_equal(g, w):
        bad = np.nonzero(g != w)[0]
        i = int(bad[0])
        raise AssertionError(f"{what}: {bad.size} of {w.size} differ; first at {i}: "
                             f"got {got[i]!r} want {want[i]!r}")
