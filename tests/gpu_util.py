"""Helpers for the GPU tests: numpy <-> CUDA tensors bit-for-bit."""
import numpy as np


def to_dev(a: np.ndarray):
    import torch
    a = np.ascontiguousarray(a)
    sig = {1: np.uint8, 4: np.int32, 8: np.int64}[a.dtype.itemsize]
    return torch.from_numpy(a.view(sig)).cuda()


def from_dev(t, dtype) -> np.ndarray:
    return t.cpu().numpy().view(dtype)


def full_dev(n: int, value: int, width: int):
    dt = np.uint32 if width == 4 else np.uint64
    return to_dev(np.full(n, value, dt))


class _DevView:
    """A raw device range as a __cuda_array_interface__ object."""

    def __init__(self, ptr: int, nbytes: int):
        self.__cuda_array_interface__ = {"shape": (nbytes,), "typestr": "|u1", "data": (ptr, False),
                                         "version": 3, "strides": None}


def device_bytes(ptr: int, nbytes: int):
    import torch
    return torch.as_tensor(_DevView(ptr, nbytes), device="cuda")


def bucket_array(m, width: int) -> np.ndarray:
    import torch
    dt = np.uint32 if width == 4 else np.uint64
    ptr, n = m.bucket_data()
    torch.cuda.synchronize()
    return device_bytes(ptr, n * 2 * width).cpu().numpy().view(dt).reshape(n, 2)


def device_mapping(m, width: int):
    """Valid (keys, values) of a libhx map sorted by key, and its buckets."""
    b = bucket_array(m, width)
    e = np.iinfo(b.dtype).max
    sel = (b[:, 0] != e) & (b[:, 0] != e - 1)
    k, v = b[sel, 0], b[sel, 1]
    o = np.argsort(k, kind="stable")
    return k[o], v[o], b
