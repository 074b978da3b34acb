"""Device buffers for GPU tests through the CUDA runtime (ctypes): the tests'
own memory for entry points that take device pointers."""
import ctypes as C

import numpy as np


class DeviceMemory:
    def __init__(self):
        self.rt = None
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                self.rt = C.CDLL(name)
                break
            except OSError:
                continue
        if self.rt is None:
            raise RuntimeError("libcudart not found")
        self.rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        self.rt.cudaFree.argtypes = [C.c_void_p]
        self.rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        self.rt.cudaMemset.argtypes = [C.c_void_p, C.c_int, C.c_size_t]
        self.ptrs = []

    def alloc(self, nbytes, fill=None):
        p = C.c_void_p()
        assert self.rt.cudaMalloc(C.byref(p), nbytes) == 0
        self.ptrs.append(p)
        if fill is not None:
            assert self.rt.cudaMemset(p, fill, nbytes) == 0
        return p

    def upload(self, arr):
        arr = np.ascontiguousarray(arr)
        p = self.alloc(arr.nbytes)
        assert self.rt.cudaMemcpy(p, arr.ctypes.data, arr.nbytes, 1) == 0
        return p

    def download(self, p, shape, dtype=np.float32):
        out = np.zeros(shape, dtype)
        assert self.rt.cudaMemcpy(out.ctypes.data, p, out.nbytes, 2) == 0
        return out

    def close(self):
        for p in self.ptrs:
            self.rt.cudaFree(p)
        self.ptrs = []
