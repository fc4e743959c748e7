"""ctypes binding of libgbsdf.so, the C ABI declared in include/gbsdf.h.

The library is built in-tree by ``neuralangelo_gb300.build``.  There is no
fallback: if the library is missing or a call fails, a RuntimeError says why.
"""
import ctypes
import os

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbsdf.so")
MAX_LEVELS = 32
F32, F16 = 0, 1

c_i32, c_i64, c_f32, c_vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.c_void_p


class GridStruct(ctypes.Structure):
    _fields_ = [("n_levels", c_i32), ("n_features", c_i32), ("log2_hashmap_size", c_i32),
                ("base_resolution", c_i32), ("per_level_scale", c_f32),
                ("scale", c_f32 * MAX_LEVELS), ("resolution", ctypes.c_uint32 * MAX_LEVELS),
                ("size", ctypes.c_uint32 * MAX_LEVELS), ("hashed", ctypes.c_uint32 * MAX_LEVELS),
                ("offset", ctypes.c_uint64 * (MAX_LEVELS + 1))]


# name -> argtypes (restype is int for every entry point except noted)
_SIGS = {
    "gbsdf_version": [],
    "gbsdf_device_count": [],
    "gbsdf_grid_init": [ctypes.POINTER(GridStruct), c_i32, c_i32, c_i32, c_i32, c_f32],
    "gbsdf_hashgrid_fwd": [ctypes.POINTER(GridStruct), c_i32, c_vp, c_i64, c_vp, c_i32, c_vp, c_i32, c_vp],
    "gbsdf_hashgrid_bwd": [ctypes.POINTER(GridStruct), c_i32, c_vp, c_i64, c_vp, c_vp, c_vp],
    "gbsdf_hashgrid_indices": [ctypes.POINTER(GridStruct), c_i32, c_vp, c_i64, c_vp, c_vp],
    "gbsdf_neus_alpha_fwd": [c_i64, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_f32, c_f32, c_vp, c_vp],
    "gbsdf_neus_alpha_bwd": [c_i64, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_f32, c_f32, c_vp, c_vp, c_vp,
                             c_vp, c_vp],
    "gbsdf_composite_weights_fwd": [c_i64, c_i64, c_vp, c_vp, c_vp],
    "gbsdf_composite_weights_bwd": [c_i64, c_i64, c_vp, c_vp, c_vp, c_vp],
    "gbsdf_dense": [c_i64, c_i32, c_i32, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_i32, c_i32,
                    c_i32, c_f32, c_vp, c_vp],
}

_lib = None


def load():
    """Load (once) and return the ctypes library; raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libgbsdf.so not found at {LIB_PATH}; build it with "
                           "`python -m neuralangelo_gb300.build` (nvcc, sm_103a)")
    lib = ctypes.CDLL(LIB_PATH)
    lib.gbsdf_last_error.restype = ctypes.c_char_p
    lib.gbsdf_last_error.argtypes = []
    for name, args in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = c_i32
    _lib = lib
    return lib


def register(name, argtypes):
    """Declare an additional entry point (used by modules that add kernels)."""
    _SIGS[name] = argtypes
    if _lib is not None:
        fn = getattr(_lib, name)
        fn.argtypes = argtypes
        fn.restype = c_i32


class KernelTimer:
    """Records a CUDA event pair around every C-ABI call on the current stream
    (the stream the kernels are launched on) while enabled; used by bench.py to
    time the dominant kernel inside the timed region and to count launches."""

    def __init__(self):
        self.enabled = False
        self.events = {}
        self.bytes = {}

    def reset(self):
        self.events = {}
        self.bytes = {}

    def count_bytes(self, name, nbytes):
        """Algorithmic bytes one call of `name` must move (summed per name while enabled)."""
        if self.enabled:
            self.bytes[name] = self.bytes.get(name, 0) + int(nbytes)

    def summary(self):
        """{name: (calls, total_ms)}; call after a device synchronize."""
        out = {}
        for name, evs in self.events.items():
            out[name] = (len(evs), sum(a.elapsed_time(b) for a, b in evs))
        return out


TIMER = KernelTimer()

# kernels launched by one call of each entry point (for launch counting)
LAUNCHES_PER_CALL = {}


def call(name, *args):
    lib = load()
    fn = getattr(lib, name)
    if TIMER.enabled:
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        st = fn(*args)
        b.record()
        TIMER.events.setdefault(name, []).append((a, b))
    else:
        st = fn(*args)
    if st != 0:
        msg = lib.gbsdf_last_error().decode(errors="replace")
        raise RuntimeError(f"{name} failed (status {st}): {msg}")


def ptr(t):
    """Raw device/host pointer of a tensor (None -> NULL)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_ptr(device=None):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def require_cuda(*tensors):
    for t in tensors:
        if t is not None and not t.is_cuda:
            raise RuntimeError("gbsdf kernels take CUDA tensors; got a tensor on " + str(t.device))
