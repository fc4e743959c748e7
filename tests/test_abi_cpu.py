"""CPU-side checks of the C ABI: the library loads, exports every symbol the
header declares, validates arguments, and builds the same level table as the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

from neuralangelo_gb300 import _lib
from neuralangelo_gb300.build import build
from oracle import hashgrid as hg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build()
    return _lib.load()


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "gbsdf.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*|size_t|int64_t)\s+(gbsdf_\w+)\s*\(", txt, re.M)))


def test_exports_every_declared_symbol(lib):
    syms = header_symbols()
    assert len(syms) >= 10
    for s in syms:
        assert hasattr(lib, s), s


def test_version_and_error(lib):
    assert lib.gbsdf_version() >= 100
    g = _lib.GridStruct()
    st = lib.gbsdf_grid_init(ctypes.byref(g), 0, 8, 22, 32, ctypes.c_float(1.3))
    assert st == 1
    assert b"n_levels" in lib.gbsdf_last_error()


@pytest.mark.parametrize("cfg", [(16, 8, 22, 32, float(np.exp((np.log(2048) - np.log(32)) / 15))),
                                 (8, 4, 16, 16, 1.5), (8, 4, 10, 16, float(8 ** (1 / 7))),
                                 (6, 2, 10, 8, float(8 ** (1 / 5)))])
def test_grid_init_matches_oracle(lib, cfg):
    from neuralangelo_gb300.encoding import GridLayout
    lay = GridLayout(*cfg)
    ref = hg.level_layout(*cfg)
    np.testing.assert_array_equal(lay.scale, ref['scale'])
    np.testing.assert_array_equal(lay.resolution, ref['resolution'])
    np.testing.assert_array_equal(lay.size, ref['size'])
    np.testing.assert_array_equal(lay.hashed, ref['hashed'])
    np.testing.assert_array_equal(lay.offset, ref['offset'])


def test_null_pointer_rejected_without_gpu(lib):
    g = _lib.GridStruct()
    assert lib.gbsdf_grid_init(ctypes.byref(g), 4, 2, 10, 8, ctypes.c_float(1.5)) == 0
    st = lib.gbsdf_hashgrid_fwd(ctypes.byref(g), 4, None, 10, None, 0, None, 0, None)
    assert st == 1 and b"NULL" in lib.gbsdf_last_error()
    assert lib.gbsdf_hashgrid_fwd(ctypes.byref(g), 9, None, 10, None, 0, None, 0, None) == 1


def test_sampler_args_layout_and_validation_without_gpu(lib):
    from neuralangelo_gb300.sampler import SamplerArgs, check_struct_size
    check_struct_size()
    a = SamplerArgs()
    a.R, a.ld, a.n_list, a.n_merge, a.n_fine = 4, 64, 64, 16, 16
    a.center = a.ray_unit = a.dists = 16            # non-NULL placeholders: validation runs first
    assert lib.gbsdf_sampler_round(ctypes.byref(a), None) == 1
    assert b"row stride" in lib.gbsdf_last_error()
    a.ld, a.n_list, a.n_merge = 600, 560, 16
    assert lib.gbsdf_sampler_round(ctypes.byref(a), None) == 1
    assert b"exceeds 512" in lib.gbsdf_last_error()
    a.n_list, a.n_merge, a.n_fine = 64, 0, 16
    a.fine_d = 16
    assert lib.gbsdf_sampler_round(ctypes.byref(a), None) == 1
    assert b"SDF values" in lib.gbsdf_last_error()


def test_field_backward_weight_gradient_arguments_without_gpu(lib):
    """The backward needs d_pre0, or d_w0 with K0 <= 64; both rejected before any launch."""
    from neuralangelo_gb300.fused import FieldArgs, check_struct_sizes
    check_struct_sizes()
    a = FieldArgs()
    assert lib.gbsdf_grid_init(ctypes.byref(a.grid), 16, 8, 14, 32, ctypes.c_float(1.3195079)) == 0
    a.Ns, a.S = 100, 10
    # non-NULL, 16-byte aligned placeholders: validation runs before anything is dereferenced
    for f in ("center", "ray_unit", "dists", "table", "w0e", "w0b", "w0x", "b0", "whead", "bhead", "grad",
              "d_sdf", "d_grad", "d_hess", "d_xc", "d_h0c", "x0ext", "d_enc", "d_whead", "d_bhead"):
        setattr(a, f, 256)
    a.active, a.K0 = 16, 128
    a.d_w0 = 256
    assert lib.gbsdf_field_mlp_bwd(ctypes.byref(a), None) == 1
    assert b"K0 <= 64" in lib.gbsdf_last_error()
    a.active, a.K0 = 8, 64
    a.d_w0 = None
    assert lib.gbsdf_field_mlp_bwd(ctypes.byref(a), None) == 1
    assert b"d_pre0" in lib.gbsdf_last_error()
    a.d_pre0 = 8                                   # misaligned
    assert lib.gbsdf_field_mlp_bwd(ctypes.byref(a), None) == 1
    assert b"d_pre0" in lib.gbsdf_last_error()


def test_x0ext_alignment_rejected_without_gpu(lib):
    """The field MLP kernels load x0ext rows by TMA: a base off 16 bytes is an argument error."""
    from neuralangelo_gb300.fused import FieldArgs
    a = FieldArgs()
    assert lib.gbsdf_grid_init(ctypes.byref(a.grid), 16, 8, 14, 32, ctypes.c_float(1.3195079)) == 0
    a.Ns, a.S = 100, 10
    for f in ("center", "ray_unit", "dists", "table", "w0e", "w0b", "w0x", "b0", "whead", "bhead", "grad",
              "d_sdf", "d_grad", "d_hess", "d_xc", "d_h0c", "d_enc", "d_whead", "d_bhead", "d_w0"):
        setattr(a, f, 256)
    a.active, a.K0 = 8, 64
    a.x0ext = 264                                  # 8 bytes past a 16-byte boundary
    assert lib.gbsdf_field_mlp_bwd(ctypes.byref(a), None) == 1
    assert b"x0ext" in lib.gbsdf_last_error()
    a.sdf, a.hess, a.h0c = 256, 256, 256
    assert lib.gbsdf_field_mlp_fwd(ctypes.byref(a), None) == 1
    assert b"x0ext" in lib.gbsdf_last_error()


def test_workspace_size_queries(lib):
    """The field calls' caller-owned buffers are sized by the library: rows are whole tiles of
    18 samples x 7 evaluations (6 taps) or 25 x 5 (4 taps); render and dense need none."""
    from neuralangelo_gb300.encoding import GridLayout
    from neuralangelo_gb300.fused import FieldWorkspace
    lay = GridLayout(8, 4, 16, 16, 1.5)
    for taps, rows in ((6, 6 * 126), (0, 6 * 126), (4, 4 * 125)):
        w = FieldWorkspace()
        assert lib.gbsdf_field_workspace_size(ctypes.c_int64(100), 32, taps, 1, ctypes.byref(lay.struct),
                                              ctypes.byref(w)) == 0
        assert w.rows == rows
        assert w.x0ext_bytes == rows * (2 * 32 + 16) * 2 and w.d_enc_bytes == rows * 32 * 4
        assert w.d_w0_bytes == 256 * 48 * 4 and w.d_pre0_bytes == 0
        assert w.d_table_fix_bytes == int(lay.struct.offset[8]) * 4 * 8
    w = FieldWorkspace()
    assert lib.gbsdf_field_workspace_size(ctypes.c_int64(1000), 80, 6, 0, None, ctypes.byref(w)) == 0
    assert w.d_w0_bytes == 0 and w.d_pre0_bytes == w.rows * 256 * 2 and w.d_table_fix_bytes == 0
    assert lib.gbsdf_field_workspace_size(ctypes.c_int64(10), 32, 5, 0, None, ctypes.byref(w)) == 1
    assert b"taps" in lib.gbsdf_last_error()
    lib.gbsdf_render_workspace_size.restype = ctypes.c_size_t
    lib.gbsdf_dense_workspace_size.restype = ctypes.c_size_t
    assert lib.gbsdf_render_workspace_size(ctypes.c_int64(16384), 128, 32) == 0
    assert lib.gbsdf_dense_workspace_size(ctypes.c_int64(1 << 21), 256, 256) == 0


def test_weightnorm_arguments_without_gpu(lib):
    """gbsdf_weightnorm_bwd: the binding's struct layout, and the argument checks that return
    before any launch."""
    from neuralangelo_gb300 import fused
    lib.gbsdf_weightnorm_layer_size.restype = ctypes.c_size_t
    assert lib.gbsdf_weightnorm_layer_size() == ctypes.sizeof(fused.WeightNormLayer)
    one = ctypes.c_float(1.0)
    assert lib.gbsdf_weightnorm_bwd(fused.WN_MAX_LAYERS + 1, None, None, one, None) == 1
    assert b"entries" in lib.gbsdf_last_error()
    arr = (fused.WeightNormLayer * 1)()
    arr[0].rows, arr[0].cols = 4, 8
    ptr = ctypes.cast(arr, ctypes.c_void_p)
    assert lib.gbsdf_weightnorm_bwd(1, ptr, None, one, None) == 1
    assert b"NULL dW" in lib.gbsdf_last_error()
    arr[0].dW, arr[0].dv, arr[0].ld_dw = 16, 16, 8
    arr[0].v = 16                                   # weight norm without g / dg
    assert lib.gbsdf_weightnorm_bwd(1, ptr, None, one, None) == 1
    assert b"needs g and dg" in lib.gbsdf_last_error()
    assert lib.gbsdf_weightnorm_bwd(0, None, None, one, None) == 0


def test_weightnorm_pack_arguments_without_gpu(lib):
    """gbsdf_weightnorm_fwd: the binding's struct layout and the checks that return before any
    launch (segment past the row, no destination)."""
    from neuralangelo_gb300 import fused
    lib.gbsdf_weightnorm_pack_size.restype = ctypes.c_size_t
    assert lib.gbsdf_weightnorm_pack_size() == ctypes.sizeof(fused.WeightNormPack)
    arr = (fused.WeightNormPack * 1)()
    e = arr[0]
    e.rows, e.cols, e.v, e.ld_src, e.col0, e.ncols = 4, 8, 16, 8, 6, 4
    ptr = ctypes.cast(arr, ctypes.c_void_p)
    assert lib.gbsdf_weightnorm_fwd(1, ptr, None) == 1
    assert b"segment" in lib.gbsdf_last_error()
    e.col0 = 0
    assert lib.gbsdf_weightnorm_fwd(1, ptr, None) == 1
    assert b"no destination" in lib.gbsdf_last_error()
    assert lib.gbsdf_weightnorm_fwd(fused.WN_MAX_LAYERS + 1, None, None) == 1
    assert lib.gbsdf_weightnorm_fwd(0, None, None) == 0
