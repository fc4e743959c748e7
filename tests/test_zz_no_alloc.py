"""The allocation-free marching-cubes entry point (gbsdf_mc_block_noalloc).

It exists for callers that cannot allocate device memory (a host application
that owns the device budget, or a loop where cudaMalloc/cudaFree could
synchronise the device): its scratch is a fixed file-scope device array of the
library, limited to blocks of 33 points per axis.  The test calls it through the
C ABI twice in a row, on two different volumes, and checks each result against
gbsdf_mc_block (caller-provided workspace) with the tolerances of the other mesh
tests: faces bit-exact, vertices to 1e-12.  This file is collected last so that
a run stopping at the first failure has already run every other test; it also
passes on its own in a fresh process."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def volumes():
    rng = np.random.default_rng(5)
    n = 33
    intv = 1.6 / n
    g = (np.arange(n) - (n - 1) / 2) * intv
    X, Y, Z = np.meshgrid(g, g, g, indexing='ij')
    sphere = (0.5 - np.sqrt(X ** 2 + Y ** 2 + Z ** 2)).astype(np.float32)
    noise = rng.normal(size=(21, 17, 33)).astype(np.float32)
    return [(sphere, np.full(3, -(n - 1) / 2 * intv), intv), (noise, np.array([-0.3, -0.25, -0.5]), 0.03)]


def test_noalloc_matches_workspace_entry_point_twice():
    from neuralangelo_gb300 import mesh as gm
    Vb = torch.empty(3 * 33 ** 3, 3, dtype=torch.float64, device=DEV)
    Fb = torch.empty(5 * 32 ** 3, 3, dtype=torch.int64, device=DEV)
    counts = torch.zeros(2, dtype=torch.int64, device=DEV)
    ref_mc = gm.MarchingCubes(33, DEV)
    for vol, origin, intv in volumes():
        v = torch.from_numpy(vol).to(DEV)
        V, F = gm.marching_cubes_noalloc(v, origin, intv, Vb, Fb, counts)
        Vr, Fr = ref_mc(v, origin, intv)
        assert F.shape[0] > 0
        assert torch.equal(F, Fr)
        assert torch.allclose(V, Vr, rtol=0, atol=1e-12)


def test_noalloc_rejects_blocks_beyond_its_limit():
    from neuralangelo_gb300 import _lib
    from neuralangelo_gb300 import mesh as gm   # noqa: F401  (registers the signature)
    lib = _lib.load()
    vol = torch.zeros(34, 4, 4, device=DEV)
    out = torch.empty(8, dtype=torch.float64, device=DEV)
    org = (ctypes.c_double * 3)(0.0, 0.0, 0.0)
    st = lib.gbsdf_mc_block_noalloc(ctypes.c_void_p(vol.data_ptr()), 34, 4, 4, 0.0, org, 0.1,
                                    ctypes.c_void_p(out.data_ptr()), 10 ** 9, ctypes.c_void_p(out.data_ptr()), 10 ** 9,
                                    ctypes.c_void_p(out.data_ptr()), None)
    assert st == 1
    assert b"33 points per axis" in lib.gbsdf_last_error()
