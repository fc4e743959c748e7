"""CPU oracle for the neural-SDF field and volume-rendering path.

TEST INFRASTRUCTURE ONLY.  Nothing in the shipped package imports this
directory; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
legs of ``bench.py`` use it, and only as the checker or the timed CPU
baseline.

Contents
--------
hashgrid.py   numpy restatement of the multi-resolution hash-grid encoding
              that NeuralSDF obtains from ``tinycudann.Encoding``
              (projects/neuralangelo/utils/modules.py:33-58, 76-95).  The
              tiny-cuda-nn package is third-party and not vendored in the
              reference (requirements.txt:3, unpinned git URL), so the
              restatement follows its published algorithm (Mueller et al.
              2022, instant-NGP) and is pinned by known-answer tests.
field.py      float64 torch restatement of NeuralSDF / NeuralRGB / NeuS alpha /
              compositing / losses, pinned against golden vectors produced by
              the reference's own modules (tests/golden/make_golden.py).
mc.c          C restatement of iso-surface marching cubes used by
              projects/neuralangelo/utils/mesh.py:119-133 (PyMCubes, third
              party, unpinned: requirements.txt:23).
mesh_out.py   numpy restatement of the mesh output stage: trimesh's per-block
              vertex merge (utils/mesh.py:121-129), the centre/scale transform
              and degenerate-face removal (scripts/extract_mesh.py:96-97);
              trimesh is third party and absent, so parity is unpinned.
sampler.py    restatement of the hierarchical sampler
              (projects/neuralangelo/model.py:232-267,
              projects/nerf/utils/nerf_util.py:20-68).

Parity status: the hash-grid index formula and the marching-cubes case table
are *unpinned* against the third-party packages themselves (absent here); the
field, rendering and loss composition are pinned against the reference's own
modules through the committed golden fixtures.
"""
