"""Launch-shape autotuner of the fused step (project-written).

The fused step's kernels have launch shapes that do not change their results but do change
their speed with the workload: the table scatter's corners per pass (register use against
resident warps), the field forward's CTAs per SM, and each dense layer shape's N tile and
pipeline depth.  ``StepTuner.tune(batch)`` runs one eager step to build the workspace, then
re-issues each of those calls on the step's own buffers for every candidate shape, times them
with CUDA events on the launching stream, and keeps the fastest.  Choices are cached per
workload key (samples, active levels, taps, ragged layout) in memory and, given a path, in a
JSON file, so a training loop tunes once per shape.  A CapturedStep captured after tuning
replays the tuned launches.
"""
import ctypes
import json
import os

import torch

from . import _lib
from . import fused as _fused

_lib.register("gbsdf_dense_tune", [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32])


class StepTuner:
    SCATTER_CPT = (2, 4, 8)
    FWD_CTAS = (1, 2)
    DENSE_SHAPES = ((128, 6), (128, 4), (128, 3), (64, 6), (256, 3))     # (n_tile, ring slots)

    def __init__(self, fused, reps=5, cache_path=None):
        self.fused = fused
        self.reps = int(reps)
        self.cache_path = cache_path
        self.cache = {}
        if cache_path and os.path.exists(cache_path):
            with open(cache_path) as fh:
                self.cache = json.load(fh)
        self.timings = {}

    def key(self, batch):
        ragged = 'ray_offsets' in batch
        ns = int(batch['dists'].numel())
        sdf = self.fused.model.neural_sdf
        return f"Ns={ns},active={sdf.active_levels},taps={self.fused.taps},ragged={int(ragged)}"

    def _time(self, fn):
        stream = torch.cuda.current_stream()
        fn()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(self.reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / self.reps

    def tune(self, batch):
        """Choose, apply and return the launch shapes for this batch's workload."""
        key = self.key(batch)
        if key in self.cache:
            self.apply(self.cache[key])
            return self.cache[key]
        ff, model = self.fused, self.fused.model
        stream = _lib.stream_ptr(batch['center'].device)
        _fused.DENSE_CALLS = []
        try:
            model.zero_grad(set_to_none=False)
            ff.step(batch, compute_loss=False)
            calls = _fused.DENSE_CALLS
        finally:
            _fused.DENSE_CALLS = None
        torch.cuda.synchronize()
        fa = ff._fa
        choice = {}

        def field_call(name, attr, value):
            setattr(fa, attr, value)
            _lib.call(name, ctypes.byref(fa), stream)

        for name, attr, cands in (("gbsdf_field_scatter", "scatter_cpt", self.SCATTER_CPT),
                                  ("gbsdf_field_mlp_fwd", "fwd_ctas", self.FWD_CTAS)):
            if attr == "scatter_cpt" and ff.F != 8:
                continue
            t = {v: self._time(lambda v=v: field_call(name, attr, v)) for v in cands}
            self.timings[name] = t
            choice[attr] = min(t, key=t.get)
        shapes = {}
        for args in calls:
            shapes.setdefault((args[1], args[2]), []).append(args)
        dense = {}
        for (K, N), group in shapes.items():
            t = {}
            for n_tile, slots in self.DENSE_SHAPES:
                if N % n_tile:
                    continue
                _lib.call("gbsdf_dense_tune", K, N, n_tile, slots)
                t[(n_tile, slots)] = self._time(lambda g=group: [_lib.call("gbsdf_dense", *a) for a in g])
            _lib.call("gbsdf_dense_tune", K, N, 0, 0)
            best = min(t, key=t.get)
            self.timings[f"gbsdf_dense K={K} N={N}"] = {f"{a}x{b}": v for (a, b), v in t.items()}
            dense[f"{K},{N}"] = list(best)
        choice["dense"] = dense
        model.zero_grad(set_to_none=False)          # the re-issued calls added into the gradients
        self.cache[key] = choice
        if self.cache_path:
            with open(self.cache_path, "w") as fh:
                json.dump(self.cache, fh, indent=1)
        self.apply(choice)
        return choice

    def apply(self, choice):
        self.fused.tuning = {k: v for k, v in choice.items() if k != "dense"}
        for kn, (n_tile, slots) in choice.get("dense", {}).items():
            K, N = (int(x) for x in kn.split(","))
            _lib.call("gbsdf_dense_tune", K, N, int(n_tile), int(slots))
