"""Benchmark: SDF samples/s for one training forward+backward of the full neural-SDF
field (16 levels x 8 features, T=2^22, 32->2048, 8 levels active; SDF MLP 256;
colour MLP 4x256 with a 16-dim appearance embedding over 100 images) on
16384 rays x 128 samples, seeded synthetic rays and colours.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--mode fused|plain]

Prints ONE JSON line (rank 0).  ``value`` is the device-resident throughput of
the selected mode (default: the fused path when built, else the plain FP32
drop-in), ``e2e`` the same step through the public API with the batch copied
from pinned host memory and the loss read back every step.  Under torchrun
every rank runs an independent replica (rays are independent, so the path has
no exchange step: replicas only) and ``value`` sums the ranks' samples over the
slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

R_RAYS, N_SAMPLES, ACTIVE = 16384, 128, 8
METRIC = "SDF samples/s fwd+bwd (full field, 16384 rays x 128 samples)"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--mode", default="auto", choices=["auto", "fused", "plain"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-plain", action="store_true", help="skip the plain FP32 denominator (profiling runs)")
    p.add_argument("--rays", type=int, default=R_RAYS)
    p.add_argument("--samples", type=int, default=N_SAMPLES)
    p.add_argument("--no-extras", action="store_true",
                   help="skip the ragged-batching, sampler and mesh measurements")
    p.add_argument("--split-colour-grads", action="store_true",
                   help="carry the colour MLP's input gradients as fp16 hi+lo pairs")
    return p.parse_args()


# --------------------------------------------------------------------------- ncu-measured traffic

def profiled_traffic(kernel):
    """(DRAM bytes per sample, source, L2 throughput % or None) of a C-ABI call's kernel from
    measured_traffic.json, or (None, None, None).  bench.py cannot run ncu itself: the figures
    come from one ncu capture of the same kernels on a smaller case of the same field,
    scaled by the samples a step processes."""
    try:
        data = json.load(open(os.path.join(ROOT, "measured_traffic.json")))
    except (OSError, ValueError):
        return None, None, None
    c = data.get("calls", {}).get(kernel)
    if not c:
        return None, None, None
    return float(c["dram_bytes_per_sample"]), f"{c.get('kernel', kernel)}: {c['source']}", c.get("l2_throughput_pct")


# kernels of this library launched by one call of each entry point
KERNELS_PER_CALL = {"gbsdf_field_fwd": 2, "gbsdf_field_bwd": 2}   # others: 1


# calls whose algorithmic bytes count every table-corner touch (mostly served by L2)
GATHER_SCATTER = ("gbsdf_field_encode", "gbsdf_field_scatter")


# --------------------------------------------------------------------------- extra workloads

def bench_ragged(model, device, steps, warmup, rays=65536, seed=0):
    """Ragged batching: 65536 rays, 30% culled to zero samples, the rest 16..256 samples
    (6.2M samples), the fused step captured in one CUDA graph; against the same rays in
    the reference's dense layout padded to 128 samples (8.4M samples, misses computed); and
    the ragged step again with the launch shapes autotune.StepTuner chose for it."""
    import torch
    from neuralangelo_gb300.fused import CapturedStep, FusedField
    from neuralangelo_gb300.workloads import make_ragged_rays, padded
    rag = make_ragged_rays(rays, seed=seed, n_images=100, device=device)
    useful = int(rag['dists'].numel())
    out = dict(rays=rays, useful_samples=useful)
    tuned = None
    for name, b in (("padded_128", padded(rag, 128, seed=seed)), ("ragged", rag), ("ragged_tuned", rag)):
        ff = FusedField(model)
        if name == "ragged_tuned":
            from neuralangelo_gb300.autotune import StepTuner
            tuned = StepTuner(ff, reps=3).tune(b)
        ns = int(b['dists'].numel())
        if name == "ragged":   # eager launches, for the graph's benefit
            ms_e = time_steps(lambda: ff.step(b, compute_loss=False), steps, warmup, lambda: None)
            out["ragged_eager_ms_per_step"] = round(ms_e, 3)
        cap = CapturedStep(ff, b)
        ms = time_steps(cap.replay, steps, warmup, lambda: None)
        out[name] = dict(samples=ns, ms_per_step=round(ms, 3), samples_per_s=round(ns / (ms * 1e-3), 1),
                         useful_samples_per_s=round(useful / (ms * 1e-3), 1))
        assert ff.check_device_errors() == 0
        del cap
        ff.release()
        torch.cuda.empty_cache()
    out["speedup_vs_padded"] = round(out["padded_128"]["ms_per_step"] / out["ragged"]["ms_per_step"], 3)
    out["tuning"] = tuned                      # autotune.StepTuner's launch shapes for this workload
    out["tuned_vs_default"] = round(out["ragged"]["ms_per_step"] / out["ragged_tuned"]["ms_per_step"], 3)
    return out


def bench_background(device, steps, warmup, rays=R_RAYS, samples=N_SAMPLES, n_bg=32, seed=0):
    """The same full-field step with the background NeRF of the reference's base config
    (8 x 256 ReLU with a skip at 4, 32 background samples per ray composited behind the
    object's: model.py:129-141), fused, against the plain FP32 path on the same rays."""
    import torch
    from neuralangelo_gb300.config import field_config
    from neuralangelo_gb300.fused import CapturedStep, FusedField
    from neuralangelo_gb300.model import FieldModel
    from neuralangelo_gb300.workloads import full_field_iteration, init_field_params, make_rays
    cfg = field_config("full", background=True)
    torch.manual_seed(seed)
    m = FieldModel(cfg).to(device)
    init_field_params(m, seed)
    m.schedule(full_field_iteration(ACTIVE))
    b = make_rays(rays, samples, seed=seed, n_images=100, device=device, n_bg=n_bg)
    ff = FusedField(m)
    cap = CapturedStep(ff, b)
    ms = time_steps(cap.replay, steps, warmup, lambda: None)
    assert ff.check_device_errors() == 0
    del cap
    ff.release()

    def plain():
        m.zero_grad(set_to_none=True)
        m.render_step(b)["loss"].backward()
    ms_plain = time_steps(plain, max(2, steps // 2), 1, lambda: None)
    torch.cuda.empty_cache()
    ns = rays * samples
    return dict(rays=rays, object_samples=ns, background_samples=rays * n_bg, ms_per_step=round(ms, 3),
                samples_per_s=round(ns / (ms * 1e-3), 1), plain_fp32_ms_per_step=round(ms_plain, 3),
                speedup_vs_plain=round(ms_plain / ms, 3))


def bench_taps4(device, steps, warmup, rays=R_RAYS, samples=N_SAMPLES, seed=0):
    """The same full-field step with the 4-tap tetrahedral stencil, the reference's default
    configuration (projects/neuralangelo/configs/base.yaml:68): 5 evaluations per sample
    instead of 7, replayed from a captured CUDA graph."""
    import torch
    from neuralangelo_gb300.fused import CapturedStep, FusedField
    from neuralangelo_gb300.workloads import make_rays
    model = make_plain(device, seed, taps=4)
    batch = make_rays(rays, samples, seed=seed, n_images=100, device=device)
    cap = CapturedStep(FusedField(model), batch)
    ms = time_steps(cap.replay, steps, warmup, lambda: None)
    out = dict(samples=rays * samples, ms_per_step=round(ms, 3),
               value=round(rays * samples / (ms * 1e-3), 1), unit="samples/s")
    del cap
    torch.cuda.empty_cache()
    return out


def bench_sampler(model, device, steps=5, warmup=2, rays=R_RAYS, seed=0):
    """The no-grad hierarchical pre-pass (64 coarse + 4 x 16 importance samples per ray,
    SDF of the fused field kernel), timed separately from the training step."""
    import torch
    from neuralangelo_gb300.sampler import HierarchicalSampler, field_sdf_fn
    from neuralangelo_gb300.workloads import make_rays, sphere_bounds
    b = make_rays(rays, 1, seed=seed, device=device)
    near, far, _ = sphere_bounds(b['center'], b['ray_unit'])
    u = torch.rand(rays, 64, device=device, generator=torch.Generator(device=device).manual_seed(seed))
    smp = HierarchicalSampler(64, 16, 4)
    fn = field_sdf_fn(model.neural_sdf)
    ms = time_steps(lambda: smp(fn, b['center'], b['ray_unit'], near, far, u=u), steps, warmup, lambda: None)
    evals = rays * (64 + 3 * 16)
    return dict(rays=rays, samples_per_ray=smp.n_samples, ms_per_call=round(ms, 3),
                rays_per_s=round(rays / (ms * 1e-3), 1), sdf_evals_per_s=round(evals / (ms * 1e-3), 1))


def bench_mesh(model, device, res=512, block_res=128, shapes_seed=7, fit_steps=300):
    """Mesh extraction from a trained-shape field: a fresh full field (L16 F8 T2^22) whose SDF
    is fitted to a seeded union of 3 spheres and 2 boxes (workloads.shapes_union, Adam on L1),
    then a 512^3 lattice in 128^3 blocks: lattice SDF kernel + GPU marching cubes per block,
    each block's mesh copied to the host as the reference does (mesh.py:33-46)."""
    import torch
    from neuralangelo_gb300.mesh import FieldSDF, extract_mesh
    from neuralangelo_gb300.workloads import fit_sdf, shapes_union
    target = shapes_union(shapes_seed)
    field = make_plain(device, seed=1)
    t_fit = time.perf_counter()
    fit_loss = fit_sdf(field.neural_sdf, target, steps=fit_steps)
    t_fit = time.perf_counter() - t_fit
    f = FieldSDF(field.neural_sdf, sign=-1.0)
    intv = 2.0 / res
    bounds = [(-1.0, 1.0)] * 3
    extract_mesh(f, [(-1.0, -0.5)] * 3, intv, block_res, device=device)   # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mesh = extract_mesh(f, bounds, intv, block_res, device=device)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    pts = (res + (res // block_res - 1)) ** 3          # lattice points incl. the block overlaps
    # output stage (extract_mesh.py:96-100): weld across blocks, transform, degenerate
    # faces on the GPU; then the PLY file
    import tempfile
    from neuralangelo_gb300.mesh import finalize_mesh, write_ply
    V = torch.from_numpy(mesh.vertices).to(device)
    F = torch.from_numpy(mesh.faces).to(device)
    finalize_mesh(V[:1000], F[:0], weld=True)                            # warm-up
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    Vo, Fo = finalize_mesh(V, F, weld=True, scale=1.0, offset=(0.0, 0.0, 0.0))
    torch.cuda.synchronize()
    t_fin = time.perf_counter() - t1
    with tempfile.TemporaryDirectory() as d:
        t2 = time.perf_counter()
        write_ply(os.path.join(d, "mesh.ply"), Vo.cpu().numpy(), Fo.cpu().numpy())
        t_ply = time.perf_counter() - t2
    with torch.no_grad():
        err = target(torch.from_numpy(mesh.vertices).to(device)).abs()
    return dict(field=f"full field fitted to shapes_union({shapes_seed}) in {fit_steps} Adam steps "
                      f"({t_fit:.1f} s, final L1 {fit_loss:.4f}); surface vertices' distance to the target "
                      f"surface: median {float(err.median()):.4f}",
                resolution=res, block_res=block_res, seconds=round(dt, 4), lattice_points=pts,
                points_per_s=round(pts / dt, 1), vertices=int(mesh.vertices.shape[0]),
                faces=int(mesh.faces.shape[0]), welded_vertices=int(Vo.shape[0]),
                finalize_seconds=round(t_fin, 5), ply_write_seconds=round(t_ply, 4))


# --------------------------------------------------------------------------- CPU baseline

def cpu_port_sample(rays=64, samples=N_SAMPLES, steps=5, warmup=2):
    """The reference's path on the host cores: the oracle's float32 restatement of the
    reference modules (pinned to them by golden vectors; the reference itself is not on
    the GPU machine and its encoder is a CUDA-only third-party package) on a bounded sample of
    the full-field workload, all host threads, `warmup` untimed steps, median of `steps`."""
    import torch
    from oracle import field as of
    from neuralangelo_gb300.workloads import full_field_iteration, make_rays
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    cfg = of.make_config(active_levels=ACTIVE, app_dim=16, n_images=100)
    params, layout = of.init_params(cfg, seed=0, dtype=torch.float32)
    params = {k: v.requires_grad_(True) for k, v in params.items()}
    b = make_rays(rays, samples, seed=0, n_images=100)
    it = full_field_iteration(ACTIVE)
    eps = of.normal_eps(cfg, ACTIVE)
    w_curv = 5e-4 / (cfg['per_level_scale'] ** (ACTIVE - 1))
    times = []
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        out = of.render_step(params, cfg, layout, b, eps, it / 500000, 0.1, w_curv)
        out['loss'].backward()
        dt = time.perf_counter() - t0
        if i >= warmup:
            times.append(dt)
        for v in params.values():
            v.grad = None
    t = statistics.median(times)
    return dict(value=rays * samples / t, unit="samples/s", cores=threads, kind="port",
                sample=f"{rays} rays x {samples} samples of the full field (L16 F8 T2^22, 8 active), float32, "
                       f"oracle restatement of the reference modules (torch CPU + numpy hash grid), "
                       f"median of {steps} after {warmup} warm-up",
                seconds_per_step=t, mean_seconds_per_step=sum(times) / len(times))


REF_RAYS = 32          # rays per reference-arm step (a bounded sample of the 16384-ray workload)


def run_reference(args):
    """The reference arm: the reference's path on the host cores (the oracle's restatement,
    see cpu_port_sample), --warmup untimed and --steps timed steps, each a bounded sample of
    REF_RAYS rays x 128 samples of the full-field workload.  Under torchrun only rank 0 runs."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    steps, warmup = max(1, args.steps), max(0, args.warmup)
    cb = cpu_port_sample(rays=REF_RAYS, steps=steps, warmup=warmup)
    value = REF_RAYS * N_SAMPLES / cb["mean_seconds_per_step"]
    cb_line = dict(value=round(value, 1), unit="samples/s", cores=cb["cores"], kind=cb["kind"], sample=cb["sample"])
    line = dict(metric=METRIC, value=round(value, 1), unit="samples/s", n_gpus=args.gpus, steps=steps,
                warmup=warmup, ms_per_step=round(cb["mean_seconds_per_step"] * 1e3, 3), higher_is_better=True,
                scaling="weak", vs_baseline=None, dtype="f32", data="synthetic",
                config=dict(workload=f"full field L16 F8 T2^22 (8 active), 16384 rays x 128 samples; "
                                     f"each step a {REF_RAYS}-ray sample on the host cores",
                            rays_per_step=REF_RAYS, samples_per_ray=N_SAMPLES, parallelism="host cores"),
                impl="reference", cpu_baseline=cb_line,
                e2e=dict(value=round(value, 1), unit="samples/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        # nvidia-smi numbers GPUs physically: query by UUID so a CUDA_VISIBLE_DEVICES
        # remapping still samples the GPU this process runs on
        self.index = str(device)
        try:
            import torch
            uuid = str(torch.cuda.get_device_properties(device).uuid)
            if uuid:
                self.index = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
        except Exception:                      # noqa: BLE001 (no CUDA or no uuid: fall back to the ordinal)
            pass
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"gbsdf_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.index, "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        try:
            os.remove(self.path)
        except OSError:
            pass
        if not sm:
            return None
        return dict(sm_mhz=statistics.median(sm), sm_max_mhz=max(mx), reasons=sorted(reasons), samples=len(sm))


# --------------------------------------------------------------------------- GPU arm

def make_plain(device, seed=0, taps=6):
    import torch
    from neuralangelo_gb300.config import field_config
    from neuralangelo_gb300.model import FieldModel
    from neuralangelo_gb300.workloads import full_field_iteration, init_field_params
    torch.manual_seed(seed)
    cfg = field_config("full")
    cfg.sdf.gradient.taps = taps
    model = FieldModel(cfg).to(device)
    init_field_params(model, seed)
    model.schedule(full_field_iteration(ACTIVE))
    assert model.neural_sdf.active_levels == ACTIVE
    return model


def step_plain(model, batch):
    model.zero_grad(set_to_none=True)
    out = model.render_step(batch)
    out["loss"].backward()
    return out["loss"]


def time_steps(fn, steps, warmup, barrier):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    barrier()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        fn()
    b.record()
    torch.cuda.synchronize()
    barrier()
    return a.elapsed_time(b) / steps


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    device = f"cuda:{local}"
    torch.cuda.set_device(device)
    from neuralangelo_gb300.replicas import ReplicaGroup
    group = ReplicaGroup()            # replicas: one independent field per rank, shared timing only
    world, rank = group.world, group.rank
    barrier, max_over_ranks = group.barrier, group.max

    import __graft_entry__
    __graft_entry__.build()
    from neuralangelo_gb300 import _lib
    from neuralangelo_gb300.workloads import encoder_bytes_per_sample, flops_per_sample, make_rays

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    R, N = args.rays, args.samples
    n_samples = R * N
    host_batch = make_rays(R, N, seed=rank, n_images=100)
    batch = {k: v.to(device) for k, v in host_batch.items()}
    pinned = {k: v.pin_memory() for k, v in host_batch.items()}
    h2d = sum(v.numel() * v.element_size() for v in pinned.values())

    model = make_plain(device)
    fused = None
    if args.mode in ("auto", "fused"):
        from neuralangelo_gb300.fused import FusedField
        fused = FusedField(model, split_colour_grads=args.split_colour_grads)
    mode = "fused" if fused is not None else "plain"

    def step_fused(b, compute_loss=False):
        model.zero_grad(set_to_none=True)
        return fused.step(b, compute_loss=compute_loss)

    def measure(fn, steps, warmup):
        _lib.TIMER.reset()
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        _lib.TIMER.enabled = True
        ms_ = time_steps(fn, steps, 0, barrier)
        _lib.TIMER.enabled = False
        torch.cuda.synchronize()
        return ms_, _lib.TIMER.summary()

    # the plain FP32 drop-in (the denominator of the fused speed-up): torch's default FP32
    # matmuls, and the same with TF32 tensor-core matmuls, as the reference's trainer sets by
    # default (imaginaire/trainers/base.py:172-175)
    plain_ms = plain_tf32_ms = float("nan")
    if not args.no_plain or fused is None:
        tf32 = (torch.backends.cuda.matmul.allow_tf32, torch.backends.cudnn.allow_tf32)
        torch.backends.cuda.matmul.allow_tf32 = torch.backends.cudnn.allow_tf32 = False
        plain_ms, plain_k = measure(lambda: step_plain(model, batch), max(2, args.steps // 2), args.warmup)
        plain_ms = max_over_ranks(plain_ms)
        if fused is not None:
            torch.backends.cuda.matmul.allow_tf32 = torch.backends.cudnn.allow_tf32 = True
            plain_tf32_ms, _ = measure(lambda: step_plain(model, batch), max(2, args.steps // 2), args.warmup)
            plain_tf32_ms = max_over_ranks(plain_tf32_ms)
        torch.backends.cuda.matmul.allow_tf32, torch.backends.cudnn.allow_tf32 = tf32
    cap = None
    if fused is not None:
        # per-call device times (CUDA events around every C-ABI call) from eager steps;
        # the headline then times the same step launched as one CUDA graph (CapturedStep)
        ksteps = max(3, args.steps // 2)
        _, ksum = measure(lambda: step_fused(batch), ksteps, args.warmup)
        kbytes = dict(_lib.TIMER.bytes)
        from neuralangelo_gb300.fused import CapturedStep
        cap = CapturedStep(fused, batch)
    clocks = ClockSampler(local)
    clocks.start()
    if cap is not None:
        ms = time_steps(cap.replay, args.steps, args.warmup, barrier)
    else:
        ms, ksum = measure(lambda: step_plain(model, batch), args.steps, args.warmup)
        kbytes = dict(_lib.TIMER.bytes)
        ksteps = args.steps
    clock = clocks.stop()
    ms = max_over_ranks(ms)
    value = world * n_samples / (ms * 1e-3)

    # end to end through the public API: H2D of the batch (from pinned memory) into the
    # graph's inputs, the step, D2H of the loss
    def e2e_step():
        if cap is not None:
            cap.replay(pinned)
            return cap.losses()["loss"]
        b = {k: v.to(device, non_blocking=True) for k, v in pinned.items()}
        return float(step_plain(model, b).detach().cpu())

    e2e_ms = time_steps(e2e_step, max(1, args.steps // 2), 1, barrier)
    e2e_ms = max_over_ranks(e2e_ms)

    # per-kernel algorithmic work (bytes, flops) of one launch, for the roofline
    # Bytes: what each launch must move per sample (table corners counted at every
    # touch, as the encoder's algorithmic figure does; L2 serves many of them).
    # FLOPs: the algorithmic MACs x 2 of the layer-0 GEMMs (no hi/lo doubling).
    F, A, H = 8, ACTIVE, 256
    K0 = 16 * ((A * F + 15) // 16)
    KX = 2 * K0 + 16                                     # x0ext row: features hi | tail | lo
    enc_read = A * 8 * F * (2 if mode == "fused" else 4)
    pair = 2 if (fused is not None and fused.pairs) else 1     # h0c and colour-tail rows as hi + lo
    work = {
        "gbsdf_hashgrid_fwd": (n_samples * (A * 8 * F * 4 + 16 * F * 4 + 12), 0),
        "gbsdf_hashgrid_bwd": (n_samples * (A * 8 * F * 8 + 16 * F * 4), 0),
        # table corners of 7 evaluations -> x0ext rows
        "gbsdf_field_encode": (n_samples * (7 * enc_read + 7 * KX * 2 + 4), 0),
        # x0ext rows -> SDF, gradient, Hessian, h0c row, colour-input tail
        "gbsdf_field_mlp_fwd": (n_samples * (7 * KX * 2 + 4 + 12 + 12 + ((H + 8) * 2 + 48 * 2) * pair),
                                n_samples * 7 * 2 * H * (K0 + 4 + 1)),
        # x0ext rows, d_h0c and the per-sample output gradients -> d_enc (fp32) and, K0 <= 64,
        # the layer-0 weight gradient in-kernel (extra MACs, no traffic), else d_pre0 (fp16)
        "gbsdf_field_mlp_bwd": (n_samples * (7 * KX * 2 + H * 4 + 52 + (0 if K0 <= 64 else 7 * H * 2) + 7 * K0 * 4),
                                n_samples * 7 * 2 * H * (2 * K0 + 4 + 1 + (K0 + 4 if K0 <= 64 else 0))),
        # d_enc -> FP32 read-modify-write of every corner touch
        "gbsdf_field_scatter": (n_samples * (7 * K0 * 4 + 7 * A * 8 * F * 8 + 4), 0),
    }
    # the dense layers, weight gradients and colour head: their algorithmic bytes as each call
    # reported them (fused.py: operand and output rows, hi + lo halves counted); their tensor
    # work is far below their HBM floor
    for name in ("gbsdf_dense", "gbsdf_wgrad", "gbsdf_rgb_head_fwd", "gbsdf_rgb_head_bwd"):
        if name in kbytes and name in ksum:
            work[name] = (kbytes[name] / ksum[name][0], 0)
    tensor_peak = peaks.get("bf16_tflops_sustained", 1700.0)

    def roofline_of(name, calls, tot_ms):
        """The binding roofline of one call: HBM (algorithmic bytes / measured copy
        bandwidth) or tensor (algorithmic FLOPs / measured sustained bf16 rate),
        whichever floor is longer."""
        per_launch_ms = tot_ms / calls
        by, fl = work[name]
        t = per_launch_ms * 1e-3
        hbm_floor, tensor_floor = by / (hbm_peak * 1e9), fl / (tensor_peak * 1e12)
        if tensor_floor > hbm_floor:
            r = dict(kernel=name, bound="tensor", achieved=round(fl / t / 1e12, 2), peak=tensor_peak,
                     unit="TFLOP/s", frac=round(fl / t / 1e12 / tensor_peak, 4),
                     peak_source="MEASURED_PEAKS.json bf16_tflops_sustained (of measured)")
        else:
            r = dict(kernel=name, bound="hbm", achieved=round(by / t / 1e9, 1), peak=hbm_peak, unit="GB/s",
                     frac=round(by / t / 1e9 / hbm_peak, 4),
                     peak_source="MEASURED_PEAKS.json hbm_gbs (burst, of measured)")
        tps, tsrc, l2pct = profiled_traffic(name)           # DRAM bytes per sample over a step's launches
        traffic = round(tps * n_samples * ksteps / calls) if tps is not None else None
        if name in GATHER_SCATTER and traffic:
            # gather and scatter touch every table corner of 7 evaluations; L2 serves most of those
            # touches (coarse levels, taps of one sample), so their HBM position is the measured DRAM
            # traffic over the time, and the per-touch rate is reported beside it
            r.update(achieved=round(traffic / t / 1e9, 1), frac=round(traffic / t / 1e9 / hbm_peak, 4),
                     touch_gbs=round(by / t / 1e9, 1), l2_throughput_pct=l2pct,
                     basis="measured DRAM bytes (ncu) per launch")
        r.update(traffic=traffic, traffic_source=tsrc,
                 dram_gbs=round(traffic / t / 1e9, 1) if traffic else None,
                 per_launch_ms=round(per_launch_ms, 4), algorithmic_bytes_per_launch=by, flops_per_launch=fl,
                 tensor_tflops=round(fl / t / 1e12, 2), launches_per_step=calls / ksteps)
        return r

    timed = [(k, v) for k, v in ksum.items() if k in work]
    dom = max(timed, key=lambda kv: kv[1][1]) if timed else None
    roof = roofline_of(dom[0], *dom[1]) if dom else None
    # the same for every timed field kernel (the dominant one is `roofline`)
    rooflines = {k: {x: y for x, y in roofline_of(k, *v).items()
                     if x in ("bound", "achieved", "unit", "frac", "per_launch_ms", "dram_gbs", "touch_gbs",
                              "l2_throughput_pct", "basis", "launches_per_step")}
                 for k, v in timed}
    launches = int(sum(c * KERNELS_PER_CALL.get(k, 1) for k, (c, _) in ksum.items()) / ksteps)
    extras = {}
    if not args.no_extras and fused is not None:
        cap = None                     # the graph holds the workspace; drop both before the extras
        fused.release()
        torch.cuda.empty_cache()
        torch.cuda.empty_cache()
        extras["taps4"] = bench_taps4(device, max(3, args.steps // 2), args.warmup)
        extras["ragged"] = bench_ragged(model, device, max(3, args.steps // 2), args.warmup)
        extras["background"] = bench_background(device, max(3, args.steps // 2), args.warmup)
        extras["sampler"] = bench_sampler(model, device)
        extras["mesh"] = bench_mesh(model, device)
    cb = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_port_sample()
        cb.pop("seconds_per_step", None)
        cb.pop("mean_seconds_per_step", None)
    if rank == 0:
        line = dict(metric=METRIC, value=round(value, 1), unit="samples/s", n_gpus=world, steps=args.steps,
                    warmup=args.warmup, ms_per_step=round(ms, 3), higher_is_better=True, scaling="weak",
                    vs_baseline=None, dtype="f32" if mode == "plain" else "f16", data="synthetic",
                    plain_fp32=(dict(value=round(world * n_samples / (plain_ms * 1e-3), 1), unit="samples/s",
                                     ms_per_step=round(plain_ms, 3)) if plain_ms == plain_ms else None),
                    speedup_vs_plain=round(plain_ms / ms, 3) if plain_ms == plain_ms else None,
                    plain_tf32=(dict(value=round(world * n_samples / (plain_tf32_ms * 1e-3), 1), unit="samples/s",
                                     ms_per_step=round(plain_tf32_ms, 3),
                                     note="plain drop-in with TF32 tensor-core matmuls (the reference "
                                          "trainer's default)") if plain_tf32_ms == plain_tf32_ms else None),
                    speedup_vs_plain_tf32=round(plain_tf32_ms / ms, 3) if plain_tf32_ms == plain_tf32_ms else None,
                    config=dict(workload=f"full field L16 F8 T2^22 (8 active), {R} rays x {N} samples, mode={mode}",
                                rays=R, samples_per_ray=N, active_levels=ACTIVE, mode=mode,
                                split_colour_grads=bool(args.split_colour_grads),
                                l2="inputs larger than L2 (1.46 GB table)", parallelism="replicas"),
                    e2e=dict(value=round(world * n_samples / (e2e_ms * 1e-3), 1), unit="samples/s",
                             h2d_bytes_per_step=h2d, d2h_bytes_per_step=32 if fused is not None else 4,
                             ms_per_step=round(e2e_ms, 3)),
                    roofline=roof, cpu_baseline=cb, gpu_launches=launches, clocks=clock,
                    flops_per_sample=flops_per_sample(model.cfg, ACTIVE),
                    encoder_bytes_per_sample=encoder_bytes_per_sample(ACTIVE, 8, 4),
                    kernel_ms_per_step={k: round(v[1] / ksteps, 4) for k, v in ksum.items()},
                    kernel_rooflines=rooflines,
                    **extras)
        print(json.dumps(line), flush=True)
    group.close()


if __name__ == "__main__":
    main()
