"""One small training forward+backward on a CUDA device, checked against the oracle:
the fused FP16 step (flagship path) and the plain FP32 drop-in on a golden case."""
import numpy as np
import torch

from tests import golden_io, params_io


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run_plain(device="cuda:0", name="field_c1_small"):
    g = golden_io.load(name)
    model = params_io.model_from_golden(g, device)
    batch = params_io.batch_to(g['batch'], device)
    out = model.render_step(batch)
    out['loss'].backward()
    torch.cuda.synchronize()
    z = g['z']
    assert rel(out['sdf'].detach().cpu(), z['sdf']) < 1e-5
    assert rel(out['rgb'].detach().cpu(), z['rgb']) < 1e-5
    grads = params_io.model_grads(model)
    assert rel(grads['table'], z['g_table']) < 1e-3
    return rel(grads['table'], z['g_table'])


def run_fused(device="cuda:0"):
    from neuralangelo_gb300.fused import FusedField
    from neuralangelo_gb300.workloads import make_rays
    from tests import test_fused_gpu as tf
    tf.DEV = device
    model = tf.build()
    batch = make_rays(16, 32, seed=7, miss_frac=0.1, n_images=10, device=device)
    ff = FusedField(model)
    model.zero_grad(set_to_none=True)
    res = ff.step(batch)
    torch.cuda.synchronize()
    assert ff.check_device_errors() == 0
    out_q, g_q = tf.oracle_run(model, batch, fp16=True)
    inside = ~batch['outside'][:, 0].cpu()
    e_sdf = rel(ff.ws['sdf'].reshape(16, 32).cpu()[inside], out_q['sdf'].detach()[inside])
    e_tab = rel(model.neural_sdf.tcnn_encoding.params.grad.double().cpu(), g_q['table'])
    assert e_sdf < 1e-4, e_sdf
    assert e_tab < 1e-3, e_tab
    assert abs(res['loss'] - float(out_q['loss'])) < 1e-5 * abs(float(out_q['loss']))
    return e_sdf, e_tab


def run(device="cuda:0"):
    return dict(plain_table_grad_rel=run_plain(device), fused_sdf_tab_rel=run_fused(device))
