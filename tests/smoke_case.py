"""One small forward+backward of the field on a CUDA device, checked against the oracle."""
import numpy as np
import torch

from tests import golden_io, params_io


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run(device="cuda:0", name="field_c1_small"):
    g = golden_io.load(name)
    model = params_io.model_from_golden(g, device)
    batch = params_io.batch_to(g['batch'], device)
    out = model.render_step(batch)
    out['loss'].backward()
    torch.cuda.synchronize()
    z = g['z']
    assert rel(out['sdf'].detach().cpu(), z['sdf']) < 1e-5
    assert rel(out['rgb'].detach().cpu(), z['rgb']) < 1e-5
    assert abs(float(out['loss']) - float(z['losses'][0])) < 1e-4 * abs(float(z['losses'][0]))
    grads = params_io.model_grads(model)
    assert rel(grads['table'], z['g_table']) < 1e-3
    return dict(loss=float(out['loss']), table_grad_rel=rel(grads['table'], z['g_table']))
