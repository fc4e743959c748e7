"""neuralangelo_gb300 -- the Neuralangelo neural-SDF field and volume-rendering
hot path as hand-written sm_103a CUDA kernels behind a C ABI (libgbsdf.so).

Public surface (mirrors the reference):
  HashGridEncoding / Encoding   tcnn.Encoding drop-in          (encoding.py)
  NeuralSDF, NeuralRGB          modules.py mirrors              (modules.py)
  compute_neus_alphas, alpha_compositing_weights, composite    (render.py)
  FieldModel                    plain FP32 drop-in training forward (model.py)
  FusedField                    fused FP16/FP32 forward+backward     (fused.py)
  extract_mesh                  block-wise SDF grid + GPU marching cubes (mesh.py)
"""
from .config import AttrDict, field_config, to_attr  # noqa: F401
from .encoding import Encoding, HashGridEncoding  # noqa: F401
