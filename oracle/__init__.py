"""The oracle: CPU restatements of Instant-angelo's NeuS / Neuralangelo hot path.

TEST INFRASTRUCTURE ONLY.  ``tests/``, ``__graft_entry__.smoke`` and the
CPU-baseline leg of ``bench.py`` import it as the checker; the product package
(``instant-angelo_gb300/angelo_gb``) never imports, links or calls anything here.

* ``oracle.c`` / ``cref.py``: float32 C restatement of tcnn HashGrid and
  SphericalHarmonics and of nerfacc 0.3.3 ray marching, occupancy threshold and
  transmittance (bit-exact integer outputs).
* ``neus_fp64.py``: FP64 differentiable PyTorch restatement of the whole path
  (hash grid, VanillaMLP, VolumeSDF finite differences and curvature, textures,
  get_alpha, weights, accumulation) -- the gradient reference.
* ``ref_harness.py``: runs the reference's own model code on the CPU with the
  restatements standing in for tinycudann / nerfacc; only the golden-vector
  generator uses it.
"""
