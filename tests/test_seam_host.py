"""The library seam (angelo_gb.seam) on the host: the stand-in modules carry
every name the reference imports from tinycudann and nerfacc
(models/network_utils.py:6,47,91,182,210, models/utils.py:11,120,
models/neus.py:11-12, models/geometry.py:15); and, when the reference's
source tree is given (INSTANT_ANGELO_SRC), its unmodified model code builds
NeuSModel on the seam with the parameter names and shapes of the golden
vectors (construction only: computing needs the GPU)."""
import os
import sys

import pytest

REFERENCE_NAMES = {
    "tinycudann": ("Encoding", "Network", "NetworkWithInputEncoding", "free_temporary_memory"),
    "nerfacc": ("ContractionType", "OccupancyGrid", "ray_marching", "render_weight_from_density",
                "render_weight_from_alpha", "accumulate_along_rays"),
    "nerfacc.intersection": ("ray_aabb_intersect",),
}


def test_seam_exports_the_reference_imports():
    from angelo_gb import seam
    mods = seam.modules()
    for name, attrs in REFERENCE_NAMES.items():
        for a in attrs:
            assert hasattr(mods[name], a), (name, a)
    assert mods["nerfacc"].intersection is mods["nerfacc.intersection"]
    ct = mods["nerfacc"].ContractionType
    assert {c.name for c in ct} >= {"AABB", "UN_BOUNDED_SPHERE"}


@pytest.mark.skipif(not os.environ.get("INSTANT_ANGELO_SRC"),
                    reason="set INSTANT_ANGELO_SRC to the reference's source tree")
def test_reference_model_builds_on_the_seam():
    import torch
    from angelo_gb import build, seam
    from golden_util import load
    from oracle import ref_harness
    build.build()
    saved = {k: v for k, v in sys.modules.items()
             if k.split(".")[0] in ("models", "systems", "utils", "tinycudann", "nerfacc")}
    try:
        models = ref_harness.install(os.environ["INSTANT_ANGELO_SRC"], seam.modules())
        from golden.make_golden import model_config
        g = load("neus_dual_grid")
        m = models.make("neus", model_config(g["cfg"]))
        names = {k: tuple(v.shape) for k, v in m.state_dict().items()}
        for k in g:
            if k.startswith("param/"):
                assert names[k[len("param/"):]] == g[k].shape, k
        assert type(m.geometry.encoding.encoding.encoding).__module__ == "angelo_gb.seam"
        assert isinstance(m.occupancy_grid, seam.OccupancyGrid)
    finally:
        for k in [k for k in sys.modules if k.split(".")[0] in
                  ("models", "systems", "utils", "tinycudann", "nerfacc")]:
            del sys.modules[k]
        sys.modules.update(saved)
