"""angelo_gb: GB300-native (sm_103a) kernels for the NeuS / Neuralangelo hot
path of Instant-angelo, behind drop-ins of the reference's entry points.

    from angelo_gb import models
    model = models.make('neus', config)      # config: the reference's model keys

The compute path is libangelo_gb.so (C ABI in include/angelo_gb.h), built by
``python -m angelo_gb.build``; there is no CPU or third-party fallback."""
from . import _lib  # noqa: F401
from . import models  # noqa: F401
from .config import Config, to_config  # noqa: F401

__all__ = ["models", "Config", "to_config", "load_library"]


def load_library():
    """Load libangelo_gb.so (raises if it has not been built)."""
    return _lib.load()
