"""Configuration objects accepted by the drop-in modules.

The reference passes OmegaConf DictConfigs (utils/misc.py:26-35) and reads them
both as attributes (``config.radius``) and as mappings (``config['n_neurons']``,
``config.get('include_xyz')``).  ``Config`` supports exactly those forms, so the
reference's YAML files, loaded by any YAML reader, or plain dicts work as-is.
"""
from __future__ import annotations

import copy


class Config(dict):
    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError as e:
            raise AttributeError(k) from e

    def __setattr__(self, k, v):
        self[k] = v

    def copy(self):
        return Config(copy.deepcopy(dict(self)))


def to_config(d):
    """Recursively wrap dicts (and objects exposing ``items()``) as Config."""
    if isinstance(d, Config):
        return d
    if hasattr(d, "items"):
        return Config({k: to_config(v) for k, v in d.items()})
    if isinstance(d, (list, tuple)):
        return [to_config(v) for v in d]
    return d


def to_primitive(d):
    if hasattr(d, "items"):
        return {k: to_primitive(v) for k, v in d.items()}
    if isinstance(d, (list, tuple)):
        return [to_primitive(v) for v in d]
    return d


def scheduled_value(value, global_step, current_epoch=0):
    """Scalar schedule of BaseSystem.C (systems/base.py:28-45):
    [start_step, start_value, end_value, end_step] (3 values imply start_step
    0), linear between the ends; an int end_step counts steps, a float one
    counts epochs."""
    if isinstance(value, (int, float)):
        return value
    value = list(value)
    if len(value) == 3:
        value = [0] + value
    assert len(value) == 4
    start_step, start_value, end_value, end_step = value
    cur = global_step if isinstance(end_step, int) else current_epoch
    frac = max(min(1.0, (cur - start_step) / (end_step - start_step)), 0.0)
    return start_value + (end_value - start_value) * frac
