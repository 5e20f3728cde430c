"""Name registry of the drop-in modules (models/__init__.py:1-16): 'neus',
'volume-sdf', 'volume-radiance', 'volume-dual-color', 'volume-dual-colorV3'."""
models = {}


def register(name):
    def decorator(cls):
        models[name] = cls
        return cls
    return decorator


def make(name, config):
    # importing the modules registers their classes
    from . import geometry, neus, texture  # noqa: F401
    return models[name](config)
