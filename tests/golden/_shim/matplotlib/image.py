"""Headless stand-in for matplotlib.image."""


def imsave(*args, **kwargs):
    raise RuntimeError("matplotlib is not available in this environment")
