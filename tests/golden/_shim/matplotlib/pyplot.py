"""Headless stand-in: the reference imports pyplot at module level only."""


def __getattr__(name):
    raise RuntimeError("matplotlib is not available in this environment")
