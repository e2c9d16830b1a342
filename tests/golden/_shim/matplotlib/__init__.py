"""Headless stand-in for matplotlib (test infrastructure: lets the reference import)."""
__version__ = "0.0"
