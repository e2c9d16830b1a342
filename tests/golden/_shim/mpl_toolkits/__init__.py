"""Headless stand-in (test infrastructure)."""
