"""Operators of the VlaPy time step on the GB300 (mirror of vlapy/core)."""
