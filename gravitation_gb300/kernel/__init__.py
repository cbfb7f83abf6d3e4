"""Kernel packages for the gravitation plugin API (see gb1)."""
