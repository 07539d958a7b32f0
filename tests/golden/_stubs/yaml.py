"""Minimal stand-in for ``yaml`` (fixture generation only; never parses)."""


def safe_load(stream):
    raise NotImplementedError("yaml is not available in this environment")
