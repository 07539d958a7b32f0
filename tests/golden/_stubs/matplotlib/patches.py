"""Empty stand-in for matplotlib.patches (fixture generation only)."""


class Rectangle:  # noqa: D101
    pass
