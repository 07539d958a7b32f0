"""Minimal stand-in for ``more_itertools.pairwise`` (fixture generation only)."""
import itertools


def pairwise(iterable):
    return itertools.pairwise(iterable)
