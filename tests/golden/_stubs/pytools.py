"""Minimal stand-in for the two ``pytools`` helpers quantumsim imports.

Used only when importing the reference package in the development
container to generate golden fixtures; never shipped or imported by the
product.
"""
import itertools
import math


def product(iterable):
    return math.prod(iterable)


def flatten(iterable):
    return itertools.chain.from_iterable(iterable)
