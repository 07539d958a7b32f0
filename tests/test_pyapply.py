"""The CPython entry point of the per-call apply path
(quantumsim_gb300/csrc/qsgb_pyapply.c), on the build host (no GPU): it
builds with the host C compiler, and it refuses malformed arguments and
missing entry points with Python exceptions instead of calling the
library."""
import importlib

import pytest

from quantumsim_gb300 import build as qbuild


@pytest.fixture(scope='module')
def mod():
    path = qbuild.build_pyapply()
    if path is None:
        pytest.skip('no C compiler or Python headers on this host')
    return importlib.import_module('quantumsim_gb300._qsgb_pyapply')


def test_argument_checks(mod):
    with pytest.raises(TypeError):
        mod.apply(1, 2, 3)
    with pytest.raises(ValueError):
        mod.set_entry_points(0, 0, len, len, len, len)
    with pytest.raises(ValueError):
        mod.set_entry_points(1, 1, None, len, len, len)


def test_plan_shape_is_checked_before_any_call(mod):
    # entry points that must never be reached: the plan is rejected first
    mod.set_entry_points(1, 1, len, len, len, len)
    try:
        with pytest.raises(TypeError):
            mod.apply(object(), b'', (1, 2), 0)
        with pytest.raises(TypeError):
            mod.apply(object(), b'', ((4,), False, (1, 2, 3), 4, 0), 0)
    finally:
        # leave no dangling addresses for a later GPU test in this process
        import quantumsim_gb300.ops as ops
        ops._PYAPPLY = None


def test_optional_output_argument(mod):
    """apply takes an optional fifth argument (the output tensor, or None);
    more arguments are refused before anything is called."""
    mod.set_entry_points(1, 1, len, len, len, len)
    try:
        with pytest.raises(TypeError):
            mod.apply(1, 2, 3, 4, None, 6)
        with pytest.raises(TypeError):
            mod.apply(object(), b'', (1, 2), 0, None)
    finally:
        import quantumsim_gb300.ops as ops
        ops._PYAPPLY = None
