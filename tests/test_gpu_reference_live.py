"""The reference's own objects drive the GB300 backend live.

``tests/reference_live.py`` runs in a child process with the reference
quantumsim package first on the path (``$QUANTUMSIM_REF``, or
``../reference`` beside the checkout, or an installed copy in
``baseline/_ref``), so that PauliVectorGB300 subclasses the reference's
PauliVectorBase exactly as it does for a quantumsim user, and compares
``FinalizedCircuit @ State``, State's trace / partial_trace / exp_value,
``Operation.from_kraus`` units on every qudit and ordered pair, and a chain
compiled into reduced bases, between PauliVectorGB300 and the reference's
PauliVectorNumpy.  Skipped where no reference package is present.
"""
import os
import subprocess
import sys

import pytest

from conftest import ROOT
from oracle.refsrc import reference_tree

pytestmark = pytest.mark.gpu


def test_reference_call_path_on_gb300_matches_numpy_backend():
    ref = reference_tree()
    if ref is None:
        pytest.skip('no reference quantumsim package ($QUANTUMSIM_REF, '
                    '../reference or baseline/_ref)')
    stubs = os.path.join(ROOT, 'tests', 'golden', '_stubs')
    env = dict(os.environ)
    env['PYTHONPATH'] = os.pathsep.join(
        [stubs, ref, ROOT] + ([env['PYTHONPATH']] if env.get('PYTHONPATH')
                              else []))
    run = subprocess.run(
        [sys.executable, os.path.join(ROOT, 'tests', 'reference_live.py')],
        env=env, capture_output=True, text=True, timeout=900)
    assert run.returncode == 0, run.stdout[-4000:] + run.stderr[-4000:]
    assert 'all scenarios agree' in run.stdout
