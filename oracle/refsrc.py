"""Where the reference quantumsim source tree is, for the recipes and tests
that read it (fixture generators, the reference-kernel build, the live
reference-object tests).  Test infrastructure only.

The tree is the directory that holds the ``quantumsim`` package.  It is taken
from ``$QUANTUMSIM_REF`` when that is set; otherwise from the first of
``../reference`` (beside the repository checkout) and ``baseline/_ref`` (an
installed copy inside the repository) that holds ``quantumsim``.  None when
there is no tree, in which case callers skip or keep what they built before.
"""
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_tree():
    env = os.environ.get('QUANTUMSIM_REF')
    cands = [env] if env else [os.path.join(os.path.dirname(ROOT), 'reference'),
                               os.path.join(ROOT, 'baseline', '_ref')]
    for c in cands:
        if c and os.path.isdir(os.path.join(c, 'quantumsim')):
            return os.path.abspath(c)
    return None


def source_tree():
    """Like reference_tree(), but only a tree that still carries the
    reference's CUDA source (``quantumsim/pauli_vectors/primitives.cu``), as
    the reference-kernel build needs."""
    t = reference_tree()
    if t and os.path.exists(os.path.join(t, 'quantumsim', 'pauli_vectors',
                                         'primitives.cu')):
        return t
    return None
