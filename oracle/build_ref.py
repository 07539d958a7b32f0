"""Recipe: compile the reference's CUDA kernels
(quantumsim/pauli_vectors/primitives.cu, included unchanged from the
reference source tree by oracle/ref_primitives.cu) into
oracle/_ref/primitives_sm103a.cubin for sm_103a.

Runs only where the reference tree is present (``oracle.refsrc``:
$QUANTUMSIM_REF, or ``../reference`` beside the checkout); elsewhere the
previously built cubin (if any) is used as it is.  Test and reference-arm infrastructure; the product never loads it.
"""
import os
import subprocess
import sys

if __package__:
    from . import refsrc
else:  # run as a script
    import refsrc

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, '_ref', 'primitives_sm103a.cubin')


def build(verbose=False):
    ref = refsrc.source_tree()
    if ref is None:
        return os.path.exists(OUT)
    src = os.path.join(ref, 'quantumsim', 'pauli_vectors', 'primitives.cu')
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = ['nvcc', '-cubin', '-gencode', 'arch=compute_103a,code=sm_103a',
           '-O3', '-DQSGB_REF_PRIMITIVES="{}"'.format(src),
           os.path.join(HERE, 'ref_primitives.cu'), '-o', OUT]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        if verbose:
            print(r.stderr, file=sys.stderr)
        return False
    return True


if __name__ == '__main__':
    print('built' if build(verbose=True) else 'not built', OUT)
