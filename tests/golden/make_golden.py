"""Generate the golden fixtures of the density-matrix hot path.

Runs the REFERENCE implementation (quantumsim's ``PauliVectorNumpy`` and its
gate library) on seeded inputs and stores inputs and outputs in
``tests/golden/pauli_vector_golden.npz``.  It needs the reference source tree
(``$QUANTUMSIM_REF``, or ``../reference`` beside the checkout) and the stand-in
modules in ``tests/golden/_stubs`` for quantumsim's optional imports
(pytools, more_itertools, yaml, matplotlib).  The fixtures it writes are
self-contained: tests read them without the reference.

Usage:  python tests/golden/make_golden.py
"""
import json
import math
import os
import sys
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle.refsrc import reference_tree  # noqa: E402
REF = reference_tree()
if REF is None:
    sys.exit('reference source tree not found: set $QUANTUMSIM_REF')
sys.path[:0] = [os.path.join(HERE, '_stubs'), REF]
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
warnings.simplefilter('ignore')

import quantumsim.bases as qb  # noqa: E402
from quantumsim.algebra import kraus_to_ptm  # noqa: E402
from quantumsim.operations import qubits as lib2  # noqa: E402
from quantumsim.operations import qutrits as lib3  # noqa: E402
from quantumsim.operations.operation import Operation  # noqa: E402
from quantumsim.pauli_vectors.numpy import PauliVectorNumpy  # noqa: E402
from scipy.stats import unitary_group  # noqa: E402

from quantumsim_gb300 import workloads  # noqa: E402
from quantumsim_gb300.ptm import kraus_to_ptm as gb_kraus_to_ptm  # noqa: E402

OUT = os.path.join(HERE, 'pauli_vector_golden.npz')

arrays = {}
cases = []
basis_table = []  # list of (key) -> index
basis_index = {}


def basis_id(b):
    key = (b.vectors.shape, np.ascontiguousarray(b.vectors).tobytes())
    if key not in basis_index:
        i = len(basis_table)
        basis_index[key] = i
        basis_table.append(i)
        arrays['basis{}_vectors'.format(i)] = np.asarray(b.vectors)
        arrays['basis{}_labels'.format(i)] = np.array(
            [str(x) for x in b.labels])
    return basis_index[key]


def add(kind, bases, pv_in, out, **meta):
    i = len(cases)
    arrays['c{}_in'.format(i)] = np.asarray(pv_in)
    if isinstance(out, dict):
        for k, v in out.items():
            arrays['c{}_{}'.format(i, k)] = np.asarray(v)
        outs = sorted(out)
    else:
        arrays['c{}_out'.format(i)] = np.asarray(out)
        outs = ['out']
    meta = dict(meta)
    if 'ptm' in meta:
        arrays['c{}_ptm'.format(i)] = np.asarray(meta.pop('ptm'))
        meta['has_ptm'] = True
    cases.append(dict(kind=kind, bases=[basis_id(b) for b in bases],
                      outs=outs, **meta))


def random_pv(rng, bases):
    dim = math.prod(b.dim_hilbert for b in bases)
    a = rng.standard_normal((dim, dim)) + 1j * rng.standard_normal((dim, dim))
    dm = a @ a.conj().T
    dm /= np.trace(dm)
    # expand in the product basis (mixed dimensions allowed):
    # pv[x...] = Re tr(dm (P_x0 (x) P_x1 ...))
    dims = [b.dim_hilbert for b in bases]
    n = len(bases)
    args = [dm.reshape(dims + dims), list(range(2 * n))]
    for i, b in enumerate(bases):
        args += [b.vectors, [2 * n + i, n + i, i]]
    return np.einsum(*args, optimize=True).real.copy()


def random_kraus(rng, dim, n=2):
    ks = [unitary_group.rvs(dim, random_state=rng) for _ in range(n)]
    decay = np.diag(rng.uniform(0.6, 1.0, dim))
    return np.array([decay @ ks[0] / math.sqrt(n)] +
                    [k / math.sqrt(n) for k in ks[1:]])


def main():
    rng = np.random.RandomState(20240611)
    g2, g3 = qb.general(2), qb.general(3)
    resh = qb.PauliBasis(np.array([g2.vectors[i] for i in (0, 2, 1, 3)]),
                         [g2.labels[i] for i in (0, 2, 1, 3)])

    # -- 1q PTMs on every position, square and rectangular
    bases = [g2] * 5
    for q in range(5):
        pv = random_pv(rng, bases)
        ptm = kraus_to_ptm(random_kraus(rng, 2), (g2,), (g2,))
        ref = PauliVectorNumpy(bases, pv.copy())
        ref.apply_ptm(ptm, q)
        add('apply', bases, pv, ref.to_pv(), qubits=[q], ptm=ptm)
    for q, sub in ((1, [0, 1, 2]), (4, [0]), (0, [0, 1])):
        pv = random_pv(rng, bases)
        ptm = kraus_to_ptm(random_kraus(rng, 2), (g2,), (g2.subbasis(sub),))
        ref = PauliVectorNumpy(bases, pv.copy())
        ref.apply_ptm(ptm, q)
        add('apply', bases, pv, ref.to_pv(), qubits=[q], ptm=ptm)

    # -- 2q PTMs on all ordered pairs of 4 qubits
    bases = [g2] * 4
    for q0 in range(4):
        for q1 in range(4):
            if q0 == q1:
                continue
            pv = random_pv(rng, bases)
            ptm = kraus_to_ptm(random_kraus(rng, 4), (g2, g2), (g2, g2))
            ref = PauliVectorNumpy(bases, pv.copy())
            ref.apply_ptm(ptm, q0, q1)
            add('apply', bases, pv, ref.to_pv(), qubits=[q0, q1], ptm=ptm)

    # -- mixed dimensions and reduced bases
    mixed = [g3, g2, g3]
    for qs in ((0,), (1,), (2,), (0, 2), (2, 0), (1, 2), (0, 1)):
        pv = random_pv(rng, mixed)
        bs = tuple(mixed[q] for q in qs)
        dim = math.prod(b.dim_hilbert for b in bs)
        # mixed qutrit-qubit PTMs: the reference kraus_to_ptm assumes one
        # Hilbert dimension, so build the (input) PTM with the package's
        ptm = gb_kraus_to_ptm(random_kraus(rng, dim), bs, bs).numpy()
        ref = PauliVectorNumpy(mixed, pv.copy())
        ref.apply_ptm(ptm, *qs)
        add('apply', mixed, pv, ref.to_pv(), qubits=list(qs), ptm=ptm)
    sub_bases = [g2.subbasis([0, 1, 2]), g2.subbasis([0, 1]), g2]
    for qs, bout in (((0, 2), (g2, g2.subbasis([0, 1]))),
                     ((2, 1), (g2.subbasis([0, 3]), g2))):
        pv = random_pv(rng, [g2] * 3)
        pv = pv[tuple(slice(0, b.dim_pauli) for b in sub_bases)].copy()
        bin_ = tuple(sub_bases[q] for q in qs)
        ptm = kraus_to_ptm(random_kraus(rng, 4), bin_, bout)
        ref = PauliVectorNumpy(sub_bases, pv.copy())
        ref.apply_ptm(ptm, *qs)
        add('apply', sub_bases, pv, ref.to_pv(), qubits=list(qs), ptm=ptm)

    # -- diagonal / trace / meas_prob / renormalize on several bases
    for bases in ([g2] * 4, [resh] * 3, [g3, g2, g3],
                  [g2.subbasis([0, 1]), g2.subbasis([0, 1, 2]), g2],
                  [qb.gell_mann(2)] * 3, [qb.gell_mann(3), g2]):
        pv = random_pv(rng, bases) * 0.7
        ref = PauliVectorNumpy(bases, pv.copy())
        outs = dict(diag=ref.diagonal(), trace=np.array(ref.trace()))
        for q in range(len(bases)):
            outs['prob{}'.format(q)] = ref.meas_prob(q)
        ref2 = PauliVectorNumpy(bases, pv.copy())
        outs['renorm_trace'] = np.array(ref2.renormalize())
        outs['renorm_pv'] = ref2.to_pv()
        add('reduce', bases, pv, outs)

    # -- partial trace
    for bases, keeps in (([g2] * 5, [(0,), (1, 3), (0, 2, 4), (4,)]),
                         ([g3, g2, g3], [(0,), (1, 2), (0, 2)]),
                         ([qb.gell_mann(2)] * 3, [(1,), (0, 2)])):
        pv = random_pv(rng, bases)
        for keep in keeps:
            ref = PauliVectorNumpy(bases, pv.copy())
            pt = ref.partial_trace(*keep)
            add('partial_trace', bases, pv, pt.to_pv(), keep=list(keep))

    # -- basis reduction / projection (selection PTM, qutrits)
    bases = [g3] * 3
    comp = [int(g3.computational_basis_indices[i]) for i in range(3)]
    for q, idx in ((0, comp), (2, comp), (1, [comp[1]]), (1, [0, 3, 4])):
        pv = random_pv(rng, bases)
        ref = PauliVectorNumpy(bases, pv.copy())
        ref.apply_ptm(np.eye(9)[idx], q)
        add('reduce_basis', bases, pv, ref.to_pv(), qubit=q, indices=idx)

    # -- gate PTMs of the reference library (pins quantumsim_gb300.ptm)
    b1, b1_3 = (g2,), (g3,)
    gates = {
        'rx_0.7': lib2.rotate_x(0.7).ptm(b1),
        'ry_2.1': lib2.rotate_y(2.1).ptm(b1),
        'rz_-1.3': lib2.rotate_z(-1.3).ptm(b1),
        'apd_0.01_0.03': lib2.amp_phase_damping(0.01, 0.03).ptm(b1),
        'cz_3.0': lib2.cphase(3.0).ptm(b1 * 2),
        'noisy_cz': Operation.from_sequence(
            lib2.cphase(math.pi).at(0, 1),
            lib2.amp_phase_damping(0.002, 0.003).at(0),
            lib2.amp_phase_damping(0.001, 0.004).at(1)).ptm(b1 * 2),
        'q3_rx_0.7': lib3.rotate_x(0.7).ptm(b1_3),
        'q3_ry_1.9': lib3.rotate_y(1.9).ptm(b1_3),
        'q3_damp': lib3.amp_damping(0.01, 0.002, 0.03, 0.04).ptm(b1_3),
        'q3_cz': lib3.cphase(math.pi + 0.013, leakage_rate=0.004).ptm(b1_3 * 2),
    }
    for k, v in gates.items():
        arrays['gate_' + k] = v

    # -- 6-qubit circuit (20 layers): the CPU-runnable configuration, PTMs
    #    from workloads.config0_circuit, run through the reference backend
    ops = workloads.config0_circuit(seed=0)
    ref = PauliVectorNumpy([g2] * 6)
    for _, ptm, qs in ops:
        ref.apply_ptm(ptm, *qs)
    arrays['circuit0_pv'] = ref.to_pv()
    arrays['circuit0_diag'] = ref.diagonal()
    arrays['circuit0_nops'] = np.array(len(ops))

    arrays['manifest'] = np.array(json.dumps(cases))
    np.savez_compressed(OUT, **arrays)
    print('wrote {} ({} cases, {} bytes)'.format(OUT, len(cases),
                                                 os.path.getsize(OUT)))


if __name__ == '__main__':
    main()
