"""Oracles of the density-matrix hot path (test infrastructure only).

``oracle/pauli_vector_np.py``: the CPU oracle.  ``oracle/ref_gpu.py``: the
reference's own CUDA kernel, compiled from the reference source tree by
``oracle/build_ref.py``.  Imported by ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline and reference legs; never by the
``quantumsim_gb300`` package.
"""
