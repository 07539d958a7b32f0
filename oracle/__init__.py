"""CPU oracle of the density-matrix hot path (test infrastructure only).

See ``oracle/pauli_vector_np.py``.  Imported by ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg; never by the
``quantumsim_gb300`` package.
"""
