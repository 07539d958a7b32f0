"""The N > 1 path of bench.py on CPU: two gloo ranks launched by torchrun
(127.0.0.1 rendezvous) agree on the slowest rank's time, report the
whole-job rate, and only rank 0 of the reference arm does any work."""
import json
import os
import socket
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_max_over_ranks_and_rank0_reference(tmp_path):
    cmd = [sys.executable, '-m', 'torch.distributed.run', '--nnodes=1',
           '--nproc-per-node', '2', '--master-addr', '127.0.0.1',
           '--master-port', str(_free_port()),
           os.path.join(HERE, '_bench_rank_worker.py')]
    env = dict(os.environ, OMP_NUM_THREADS='1', QSGB_RANK_OUT=str(tmp_path))
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300,
                       env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [json.loads((tmp_path / ('%d.json' % k)).read_text())
             for k in range(2)]
    assert sorted(d['rank'] for d in lines) == [0, 1]
    for d in lines:
        assert d['world'] == 2 and d['local'] == d['rank']
        assert d['ms'] == 15.0                      # max of 10 and 15
        assert abs(d['rate'] - 70 * 2 / 0.015) < 1e-6
        if d['rank'] == 1:
            assert d['reference_output'] == ''
