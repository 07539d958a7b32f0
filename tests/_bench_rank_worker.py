"""Worker for test_bench_ranks: one rank of a gloo job on CPU that runs the
multi-rank pieces of bench.py (rank environment, max over ranks, whole-job
rate, the reference arm's rank-0-only rule) and writes its results to
$QSGB_RANK_OUT/<rank>.json."""
import io
import json
import os
import sys
from contextlib import redirect_stdout

import torch.distributed as dist

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

world, rank, local = bench._dist()
dist.init_process_group('gloo')
# every rank times something different; all must agree on the slowest
ms = bench.max_over_ranks(10.0 + 5.0 * rank, 'cpu', world)
rate = bench.whole_job_rate(70, world, ms / 1e3)
# the reference arm: ranks other than 0 return without work or output
out = io.StringIO()
if rank != 0:
    with redirect_stdout(out):
        bench.run_reference(None)
dist.barrier()
dist.destroy_process_group()
with open(os.path.join(os.environ['QSGB_RANK_OUT'], '%d.json' % rank),
          'w') as f:
    json.dump({'rank': rank, 'world': world, 'local': local, 'ms': ms,
               'rate': rate, 'reference_output': out.getvalue()}, f)
