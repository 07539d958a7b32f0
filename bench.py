"""Benchmark of the density-matrix hot path on GB300.

Workload (the 14-qubit FP64 configuration): a Pauli vector of 14 qubits in
the full ``general(2)`` basis (4^14 = 268,435,456 float64 entries, 2.15 GB)
on one GPU.  One step applies 7 noisy-CZ 16x16 PTMs (CZ followed by
amplitude + phase damping on both qubits, seeded T1/T2) on uniformly random
ordered qubit pairs, so every stride class occurs.  The vector (2.15 GB) is
larger than L2 (129 MB), so no flush is needed between steps.

Prints ONE JSON line (rank 0).  ``value`` = 2q-PTM applications per second
with the state resident in HBM; ``e2e`` = the same through the public API
(host numpy PTMs passed per call, the trace read back every step);
``roofline`` = the dominant kernel's algorithmic bytes per launch over its
CUDA-event duration against the measured HBM copy peak; ``cpu_baseline`` =
the oracle (numpy einsum restatement of the reference backend) on the host
cores for a bounded sample.

``batched`` = the batched configuration: 512 circuits of 4..12 qubits, depth
30, FP32 Pauli vectors with FP64 reductions, forward + adjoint of all of them
in one persistent launch (CUDA graph), against the plain GPU path run one
instance at a time, with the maximum probability error against FP64.

``--impl reference`` times the reference's CPU implementation of the path
(the oracle port of PauliVectorNumpy, all host threads) on the same
workload and prints the same line with ``"impl": "reference"``.

With ``--gpus N > 1`` (torchrun) every rank runs an independent replica
(the path is not sharded; no collective on the data path); value = all
ranks' applications / max rank time.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_QUBITS = 14
APPS_PER_STEP = 7
# DRAM bytes (read + write) of one 14-qubit noisy-CZ launch, scaled from an
# ncu capture of the same kernel on 13 qubits (536.9 MB read, 486.8 MB
# written per launch; reads scale 4x, writes 4x minus the ~50 MB still in L2
# at kernel end)
TRAFFIC_14Q = 4 * 536.9e6 + 4 * 536.9e6 - 50e6
METRIC = ('2q-PTM apps/s & HBM GB/s (14q fp64); batched fp32 fwd+adjoint vs '
          'plain, err<1e-6')
WORKLOAD = ('14-qubit FP64 Pauli vector (4^14 entries, 2.15 GB); step = 7 '
            'noisy-CZ 16x16 PTMs on uniformly random ordered qubit pairs')


def _peaks():
    path = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    except Exception:
        return 6800.0, 'fallback'


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    QUERY = ('index,clocks.sm,clocks.max.sm,power.draw,'
             'clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
             'clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,'
             'clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index),
                 '--query-gpu=' + self.QUERY, '--format=csv,noheader,nounits',
                 '-lms', '100'], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': [],
                    'samples': 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown',
                 'sw_power_cap']
        for line in self.lines:
            parts = [p.strip() for p in line.split(',')]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == 'active':
                    reasons.add(name)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {'sm_mhz': med, 'sm_max_mhz': smax, 'reasons': sorted(reasons),
                'samples': len(sm)}


def _dist():
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return world, rank, local


def max_over_ranks(x, device, world):
    """Maximum of the float x over all ranks (x itself on one rank)."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, seconds):
    """Units all ranks processed per second of the slowest rank (every
    replica does the same work: weak scaling)."""
    return units_per_rank * world / seconds


def cpu_baseline_sample(n_apps, seed=123):
    """Time the oracle (numpy einsum restatement of PauliVectorNumpy) on
    `n_apps` noisy-CZ applications of the 14-qubit workload."""
    import numpy as np
    from oracle import pauli_vector_np as O
    from quantumsim_gb300 import workloads
    rng = np.random.default_rng(seed)
    pv = rng.standard_normal((4,) * N_QUBITS) * 2.0 ** -14
    ops = workloads.config1_2q_batch(seed, N_QUBITS, n_apps + 1)
    pv = O.apply_ptm(pv, ops[0][1], *ops[0][2])  # warm-up
    t0 = time.perf_counter()
    for _, ptm, qs in ops[1:]:
        pv = O.apply_ptm(pv, ptm, *qs)
    dt = time.perf_counter() - t0
    return n_apps / dt, dt


def run_reference(args):
    world, rank, _ = _dist()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    vals = []
    for i in range(args.warmup + args.steps):
        v, _ = cpu_baseline_sample(1, seed=1000 + i)
        if i >= args.warmup:
            vals.append(v)
    value = len(vals) / sum(1.0 / v for v in vals)
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': value,
        'unit': 'apps/s', 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': 1000.0 / value,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f64', 'data': 'synthetic',
        'config': {'workload': WORKLOAD, 'n_qubits': N_QUBITS,
                   'sample': '1 noisy-CZ application per step'},
        'cpu_baseline': {'value': value, 'unit': 'apps/s', 'cores': cores,
                         'kind': 'port',
                         'sample': '1 application of the 14-qubit 2q '
                                   'workload per step (numpy einsum, '
                                   'OpenBLAS threads = cores)'},
        'e2e': {'value': value, 'unit': 'apps/s', 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': 0},
    }
    gk = reference_gpu_kernel(args)
    if gk is not None:
        line['gpu_kernel'] = gk
    print(json.dumps(line), flush=True)


def reference_gpu_kernel(args):
    """The reference's own CUDA kernel (primitives.cu two_qubit_general_ptm,
    compiled unchanged for sm_103a into oracle/_ref, launched with the
    geometry of quantumsim/pauli_vectors/cuda.py:151-221) on this arm's
    workload: the 14-qubit FP64 vector, steps of 7 noisy CZs on random
    ordered pairs, CUDA events around `steps` steps after `warmup`.  None
    when there is no GPU or the kernel was not built."""
    try:
        import torch
        from oracle import ref_gpu
    except Exception:
        return None
    if not torch.cuda.is_available() or not ref_gpu.available():
        return None
    import numpy as np
    from quantumsim_gb300 import workloads
    rng = np.random.default_rng(7)
    x = torch.from_numpy(rng.standard_normal((4,) * N_QUBITS) * 2.0 ** -14) \
        .cuda()
    n_steps = args.warmup + max(1, args.steps)
    steps = [workloads.config1_2q_batch(1000 + i, N_QUBITS, APPS_PER_STEP)
             for i in range(n_steps)]
    for i in range(args.warmup):
        for _, ptm, qs in steps[i]:
            x = ref_gpu.apply(x, ptm, qs)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(args.warmup, n_steps):
        for _, ptm, qs in steps[i]:
            x = ref_gpu.apply(x, ptm, qs)
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    apps = (n_steps - args.warmup) * APPS_PER_STEP
    return {'value': apps / sec, 'unit': 'apps/s',
            'gbs': apps * 2 * 4 ** N_QUBITS * 8 / sec / 1e9,
            'kernel': 'two_qubit_general_ptm (quantumsim primitives.cu, '
                      'compiled unchanged for sm_103a, PyCUDA launch '
                      'geometry); PTMs uploaded on first use and cached by '
                      'content, as the reference does'}


def run_gb300(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    world, rank, local = _dist()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group('nccl')
    from quantumsim_gb300 import build as qbuild
    qbuild.build()
    import quantumsim_gb300 as qg
    from quantumsim_gb300 import bases, workloads, ops as qops

    dev = torch.device('cuda', local)
    n_entries = 4 ** N_QUBITS
    s = qg.PauliVectorGB300([bases.general(2)] * N_QUBITS, force=True,
                            device=dev)
    # a generic mixed state: one layer of the circuit (rotations + CZs)
    rng = np.random.default_rng(7 + rank)
    t1, t2 = workloads.coherence_times(rng, N_QUBITS)
    for op in workloads.config1_layer(rng, N_QUBITS, t1, t2, 7):
        s.apply_ptm(op[1], *op[2])
    torch.cuda.synchronize()

    n_steps = args.warmup + args.steps
    steps = [workloads.config1_2q_batch(1000 * rank + i, N_QUBITS,
                                        APPS_PER_STEP) for i in range(n_steps)]
    stream = torch.cuda.current_stream(dev)

    def step(ops_):
        for _, ptm, qs in ops_:
            s.apply_ptm(ptm, *qs)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-resident timing (value)
    for i in range(args.warmup):
        step(steps[i])
    sampler = ClockSampler(local)
    barrier()
    sampler.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(args.warmup, n_steps):
        step(steps[i])
    e1.record(stream)
    barrier()
    clocks = sampler.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), dev, world)
    apps = args.steps * APPS_PER_STEP
    value = whole_job_rate(apps, world, ms / 1e3)
    bytes_per_app = 2 * n_entries * 8

    # ---- per-launch durations of the dominant kernel (same stream)
    per = []
    probe = steps[args.warmup] if args.steps else steps[0]
    for _, ptm, qs in probe * 2:
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        s.apply_ptm(ptm, *qs)
        b.record(stream)
        per.append((a, b))
    torch.cuda.synchronize()
    launch_ms = sum(a.elapsed_time(b) for a, b in per) / len(per)
    peak, peak_kind = _peaks()
    achieved = bytes_per_app / (launch_ms / 1e3) / 1e9
    traffic = args.traffic if args.traffic else TRAFFIC_14Q

    # ---- per-target breakdown (1q positions, 2q stride classes)
    per_target = {}
    if not args.no_sweep:
        for q in range(N_QUBITS):
            ptm = workloads.noisy_1q(rng, t1[q], t2[q])
            per_target['1q_q{}'.format(q)] = _time_app(s, ptm, (q,),
                                                       bytes_per_app)
        for pair in [(0, 1), (12, 13), (0, 13), (13, 0), (3, 7), (6, 7),
                     (1, 12)]:
            ptm = workloads.noisy_cz(rng, pair, t1, t2)
            per_target['2q_{}_{}'.format(*pair)] = _time_app(
                s, ptm, pair, bytes_per_app)
        dense = rng.standard_normal((4, 4, 4, 4)) * 0.25
        per_target['2q_dense_3_7'] = _time_app(s, dense, (3, 7), bytes_per_app)
        per_target['2q_dense_12_13'] = _time_app(s, dense, (12, 13),
                                                 bytes_per_app)
        # the same launches with each arithmetic forced
        cz = workloads.noisy_cz(rng, (3, 7), t1, t2)
        r1 = workloads.noisy_1q(rng, t1[5], t2[5])
        for pair in [(0, 1), (12, 13), (13, 0), (6, 11)]:
            per_target['2q_dense_{}_{}'.format(*pair)] = _time_app(
                s, dense, pair, bytes_per_app)
        for arith in ('f64', 'df64', 'auto', 'tc'):
            s._arith_key, s._arith = arith, qops_arith(arith)
            per_target['arith_{}_2q_cz_3_7'.format(arith)] = _time_app(
                s, cz, (3, 7), bytes_per_app)
            per_target['arith_{}_1q_q5'.format(arith)] = _time_app(
                s, r1, (5,), bytes_per_app)
            per_target['arith_{}_2q_dense_3_7'.format(arith)] = _time_app(
                s, dense, (3, 7), bytes_per_app)
        s._arith_key, s._arith = 'auto', qops_arith('auto')
        # FP32 storage (FP32 arithmetic): half the bytes per application
        s32 = qg.PauliVectorGB300([bases.general(2)] * N_QUBITS, force=True,
                                  dtype=np.float32, device=dev)
        s32._data.copy_(s._data.float())
        b32 = bytes_per_app // 2
        per_target['f32_2q_cz_3_7'] = _time_app(s32, cz, (3, 7), b32)
        per_target['f32_2q_cz_12_13'] = _time_app(s32, cz, (12, 13), b32)
        per_target['f32_1q_q5'] = _time_app(s32, r1, (5,), b32)
        per_target['f32_1q_q13'] = _time_app(s32, r1, (13,), b32)
        per_target['f32_2q_dense_3_7'] = _time_app(s32, dense, (3, 7), b32)
        del s32

    # ---- end to end through the public API (host PTMs, trace read back)
    e2e_steps = [workloads.config1_2q_batch(50000 + 1000 * rank + i,
                                            N_QUBITS, APPS_PER_STEP)
                 for i in range(n_steps)]
    for i in range(args.warmup):
        step(e2e_steps[i])
        s.trace()
    barrier()
    t0 = time.perf_counter()
    for i in range(args.warmup, n_steps):
        step(e2e_steps[i])
        s.trace()
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dev, world)
    e2e_value = whole_job_rate(apps, world, e2e_s)
    h2d = APPS_PER_STEP * 16 * 16 * 8
    qops.check_device_status(dev)

    # ---- batched FP32 forward + adjoint vs the plain path (rank 0, N = 1)
    batched = None
    if rank == 0 and world == 1 and not args.no_batched:
        from quantumsim_gb300 import batch as qbatch
        batched = qbatch.benchmark(n_instances=args.batch_instances,
                                   f64_check='all',
                                   plain_all=args.plain_all)
        # whole step (forward + adjoint of every circuit) against HBM;
        # instances of up to 10 qubits largely live in L2
        batched['hbm_frac'] = batched['achieved_gbs'] / peak

    extra = {}
    if rank == 0 and world == 1 and not args.no_configs:
        extra['qutrit_8q'] = run_qutrit_config()
        extra['grad_10q'] = run_grad_config()
        extra.update(run_circuit_configs())
        extra['ops'] = run_ops_config()

    # ---- CPU baseline (rank 0, N = 1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, dt = cpu_baseline_sample(args.cpu_apps)
        cpu = {'value': v, 'unit': 'apps/s', 'cores': os.cpu_count(),
               'kind': 'port',
               'sample': '{} noisy-CZ applications on the 14-qubit state '
                         '({:.1f} s; numpy einsum restatement of '
                         'PauliVectorNumpy)'.format(args.cpu_apps, dt)}

    if rank == 0:
        line = {
            'metric': METRIC, 'value': value, 'unit': 'apps/s',
            'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': ms / args.steps, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'arith': 'per PTM row: native FP64 FMA or float-float (48-bit '
                     'significand) on the FP32 pipes, chosen by a pipe cost '
                     'model; kernel specialised to the PTM sparsity pattern '
                     'at run time (NVRTC, cached)',
            'data': 'synthetic',
            'config': {'workload': WORKLOAD, 'n_qubits': N_QUBITS,
                       'entries': n_entries, 'apps_per_step': APPS_PER_STEP,
                       'l2': 'inputs (2.15 GB) larger than L2, no flush',
                       'parallelism': 'replicas' if world > 1 else 'single'},
            'hbm_gbs': bytes_per_app * apps / (ms / 1e3) / 1e9,
            'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': peak,
                         'unit': 'GB/s', 'frac': achieved / peak,
                         'peak_kind': peak_kind, 'traffic': traffic,
                         'kernel': 'qsgb_jit (apply kernel specialised to '
                                   'the noisy-CZ sparsity pattern, 2q)',
                         'bytes_per_launch': bytes_per_app,
                         'launch_ms': launch_ms},
            'cpu_baseline': cpu,
            'e2e': {'value': e2e_value, 'unit': 'apps/s',
                    'h2d_bytes_per_step': h2d, 'd2h_bytes_per_step': 8},
            'gpu_launches': apps,
            'clocks': clocks,
            'per_target_gbs': per_target,
            'batched': batched,
            'configs': extra,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_qutrit_config():
    """8 qutrits (9^8 float64 entries, 344 MB): the 30-layer leakage
    circuit with the mid-circuit basis reduction, projection and
    renormalisation; plus per-application GB/s of the 9x9 and 81x81 PTMs."""
    import numpy as np
    import torch
    import quantumsim_gb300 as qg
    from quantumsim_gb300 import bases, workloads
    ops = workloads.config2_circuit(seed=2)
    n_ptm = sum(1 for op in ops if op[0] == 'ptm')
    for rep in range(2):  # the first pass compiles the PTM patterns
        s = qg.PauliVectorGB300([bases.general(3)] * 8, force=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        traces = workloads.run(s, ops)
        tr = s.trace()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
    x_unfused = s.to_pv()
    rng = np.random.default_rng(5)
    s = qg.PauliVectorGB300([bases.general(3)] * 8, force=True)
    nbytes = 2 * 9 ** 8 * 8
    res = {'workload': '8 qutrits, 30 layers (9x9 and 81x81 PTMs), '
                       'reduce+project 2 qutrits mid-circuit',
           'circuit_s': dt, 'ptm_apps': n_ptm, 'apps_per_s': n_ptm / dt,
           'renorm_trace': traces[0] if traces else None,
           'final_trace': tr}
    # the same circuit with the PTM runs between the basis reductions fused
    from quantumsim_gb300 import circuit as qc
    segments, seg = [], []
    for op in ops:
        if op[0] == 'ptm':
            seg.append((op[1], op[2]))
        else:
            if seg:
                segments.append(qc.FusedCircuit(seg))
                seg = []
            segments.append(op)
    if seg:
        segments.append(qc.FusedCircuit(seg))
    for rep in range(2):
        s = qg.PauliVectorGB300([bases.general(3)] * 8, force=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for item in segments:
            if isinstance(item, qc.FusedCircuit):
                item(s)
            else:
                workloads.run(s, [item])
        tr_f = s.trace()
        torch.cuda.synchronize()
        dt_f = time.perf_counter() - t0
    res['fused_circuit_s'] = dt_f
    res['fused_passes'] = sum(c.n_passes for c in segments
                              if isinstance(c, qc.FusedCircuit))
    res['fused_final_trace'] = tr_f
    res['fused_max_abs_diff'] = float(np.abs(s.to_pv() - x_unfused).max())
    s = qg.PauliVectorGB300([bases.general(3)] * 8, force=True)
    s._data.copy_(torch.rand_like(s._data) * 2.0 ** -12)
    dense81 = rng.standard_normal((9, 9, 9, 9)) / 9
    for name, ptm, qs in (('9x9_q4', workloads.qutrit_1q(rng), (4,)),
                          ('81x81_q2_q5', workloads.qutrit_2q(rng), (2, 5)),
                          ('81x81_q7_q6', workloads.qutrit_2q(rng), (7, 6)),
                          # a dense 81x81 (6561 terms): the generic kernel
                          ('81x81_dense_q2_q5', dense81, (2, 5))):
        res[name + '_gbs'] = _time_app(s, ptm, qs, nbytes)
    return res


def run_circuit_configs():
    """Whole circuits, unit by unit against fused (quantumsim_gb300.circuit):
    the 14-qubit noisy circuit (50 layers of 14 noisy rotations and 7 noisy
    CZs on random pairs, 1050 units, then the partial trace keeping 4
    qubits) and the 6-qubit, 20-layer circuit (eager, fused, fused CUDA-graph
    replay, and the oracle on the host for scale)."""
    import numpy as np
    import torch
    import quantumsim_gb300 as qg
    from quantumsim_gb300 import bases, workloads, circuit as qc
    out = {}
    ops, keep = workloads.config1_circuit(seed=1)
    units = [(p, qs) for _, p, qs in ops]
    t0 = time.perf_counter()
    fused = qc.FusedCircuit(units)
    plan_s = time.perf_counter() - t0
    unfused = qc.FusedCircuit(units, fuse=False)
    rng = np.random.default_rng(2)
    res = {}
    for name, circ in (('unit_by_unit', unfused), ('fused', fused)):
        for rep in range(2):  # the first pass compiles the PTM patterns
            s = qg.PauliVectorGB300([bases.general(2)] * 14, force=True)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            circ(s)
            pt = s.partial_trace(*keep)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
        res[name] = (dt, pt.to_pv())
    diff = float(np.abs(res['fused'][1] - res['unit_by_unit'][1]).max())
    out['circuit_14q'] = {
        'workload': '14 qubits FP64, 50 layers x (14 noisy rotations + 7 '
                    'noisy CZ on random pairs), partial trace keeping {}'
                    .format(list(keep)),
        'units': fused.n_units, 'fused_passes': fused.n_passes,
        'plan_s': plan_s,
        'unit_by_unit_s': res['unit_by_unit'][0], 'fused_s': res['fused'][0],
        'speedup': res['unit_by_unit'][0] / res['fused'][0],
        'max_abs_diff_partial_trace': diff}
    # small state: host cost per unit dominates
    ops0 = workloads.config0_circuit(seed=0)
    units0 = [(p, qs) for _, p, qs in ops0]
    f0 = qc.FusedCircuit(units0)
    u0 = qc.FusedCircuit(units0, fuse=False)
    b6 = [bases.general(2)] * 6
    times = {}
    for name, circ in (('unit_by_unit', u0), ('fused', f0)):
        circ(qg.PauliVectorGB300(b6))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(20):
            circ(qg.PauliVectorGB300(b6))
        torch.cuda.synchronize()
        times[name] = (time.perf_counter() - t0) / 20
    graph = f0.capture(qg.PauliVectorGB300(b6))
    s = qg.PauliVectorGB300(b6)
    graph.run(s)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(200):
        graph.run(s)
    torch.cuda.synchronize()
    times['fused_graph'] = (time.perf_counter() - t0) / 200
    from oracle import pauli_vector_np as O
    x = O.initial_pv(b6)
    t0 = time.perf_counter()
    for _ in range(5):
        y = x
        for p, qs in units0:
            y = O.apply_ptm(y, p, *qs)
    times['oracle_host'] = (time.perf_counter() - t0) / 5
    out['circuit_6q'] = {
        'workload': '6 qubits FP64, 20 layers x (6 noisy rotations + CZ on '
                    'a line matching)',
        'units': f0.n_units, 'fused_passes': f0.n_passes,
        'seconds': times}
    return out


def run_ops_config():
    """The non-apply operations of the backend, on resident states: on the
    14-qubit FP64 vector diagonal, trace, meas_prob, partial_trace (keep 4)
    and renormalize; on the 8-qutrit vector reduce_basis (9 -> 3, the
    computational subbasis) and project.  Host wall time per call with a
    device synchronisation, averaged over repetitions (diagonal and
    partial_trace leave their result on the device)."""
    import numpy as np
    import torch
    import quantumsim_gb300 as qg
    from quantumsim_gb300 import bases

    def per_call(fn, reps):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps

    out = {}
    n = N_QUBITS
    s = qg.PauliVectorGB300([bases.general(2)] * n, force=True)
    s._data.copy_(torch.rand_like(s._data) * 2.0 ** -14)
    nbytes = 2 * 4 ** n * 8
    out['diagonal_us'] = per_call(lambda: s.diagonal(get_data=False), 50) * 1e6
    out['trace_us'] = per_call(s.trace, 50) * 1e6
    out['meas_prob_us'] = per_call(lambda: s.meas_prob(5), 50) * 1e6
    out['partial_trace_keep4_us'] = per_call(
        lambda: s.partial_trace(0, 3, 5, 7), 20) * 1e6
    t = per_call(s.renormalize, 10)
    out['renormalize_ms'] = t * 1e3
    out['renormalize_gbs'] = nbytes / t / 1e9
    # host time per call on a 6-qubit state (32 KB, kernels of a few us):
    # apply_ptm calls queued back to back with one synchronisation at the
    # end; trace and meas_prob return host values, so each call waits for
    # its own result
    from quantumsim_gb300 import workloads
    rng = np.random.default_rng(0)
    t1, t2 = workloads.coherence_times(rng, 6)
    cz = workloads.noisy_cz(rng, (1, 2), t1, t2)
    rot = workloads.noisy_1q(rng, t1[3], t2[3])
    s6 = qg.PauliVectorGB300([bases.general(2)] * 6)
    out['apply_ptm_2q_6q_host_us'] = per_call(
        lambda: s6.apply_ptm(cz, 1, 2), 2000) * 1e6
    out['apply_ptm_1q_6q_host_us'] = per_call(
        lambda: s6.apply_ptm(rot, 3), 2000) * 1e6
    out['trace_6q_us'] = per_call(s6.trace, 200) * 1e6
    out['meas_prob_6q_us'] = per_call(lambda: s6.meas_prob(3), 200) * 1e6
    del s6
    del s
    g3 = bases.general(3)
    comp = [g3.computational_basis_indices[i] for i in range(3)]

    def reduce():
        q = qg.PauliVectorGB300([g3] * 8, force=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        q.reduce_basis(3, comp)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        q.project(5, 1)
        torch.cuda.synchronize()
        return t1 - t0, time.perf_counter() - t1
    reduce()
    tr, tp = min(reduce() for _ in range(5))
    n_red = 9 ** 7 * 3  # entries kept by reduce_basis
    out['reduce_basis_9to3_ms'] = tr * 1e3
    out['reduce_basis_gbs'] = 2 * n_red * 8 / tr / 1e9
    out['project_ms'] = tp * 1e3
    # the take kernel alone: 20 launches on resident tensors larger than L2,
    # replayed from a CUDA graph (a project kernel runs for a few us, less
    # than one host call) and timed with CUDA events on the replaying
    # stream; bytes = entries kept, read and written
    q = qg.PauliVectorGB300([g3] * 8, force=True)
    q._data.copy_(torch.rand_like(q._data))
    red = torch.ops.qsgb.take_axis(q._data, 3, comp)
    for name, x, axis, idx, n_keep in (
            ('reduce_basis_9to3', q._data, 3, comp, n_red),
            ('project_9to1', red, 5, [comp[1]], 9 ** 6 * 3)):
        torch.ops.qsgb.take_axis(x, axis, idx)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            with torch.cuda.graph(graph, stream=side):
                for _ in range(20):
                    torch.ops.qsgb.take_axis(x, axis, idx)
        torch.cuda.current_stream().wait_stream(side)
        graph.replay()
        stream = torch.cuda.current_stream()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        graph.replay()
        b.record(stream)
        torch.cuda.synchronize()
        dt = a.elapsed_time(b) / 1e3 / 20
        out[name + '_kernel_us'] = dt * 1e6
        out[name + '_kernel_gbs'] = 2 * n_keep * 8 / dt / 1e9
        del graph
    del q, red
    out['workload'] = ('14 qubits FP64 (diagonal, trace, meas_prob, '
                       'partial_trace keeping 4, renormalize); 8 qutrits '
                       'FP64 (reduce_basis 9 -> 3 on one qutrit, then '
                       'project another)')
    return out


def run_grad_config():
    """10 qubits, 40 layers, 249 physical parameters: one gradient step
    (forward, KL loss, adjoint with checkpoints every 8 layers) in FP64 and
    with FP32 storage, unit by unit and with each CZ absorbing its qubits'
    rotations."""
    import torch
    from quantumsim_gb300 import fitting
    m = fitting.NoisyCircuitModel()
    target = m.probabilities(m.perturbed()).detach()
    out = {'params': m.n_params, 'qubits': m.n, 'layers': m.n_layers,
           'checkpoint_every': 8}
    for name, dtype in (('f64', torch.float64), ('f32', torch.float32)):
        for fuse in (False, True):
            ts = []
            for rep in range(3):
                p = m.params()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                loss = m.loss(p, target, dtype=dtype, checkpoint_every=8,
                              fuse=fuse)
                loss.backward()
                torch.cuda.synchronize()
                ts.append(time.perf_counter() - t0)
            out[name + ('_fused' if fuse else '') + '_step_s'] = min(ts[1:])
        # the circuit part of the step replayed from a CUDA graph (PTMs
        # built on the GPU; fused layers)
        step = fitting.GraphedGradient(m, target, dtype=dtype,
                                       checkpoint_every=8, fuse=True)
        ts = []
        for rep in range(5):
            p = {k: v.clone().to(step.dev).requires_grad_(True)
                 for k, v in m.init.items()}
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            loss = step.step(p)
            float(loss)
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        out[name + '_graph_step_s'] = min(ts[1:])
        del step
    return out


def qops_arith(name):
    from quantumsim_gb300.pauli_vector import _ARITH
    return _ARITH[name]


def _time_app(s, ptm, qs, bytes_per_app, reps=3):
    import torch
    stream = torch.cuda.current_stream()
    s.apply_ptm(ptm, *qs)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        s.apply_ptm(ptm, *qs)
    b.record(stream)
    torch.cuda.synchronize()
    return round(bytes_per_app * reps / (a.elapsed_time(b) / 1e3) / 1e9, 1)


def run_profile_case(args):
    """Small workload for ncu captures: a 12-qubit FP64 state (134 MB, larger
    than L2); one circuit layer (12 noisy rotations + 3 noisy CZs), then 3x
    [noisy CZ on (3, 7), noisy rotation on qubit 5, dense 16x16 PTM on
    (3, 7), noisy CZ on the last two qubits].
    Launch order: 15 setup launches, then 4 per repetition."""
    import numpy as np
    import torch
    from quantumsim_gb300 import build as qbuild
    qbuild.build()
    import quantumsim_gb300 as qg
    from quantumsim_gb300 import bases, workloads
    n = args.profile_qubits
    s = qg.PauliVectorGB300([bases.general(2)] * n, force=True)
    rng = np.random.default_rng(3)
    t1, t2 = workloads.coherence_times(rng, n)
    for op in workloads.config1_layer(rng, n, t1, t2, 3):
        s.apply_ptm(op[1], *op[2])
    cz = workloads.noisy_cz(rng, (3, 7), t1, t2)
    r1 = workloads.noisy_1q(rng, t1[5], t2[5])
    dense = rng.standard_normal((4, 4, 4, 4)) * 0.25
    last = workloads.noisy_cz(rng, (n - 2, n - 1), t1, t2)
    for _ in range(3):
        s.apply_ptm(cz, 3, 7)
        s.apply_ptm(r1, 5)
        s.apply_ptm(dense, 3, 7)
        s.apply_ptm(last, n - 2, n - 1)
    torch.cuda.synchronize()
    print(json.dumps({'profile_case': n, 'trace': s.trace()}))


def run_profile_tc(args):
    """Small workload for ncu captures of the tensor-core kernel for dense
    16x16 PTMs: a 12-qubit FP64 state (134 MB, larger than L2), one circuit
    layer (12 noisy rotations + 3 noisy CZs), then 3x [dense PTM on (3, 7),
    on the last two qubits (10, 11), and on (0, 11)].
    Launch order: 15 setup launches, then 3 per repetition."""
    import numpy as np
    import torch
    from quantumsim_gb300 import build as qbuild
    qbuild.build()
    import quantumsim_gb300 as qg
    from quantumsim_gb300 import bases, workloads
    n = args.profile_qubits
    s = qg.PauliVectorGB300([bases.general(2)] * n, force=True)
    rng = np.random.default_rng(3)
    t1, t2 = workloads.coherence_times(rng, n)
    for op in workloads.config1_layer(rng, n, t1, t2, 3):
        s.apply_ptm(op[1], *op[2])
    dense = rng.standard_normal((4, 4, 4, 4)) * 0.25
    for _ in range(3):
        s.apply_ptm(dense, 3, 7)
        s.apply_ptm(dense, n - 2, n - 1)
        s.apply_ptm(dense, 0, n - 1)
    torch.cuda.synchronize()
    print(json.dumps({'profile_case': 'tc', 'trace': s.trace()}))


def run_profile_grad(args):
    """ncu workload for the graphed gradient step of the 249-parameter
    10-qubit model (--profile-dtype f64 or f32): the graph is captured and
    replayed once outside the profiled range, then replayed once between
    cudaProfilerStart and cudaProfilerStop (run ncu with
    --profile-from-start off). The graph holds the whole step: the batched
    PTM builder and its backward (a few hundred small torch kernels) and
    about 1,100 launches of the apply, tensor-core and PTM-gradient
    kernels."""
    import torch
    from quantumsim_gb300 import build as qbuild
    qbuild.build()
    from quantumsim_gb300 import fitting
    dtype = torch.float32 if args.profile_dtype == 'f32' else torch.float64
    m = fitting.NoisyCircuitModel()
    target = m.probabilities(m.perturbed()).detach()
    step = fitting.GraphedGradient(m, target, dtype=dtype, checkpoint_every=8,
                                   fuse=True)
    step.graph.replay()
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    step.graph.replay()
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    print(json.dumps({'profile_case': 'grad', 'dtype': args.profile_dtype,
                      'loss': float(step.loss)}))


def run_profile_fused(args):
    """ncu workload for the specialised kernels on fused passes of the
    14-qubit noisy circuit: a 12-qubit FP64 state (268 MB) and three fused
    two-qubit PTMs from the assignment plan of that circuit -- the first
    off the last qubit, at least two qubits apart, with 3.12, 4.38 and 6.25
    non-zero terms per row -- each applied three times on its own pair.
    Launch order: 3 per PTM."""
    import numpy as np
    import torch
    from quantumsim_gb300 import build as qbuild
    qbuild.build()
    import quantumsim_gb300 as qg
    from quantumsim_gb300 import bases, workloads, circuit as qc
    ops, _ = workloads.config1_circuit(seed=1)
    plan = qc._plan_assigned([(p, qs) for _, p, qs in ops])
    n = 12
    pick = {}
    for p, qs in plan:
        k = int(np.prod(p.shape[:len(qs)]))
        t = qc.terms_per_row(p.reshape(k, k))
        if len(qs) != 2 or max(qs) >= n or abs(qs[0] - qs[1]) < 2:
            continue
        for target in (3.12, 4.38, 6.25):
            if abs(t - target) < 0.01 and target not in pick:
                pick[target] = (p, qs)
    s = qg.PauliVectorGB300([bases.general(2)] * n, force=True)
    s._data.copy_(torch.rand_like(s._data) * 2.0 ** -12)
    out = {}
    for target in (3.12, 4.38, 6.25):
        p, qs = pick[target]
        for _ in range(3):
            s.apply_ptm(p, *qs)
        out[str(target)] = list(qs)
    torch.cuda.synchronize()
    print(json.dumps({'profile_case': 'fused', 'pairs': out}))


def run_profile_take(args):
    """Small workload for ncu captures of the take-along-an-axis kernels
    (reduce_basis / project): 8 qutrits (9^8 float64 entries, 344 MB); 3x
    [reduce_basis 9 -> 3 of qutrit 3 (rows of 6561 entries, 16-byte units),
    the same of qutrit 7 (rows of one entry), project 9 -> 1 of qutrit 5 of
    the reduced vector].  Launch order: 3 per repetition."""
    import torch
    from quantumsim_gb300 import build as qbuild
    qbuild.build()
    import quantumsim_gb300 as qg
    from quantumsim_gb300 import bases
    g3 = bases.general(3)
    comp = [g3.computational_basis_indices[i] for i in range(3)]
    q = qg.PauliVectorGB300([g3] * 8, force=True)
    q._data.copy_(torch.rand_like(q._data))
    for _ in range(3):
        red = torch.ops.qsgb.take_axis(q._data, 3, comp)
        torch.ops.qsgb.take_axis(q._data, 7, comp)
        torch.ops.qsgb.take_axis(red, 5, [comp[1]])
    torch.cuda.synchronize()
    print(json.dumps({'profile_case': 'take', 'sum': float(red.sum())}))


def run_profile_qutrits(args):
    """Small workload for ncu captures of the qutrit kernels: 8 qutrits
    (9^8 float64 entries, 344 MB); one layer of 9x9 PTMs on every qutrit, then
    3x [9x9 on qutrit 4, 81x81 CZ with leakage on (2, 5), the same on
    (7, 6), 9x9 on qutrit 7, 81x81 on (0, 7)].  Launch order: 8 setup
    applications, then 5 per repetition."""
    import numpy as np
    import torch
    from quantumsim_gb300 import build as qbuild
    qbuild.build()
    import quantumsim_gb300 as qg
    from quantumsim_gb300 import bases, workloads
    rng = np.random.default_rng(5)
    s = qg.PauliVectorGB300([bases.general(3)] * 8, force=True)
    for q in range(8):
        s.apply_ptm(workloads.qutrit_1q(rng), q)
    p1 = workloads.qutrit_1q(rng)
    p2 = workloads.qutrit_2q(rng)
    for _ in range(3):
        s.apply_ptm(p1, 4)
        s.apply_ptm(p2, 2, 5)
        s.apply_ptm(p2, 7, 6)
        s.apply_ptm(p1, 7)
        s.apply_ptm(p2, 0, 7)
    torch.cuda.synchronize()
    print(json.dumps({'profile_case': 'qutrits', 'trace': s.trace()}))


def run_profile_circuit(args):
    """The fused 14-qubit noisy circuit (1050 units, 337 passes) applied
    once to the |0..0> state, then the partial trace; for an ncu launch
    list (gpu__time_duration only: one pass per launch).  Prints the terms
    per row of every fused pass, in launch order."""
    import numpy as np
    import torch
    from quantumsim_gb300 import build as qbuild
    qbuild.build()
    import quantumsim_gb300 as qg
    from quantumsim_gb300 import bases, workloads, circuit as qc
    ops, keep = workloads.config1_circuit(seed=1)
    circ = qc.FusedCircuit([(p, qs) for _, p, qs in ops])
    s = qg.PauliVectorGB300([bases.general(2)] * 14, force=True)
    circ(s)
    s.partial_trace(*keep)
    torch.cuda.synchronize()
    terms = [round(qc.terms_per_row(p.reshape(int(np.sqrt(p.size)), -1)), 2)
             for p, _ in circ.fused]
    print(json.dumps({'profile_case': 'circuit', 'passes': len(terms),
                      'terms_per_row': terms,
                      'qudits': [list(q) for _, q in circ.fused]}))


def run_profile_batched(args):
    """Workload for ncu captures of the batched kernel: 16 circuits of 11 and
    12 qubits (0.9 GB of FP32 state, 2.6 GB with adjoint and checkpoints),
    depth 3, checkpoints every 2 layers; one plain (non-graph) launch per
    step with a fixed tile, 2 steps."""
    import torch
    from quantumsim_gb300 import build as qbuild
    qbuild.build()
    from quantumsim_gb300 import batch as BT
    import numpy as np
    specs = [BT.CircuitSpec(11 + (i % 2), 3, i) for i in range(16)]
    targets = [BT.target_probabilities(sp, 1000 + i)
               for i, sp in enumerate(specs)]
    sim = BT.BatchedSimulator(specs, targets, checkpoint_every=2, tile=8192)
    sim.set_ptms([BT.instance_ptms(sp) for sp in specs])
    for _ in range(2):
        sim.step(use_graph=False)
    torch.cuda.synchronize()
    sim.check()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    sim.step(use_graph=False)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    print(json.dumps({'profile_case': 'batched',
                      'loss0': float(sim.results()[1][0]), 'step_ms': ms,
                      'algorithmic_bytes': sim.algorithmic_bytes(),
                      'achieved_gbs': sim.algorithmic_bytes() / ms / 1e6}))


def run_profile_adjoint2(args):
    """Workload for ncu captures of the batched two-qubit adjoint: 16
    circuits of 12 qubits, each 12 CZs on the pair `--profile-pair` (default
    5,6), forward + adjoint as one plain launch per step, 2 steps (3.2 GB on
    the device with adjoint and checkpoint buffers)."""
    import math
    import torch
    from quantumsim_gb300 import build as qbuild
    qbuild.build()
    from quantumsim_gb300 import batch as BT
    from quantumsim_gb300 import ptm as P
    q0, q1 = (int(v) for v in args.profile_pair.split(','))
    cz = P.cphase(math.pi).reshape(16, 16).double()

    class PairSpec(BT.CircuitSpec):
        def ops(self):
            return [(0, (q0, q1))] * 12

    specs = [PairSpec(12, 1, i) for i in range(16)]
    uniform = [torch.full((2 ** 12,), 1.0 / 2 ** 12, dtype=torch.float64)
               for _ in specs]
    sim = BT.BatchedSimulator(specs, uniform, checkpoint_every=8, tile=8192)
    sim.set_ptms([[cz] * 12 for _ in specs])
    for _ in range(2):
        sim.step(use_graph=False)
    torch.cuda.synchronize()
    sim.check()
    print(json.dumps({'profile_case': 'adjoint2', 'pair': [q0, q1],
                      'loss0': float(sim.results()[1][0])}))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split('\n')[0])
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--cpu-apps', type=int, default=16)
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-sweep', action='store_true')
    ap.add_argument('--no-batched', action='store_true',
                    help='skip the batched FP32 forward+adjoint measurement')
    ap.add_argument('--batch-instances', type=int, default=512)
    ap.add_argument('--plain-all', action='store_true',
                    help='also time the plain path on every batched instance '
                         '(about 100 s)')
    ap.add_argument('--no-configs', action='store_true',
                    help='skip the qutrit and differentiation measurements')
    ap.add_argument('--traffic', type=float, default=0.0,
                    help='dram bytes per launch from an ncu capture')
    ap.add_argument('--profile-case', nargs='?', const='apply',
                    choices=['apply', 'qutrits', 'tc', 'take', 'batched',
                             'circuit', 'adjoint2', 'grad', 'fused'],
                    help='run a small ncu profiling workload and exit')
    ap.add_argument('--profile-qubits', type=int, default=12)
    ap.add_argument('--profile-dtype', choices=['f64', 'f32'], default='f64',
                    help='storage of the grad profiling workload')
    ap.add_argument('--profile-pair', default='5,6',
                    help='qubit pair of the adjoint2 profiling workload')
    args = ap.parse_args()
    if args.profile_case:
        {'apply': run_profile_case, 'qutrits': run_profile_qutrits,
         'tc': run_profile_tc, 'take': run_profile_take,
         'batched': run_profile_batched, 'adjoint2': run_profile_adjoint2,
         'circuit': run_profile_circuit, 'fused': run_profile_fused,
         'grad': run_profile_grad}[args.profile_case](args)
        return
    if args.warmup < 3 and args.impl == 'gb300':
        print('warning: fewer than 3 warm-up steps', file=sys.stderr)
    if args.impl == 'reference':
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == '__main__':
    main()
