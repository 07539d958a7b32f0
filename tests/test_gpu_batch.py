"""Batched forward + adjoint (one persistent launch, FP32 Pauli vectors, FP64
reductions) against the plain GPU path run one instance at a time, and the
probabilities against FP64."""
import numpy as np
import pytest
import torch

from quantumsim_gb300 import batch as BT

pytestmark = pytest.mark.gpu


def _setup(ns, depth, every, seed=0):
    specs = [BT.CircuitSpec(n, depth, seed + i) for i, n in enumerate(ns)]
    targets = [BT.target_probabilities(s, 1000 + i)
               for i, s in enumerate(specs)]
    ptms = [BT.instance_ptms(s) for s in specs]
    return specs, targets, ptms


@pytest.mark.parametrize('use_graph', [False, True])
def test_batched_matches_plain_path(use_graph):
    ns = [3, 5, 4, 6, 2, 5]
    specs, targets, ptms = _setup(ns, depth=10, every=4)
    sim = BT.BatchedSimulator(specs, targets, checkpoint_every=4, tile=64)
    sim.set_ptms(ptms)
    for _ in range(2):  # the second replay must give the same results
        sim.step(use_graph=use_graph)
    torch.cuda.synchronize()
    probs, loss, grads = sim.results()
    for i, s in enumerate(specs):
        p32, l32, g32 = BT.plain_gradients(s, ptms[i], targets[i],
                                           dtype=torch.float32,
                                           checkpoint_every=4)
        p64, l64, g64 = BT.plain_gradients(s, ptms[i], targets[i],
                                           dtype=torch.float64,
                                           checkpoint_every=4)
        # probabilities: FP32 storage within 1e-6 of FP64
        assert float((probs[i] - p64).abs().max()) < 1e-6
        np.testing.assert_allclose(probs[i].cpu(), p32.cpu(), rtol=0,
                                   atol=1e-6)
        # the loss is a sum of t*log(t/p); FP32 storage moves it by ~1e-5
        # relative against FP64 and by less against the FP32 plain path
        assert float(loss[i]) == pytest.approx(float(l32), rel=2e-5,
                                               abs=1e-9)
        assert float(loss[i]) == pytest.approx(float(l64), rel=1e-3,
                                               abs=1e-8)
        scale = max(float(g.abs().max()) for g in g64)
        for gb, gr in zip(grads[i], g64):
            assert float((gb - gr.to(gb.device)).abs().max()) < 1e-4 * scale


def test_batched_tiles_and_autotune_give_same_results():
    """Probabilities and losses do not depend on the tile size; the PTM
    gradients only through the FP32 rounding of their partial sums (a
    thread carries FP32 products over 4 tiles of its item before folding
    them into FP64, so the item size moves that rounding: 1e-6 of the
    largest gradient entry).  The same tile gives bit-identical results."""
    ns = [7, 4, 6]
    specs, targets, ptms = _setup(ns, depth=9, every=3, seed=5)
    sim = BT.BatchedSimulator(specs, targets, checkpoint_every=3, tile=256)
    sim.set_ptms(ptms)
    sim.step(use_graph=False)
    torch.cuda.synchronize()
    p_a, l_a, g_a = [x.clone() if torch.is_tensor(x) else
                     [[t.clone() for t in gi] for gi in x]
                     for x in (torch.cat(sim.results()[0]), sim.results()[1],
                               sim.results()[2])]
    times = sim.autotune(candidates=(32, 128, 1024), reps=1)
    assert set(times) == {32, 128, 1024} and sim.tile in times
    chosen = sim.tile
    for tile in (32, 128, 1024, chosen):
        sim._build_program(tile)
        sim.set_ptms(ptms)
        sim.step(use_graph=False)
        torch.cuda.synchronize()
        p_b, l_b, g_b = sim.results()
        np.testing.assert_allclose(torch.cat(p_b).cpu(), p_a.cpu(), rtol=0,
                                   atol=1e-12)
        np.testing.assert_allclose(l_b.cpu(), l_a.cpu(), rtol=1e-12,
                                   atol=1e-14)
        for gi_a, gi_b in zip(g_a, g_b):
            scale = max(float(a.abs().max()) for a in gi_a)
            for a, b in zip(gi_a, gi_b):
                np.testing.assert_allclose(b.cpu(), a.cpu(), rtol=0,
                                           atol=1e-6 * scale)
    # a fixed tile is deterministic: a second step gives identical bits
    p_b = torch.cat(p_b).clone()
    l_b = l_b.clone()
    g_b = [[t.clone() for t in gi] for gi in g_b]
    sim.set_ptms(ptms)
    sim.step(use_graph=False)
    torch.cuda.synchronize()
    p_c, l_c, g_c = sim.results()
    assert torch.equal(torch.cat(p_c), p_b)
    assert torch.equal(l_c, l_b)
    for gi_b, gi_c in zip(g_b, g_c):
        for b, c in zip(gi_b, gi_c):
            assert torch.equal(b, c)


def test_grid_barrier_wait_expires_and_context_survives():
    """Every grid barrier polls a bounded number of times.  A barrier that no
    block can complete (its arrival counter starts past the grid size, a
    flag nothing will set) ends after the spin limit: the kernel reports
    QSGB_DEV_TIMEOUT, all blocks return, and the next normal step on the same
    context gives the same results as before."""
    import ctypes

    from quantumsim_gb300 import _lib as L

    ns = [5, 4, 6]
    specs, targets, ptms = _setup(ns, depth=4, every=2, seed=21)
    sim = BT.BatchedSimulator(specs, targets, checkpoint_every=2, tile=256)
    sim.set_ptms(ptms)
    sim.step(use_graph=False)
    torch.cuda.synchronize()
    probs0, loss0, _ = [x for x in sim.results()]
    probs0 = [p.clone() for p in probs0]
    loss0 = loss0.clone()

    sim.work.zero_()
    sim.work[sim.n_stages] = 1 << 30  # barrier arrival counter
    st = sim.lib.qsgb_batch_run(
        ctypes.byref(sim.prog), sim.max_grid, BT.BLOCK, 1,
        ctypes.c_void_p(sim.status.data_ptr()), 20000,
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    L.check(st, 'qsgb_batch_run')
    torch.cuda.synchronize()
    assert int(sim.status.item()) & L.DEV_TIMEOUT
    with pytest.raises(RuntimeError, match='device status'):
        sim.check()  # reports and clears the status

    sim.step(use_graph=False)
    torch.cuda.synchronize()
    probs1, loss1, _ = sim.results()
    for a, b in zip(probs0, probs1):
        assert torch.equal(a, b)
    assert torch.equal(loss0, loss1)


def test_fused_units_match_unfused_program():
    """Units (a CZ absorbing the rotations before it) against one unit per
    op: the same probabilities, losses and per-op gradients up to the FP32
    rounding of the different products."""
    ns = [5, 3, 6, 4]
    specs, targets, ptms = _setup(ns, depth=6, every=2, seed=31)
    out = []
    for fuse in (True, False):
        sim = BT.BatchedSimulator(specs, targets, checkpoint_every=2,
                                  tile=128, fuse=fuse)
        sim.set_ptms(ptms)
        sim.step(use_graph=True)
        torch.cuda.synchronize()
        p, l, g = sim.results()
        out.append(([t.clone() for t in p], l.clone(),
                    [[t.clone() for t in gi] for gi in g], sim.n_ptm))
    (pf, lf, gf, nf), (pu, lu, gu, nu) = out
    assert nf < nu
    for a, b in zip(pf, pu):
        assert float((a - b).abs().max()) < 1e-6
    np.testing.assert_allclose(lf.cpu(), lu.cpu(), rtol=1e-4, atol=1e-8)
    for gi_f, gi_u in zip(gf, gu):
        scale = max(float(t.abs().max()) for t in gi_u)
        for a, b in zip(gi_f, gi_u):
            assert float((a - b).abs().max()) < 1e-4 * scale


@pytest.mark.parametrize('field,value', [('inst', None), ('q1', 'q0'),
                                         ('end', 'past')])
def test_malformed_items_are_skipped_and_reported(field, value):
    """The kernel checks every item against its instance before touching
    memory: an instance index at the count, a second target equal to the
    first, a range past the vector.  Each is skipped with QSGB_DEV_BADITEM,
    and the context then gives the same results as before."""
    from quantumsim_gb300 import _lib as L

    specs, targets, ptms = _setup([4, 5], depth=2, every=2, seed=41)
    sim = BT.BatchedSimulator(specs, targets, checkpoint_every=2, tile=64)
    sim.set_ptms(ptms)
    sim.step(use_graph=False)
    torch.cuda.synchronize()
    p0 = [p.clone() for p in sim.results()[0]]
    good = sim.items_dev.clone()
    items = good.cpu().numpy().view(BT._ITEM_DTYPE).copy()
    j = int(np.nonzero((items['op'] == BT.BOP_APPLY) & (items['q1'] >= 0))[0][0])
    if field == 'inst':
        items['inst'][j] = sim.n_inst
    elif field == 'q1':
        items['q1'][j] = items['q0'][j]
    else:
        items['end'][j] = items['end'][j] + 4 ** 8
    sim.items_dev.copy_(torch.from_numpy(items.view(np.uint8).copy()))
    sim.step(use_graph=False)
    torch.cuda.synchronize()
    assert int(sim.status.item()) & L.DEV_BADITEM
    with pytest.raises(RuntimeError, match='device status'):
        sim.check()
    sim.items_dev.copy_(good)
    sim.step(use_graph=False)
    torch.cuda.synchronize()
    for a, b in zip(p0, sim.results()[0]):
        assert torch.equal(a, b)


def test_new_ptms_after_the_graph_is_captured():
    """set_ptms after the step's graph was captured: the replayed graph
    reads the new unit PTMs and the new gradient-mapping factors (updated
    in place), giving bit for bit what a fresh simulator gives."""
    ns = [5, 4, 7, 6]
    specs, targets, ptms = _setup(ns, depth=9, every=4, seed=3)
    other = [BT.instance_ptms(s, angle_offset=torch.from_numpy(
        np.random.default_rng(40 + i).normal(0, 0.1, (s.depth, s.n))))
        for i, s in enumerate(specs)]
    sim = BT.BatchedSimulator(specs, targets, checkpoint_every=4, tile=64)
    sim.set_ptms(ptms)
    sim.step(use_graph=True)
    graph = sim.graph
    sim.set_ptms(other)
    assert sim.graph is graph  # same structure: the graph is kept
    sim.step(use_graph=True)
    torch.cuda.synchronize()
    p1, l1, g1 = sim.results()
    fresh = BT.BatchedSimulator(specs, targets, checkpoint_every=4, tile=64)
    fresh.set_ptms(other)
    fresh.step(use_graph=True)
    torch.cuda.synchronize()
    p2, l2, g2 = fresh.results()
    assert torch.equal(l1, l2)
    for i in range(len(specs)):
        assert torch.equal(p1[i], p2[i])
        for a, b in zip(g1[i], g2[i]):
            assert torch.equal(a, b)
