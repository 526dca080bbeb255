"""Batches of independent cases (mrlbm_batch_*) and the autotuner (mrlbm_autotune).

A batch advances its cases with one persistent step-kernel launch over all cases' work items
plus one node-list and one wall launch, replayed from CUDA graphs.  The arithmetic per node
is that of a single-case step, and no tiling changes results, so every case of a batch must
match the same case stepped alone bit for bit (forces: to FP64 round-off, atomics order)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def mixed_cases():
    from mrlbm_3d_cuda_gb300 import cases
    return [
        cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0),
        cases.annulus(48, 48, 8, 8.0, 20.0, 0.05, 50.0),
        cases.periodic_box(40, 24, 12, u0=0.04, re=100.0),
        cases.cylinder_channel(96, 48, 24, 8, 32.0, 24.0, 0.05, 120.0, periodic_y=True, convective=True),
    ]


def init_case(sim, i):
    from mrlbm_3d_cuda_gb300 import native as N
    if i == 2:
        sim.init(N.INIT_NOISY_UNIFORM, (0.03, 0.01, -0.02, 0.3, 11))
    else:
        sim.init(N.INIT_REST)


def run_alone(descs, steps):
    from mrlbm_3d_cuda_gb300 import Simulation
    out = []
    for i, d in enumerate(descs):
        sim = Simulation(d, init=False)
        init_case(sim, i)
        sim.set_sampling(1, 0)
        sim.step(steps)
        st, f = sim.force_history()
        out.append((sim.moments(), f))
        sim.close()
    return out


def check_against(batch, alone):
    for i, c in enumerate(batch.cases):
        m = c.moments()
        assert np.array_equal(m, alone[i][0]), f"case {i} moments differ"
        _, f = c.force_history()
        assert f.shape == alone[i][1].shape, (i, f.shape, alone[i][1].shape)
        if f.size:
            # FP64 sums whose block partials are added atomically: equal up to the order of
            # those additions, i.e. to ~1e-9 of each wall's force scale
            scale = np.abs(alone[i][1]).max(axis=(0, 2), keepdims=True)
            assert np.all(np.abs(f - alone[i][1]) <= 1e-9 * np.maximum(scale, 1e-12)), i


def test_batch_graph_and_sequential_steps_match_single_cases(cuda_device):
    from mrlbm_3d_cuda_gb300 import Batch
    descs = mixed_cases()
    alone = run_alone(descs, 21)
    b = Batch(descs)
    for i, c in enumerate(b.cases):
        init_case(c, i)
    b.set_sampling(1)
    b.step(10)             # graph replay, both parities
    b.step_sequential(5)   # plain per-case launches
    b.step(6)
    b.sync()
    check_against(b, alone)
    b.close()


def test_batch_autotune_restores_state(cuda_device):
    from mrlbm_3d_cuda_gb300 import Batch
    descs = mixed_cases()
    alone = run_alone(descs, 9)
    b = Batch(descs)
    for i, c in enumerate(b.cases):
        init_case(c, i)
    before = [c.moments() for c in b.cases]
    tile = b.autotune(2)
    assert tile[0] == 32 and tile[1] in (4, 8, 16)
    for c, m in zip(b.cases, before):
        assert np.array_equal(c.moments(), m)
    b.set_sampling(1)
    b.step(9)
    b.sync()
    check_against(b, alone)
    b.close()


def test_single_case_autotune_restores_state_and_results(cuda_device):
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0)
    ref = Simulation(desc, init=False)
    ref.init(N.INIT_REST)
    ref.step(3)
    ref.set_sampling(1, 1)
    ref.step(7)
    want = ref.moments()
    ref.close()
    sim = Simulation(desc, init=False)
    sim.init(N.INIT_REST)
    sim.step(3)
    before = sim.moments()
    tile = sim.autotune(2)
    assert tile[1] in (4, 8, 16) and 1 <= tile[2] <= desc.nz
    assert np.array_equal(sim.moments(), before)
    assert sim.get_info().step == 3
    sim.set_sampling(1, 1)
    sim.step(7)
    assert np.array_equal(sim.moments(), want)
    steps, _ = sim.diagnostics()
    assert list(steps) == list(range(3, 10))
    sim.close()


def test_batch_handles_refuse_single_case_calls(cuda_device):
    from mrlbm_3d_cuda_gb300 import Batch, MrlbmError
    b = Batch(mixed_cases()[:2])
    with pytest.raises(MrlbmError):
        b.cases[0].step(1)
    b.close()


def test_batch_with_stochastic_rounding_matches_single_cases(cuda_device):
    """16-bit storage with stochastic rounding in a batch: the batch graph advances every case's
    random-bit counter with one launch per step, so each case still matches the same case
    stepped alone bit for bit (its random bits depend only on node, field pair and step)."""
    from mrlbm_3d_cuda_gb300 import Batch
    descs = mixed_cases()
    for d in descs:
        d.storage = 1
        d.stochastic_rounding = 1
    descs[2].stochastic_rounding = 0  # one case rounds to nearest: the tick skips it
    steps = 12
    alone = run_alone(descs, steps)
    b = Batch(descs)
    for i, c in enumerate(b.cases):
        init_case(c, i)
    b.set_sampling(1)
    b.step(steps)
    check_against(b, alone)
    b.close()
