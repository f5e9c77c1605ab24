"""The allocation-free walk entry point (madi_walk_noalloc) through the C ABI.

Some callers cannot allocate device memory around a walk (graph capture,
plug-in hosts with only pre-sized buffers, exhausted fixed pools).  This entry
point takes the persistent walker's tile counter from a static device array
instead of a caller buffer.  Its sums must equal madi_walk's exactly, and a
second call in a row must again (each call clears the shared counter).  The file
is named to be collected last.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_walk_equals_walk_on_two_calls_in_a_row():
    import torch
    from custom_madi_gb300 import _native as N
    from custom_madi_gb300 import signal as S
    from custom_madi_gb300.config import SimConfig
    from custom_madi_gb300.ensemble import create_ensemble
    from custom_madi_gb300.walker_gpu import LaunchConfig, WalkBatch, WalkJob, kio_to_pp, pair_layout

    cfg = SimConfig(boundary_mode="periodic", n_cells=64, n_walkers=4096, n_ensembles=1, ts=0.01, T_max_ms=46.0,
                    small_deltas=[6.0], big_deltas=[15.0, 25.0, 30.0, 40.0],
                    b_values=[0.0, 1000.0, 2500.0, 4000.0, 6000.0], geometry_validation_points=20_000,
                    geometry_vi_tolerance=0.1)
    ens = create_ensemble(2.0e5, 4.0, cfg, seed=0)
    cols = S.build_columns(cfg)
    lay = pair_layout(cols.j_delta, cols.j_Delta, cols.j_sum, cols.phase_coef)
    jobs = [WalkJob(ens, kio_to_pp(20.0, ens.mean_AV, cfg), 7, 4096), WalkJob(ens, 0.01, 8, 3000)]
    batch = WalkBatch(jobs, cfg, layout=lay, dirs=cfg.direction_array(),
                      launch=LaunchConfig(tile_walkers=128, blocks_per_sm=1))
    assert batch.desc.grid_blocks > 0          # persistent: the tile counter is in use
    batch.launch()
    torch.cuda.synchronize()
    ref = [t.clone() for t in (batch.accum, batch.occupancy, batch.counters)]
    assert int(ref[2][:, 0].sum()) == 4096 + 3000

    desc = N.MadiWalkDesc.from_buffer_copy(batch.desc)
    desc.work_counter = None                   # the caller provides no scratch
    stream = torch.cuda.current_stream()
    for _ in range(2):
        for t in (batch.accum, batch.occupancy, batch.counters):
            t.zero_()
        N.check(N.lib().madi_walk_noalloc(C.byref(desc), stream.cuda_stream), "madi_walk_noalloc")
        torch.cuda.synchronize()
        assert torch.equal(batch.accum, ref[0])
        assert torch.equal(batch.occupancy, ref[1])
        assert torch.equal(batch.counters, ref[2])
