"""bench.py's host-side helpers (no GPU): the committed render-kernel
counters that its issue-rate roofline reads, the launch count rule, and the
per-channel RMSE."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_counters_match_the_current_render_source():
    """The counters file holds an entry for the terrain workload's autotuned
    settings (register variant 2, cut 1/128, 128-thread blocks, 32-sample
    segments) taken with the render source in the tree, so the bench reports
    a live issue-rate fraction.  A changed render.cu needs a new capture."""
    entry, why = bench.launch_counters(2, 1.0 / 128, (128, 32))
    assert why == "matched", why
    assert entry["render_cu_sha16"] == bench.source_sha16()
    rays = entry["rays"]
    assert rays == 256 * 6000 * 256
    per_ray = entry["warp_instructions"] / rays
    assert 20 < per_ray < 80
    assert 20 < entry["thread_instructions"] / entry["warp_instructions"] <= 32  # lanes per instruction
    assert 0 < entry["dram_bytes"] / rays < 10 and 0 < entry["l2_bytes"] / rays < 1000
    # other settings have no counters, and the bench then reports none
    entry, why = bench.launch_counters(1, 1.0 / 128, (128, 32))
    assert entry is None and "no counters" in why


def test_launch_count_rule():
    """Kernels per render launch: the render kernel, the near-field cut when
    a radius is set, and the chunk sums when an ommatidium's samples span
    several warp segments that a block cannot hold (as planRender decides)."""
    assert bench.render_kernels_per_launch(256, (128, 32), 1.0 / 128) == 3  # 8 chunks, 4-warp blocks: scratch
    assert bench.render_kernels_per_launch(256, (256, 32), 1.0 / 128) == 2  # 8-warp blocks hold the 8 chunks
    assert bench.render_kernels_per_launch(256, (512, 32), 0.0) == 1
    assert bench.render_kernels_per_launch(32, (128, 32), 0.0) == 1  # one segment per ommatidium
    assert bench.render_kernels_per_launch(256, (0, 32), 0.0) == 1  # automatic blocks choose in-block sums


def test_rmse_per_channel():
    ref = np.zeros((2, 3, 3), np.float32)
    a = ref.copy()
    a[..., 0] = 0.3
    a[..., 2] = -0.1
    r = bench.rmse_per_channel(a, ref)
    assert np.allclose(r, [0.3, 0.0, 0.1])
