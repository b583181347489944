"""The bench line's ncu figures (profiles/traffic.json), read on CPU."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_every_stage_has_its_traffic_and_only_its_kernels():
    for stage, kernels in bench.STAGE_KERNELS.items():
        traffic, figs = bench.ncu_figures(stage)
        if stage != "upload":  # k_prep runs for batches only
            assert isinstance(traffic, int) and traffic > 0, stage
        for name, per in figs.items():
            assert per, (stage, name)
            for k, v in per.items():
                assert k.split("<")[0] in kernels, (stage, name, k)
                assert isinstance(v, (int, float)), (stage, name, k)
        json.dumps(figs)


def test_traversal_and_narrow_figures():
    _, tr = bench.ncu_figures("traverse")
    assert set(tr["threads_per_warp_instruction"]) == {"k_traverse_wave<0>", "k_traverse_wave<1>"}
    assert all(0 < v <= 32 for v in tr["threads_per_warp_instruction"].values())
    assert set(tr["l2_hit_pct"]) == {"k_traverse_wave<0>", "k_traverse_wave<1>"}
    _, nw = bench.ncu_figures("narrow")
    for key in ("fp64_pipe_active_pct", "fp32_pipe_active_pct"):
        assert {"k_narrow_signs", "k_narrow_hits"} <= set(nw[key])
        assert all(0 <= v <= 100 for v in nw[key].values())
