"""Host logic of the order evaluation and the anytime report, on the CPU:
the learned / plain ratios of learned_order.summarize and the coverage curve
of anytime_run.coverage_at."""
import math

import numpy as np

from sgfim import anytime_run, learned_order

KEYS = ("t50", "t90", "t95", "n50", "n90", "n95", "total_s", "nodes")


def _rec(scale):
    return {k: scale * (i + 1) for i, k in enumerate(KEYS)}


def test_summarize_ratios_against_plain_order():
    rows = [
        {"seed": 1, "identical": True, "support_desc": _rec(1.0), "learned": _rec(0.5), "support": _rec(0.25)},
        {"seed": 2, "identical": True, "support_desc": _rec(2.0), "learned": _rec(1.6), "support": _rec(1.0)},
    ]
    out = learned_order.summarize(rows)
    assert out["identical_all"] and out["seeds"] == 2
    for k in KEYS:
        assert math.isclose(out[f"{k}_ratio_geomean"], math.sqrt(0.5 * 0.8))
        assert math.isclose(out[f"{k}_ratio_median"], (0.5 + 0.8) / 2)
        assert math.isclose(out[f"canonical_{k}_ratio_geomean"], math.sqrt(0.25 * 0.5))
    rows[1]["identical"] = False
    assert not learned_order.summarize(rows)["identical_all"]


def test_orders_are_compared_at_a_fixed_wave_size():
    assert learned_order.EVAL_WAVE_NODES == 8192


def test_coverage_at_checkpoints():
    t = np.array([2.5, 0.5, 7.0, 1.5])
    cov = anytime_run.coverage_at(t, [1.0, 2.0, 5.0, 10.0, 0.1])
    assert cov == {"1.0": 0.25, "2.0": 0.5, "5.0": 0.75, "10.0": 1.0, "0.1": 0.0}
    # an emission exactly at a checkpoint counts at that checkpoint
    assert anytime_run.coverage_at(np.array([1.0, 3.0]), [1.0])["1.0"] == 0.5
    assert anytime_run.coverage_at(np.zeros(0), [1.0])["1.0"] == 0.0
