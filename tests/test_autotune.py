"""Selection logic of the launch-shape / re-sort autotuner on fake timings (no GPU)."""
import numpy as np

from diffskill_gb300 import autotune as at


def test_pick_keeps_the_current_choice_within_the_margin():
    times = {7: [10.0, 10.1, 9.9], 6: [9.95, 9.96, 9.97], 8: [12.0, 12.0, 12.0]}
    assert at.pick(times, [7, 6, 8], margin=0.01) == 7      # 6 is faster by 0.4 %: noise
    assert at.pick(times, [7, 6, 8], margin=0.001) == 6     # a tighter margin lets it win
    times[8] = [8.0, 8.1, 30.0]                             # the median ignores one outlier
    assert at.pick(times, [7, 6, 8], margin=0.01) == 8


def test_coordinate_descent_finds_each_fields_optimum():
    best = {"p2g_ctas": 8, "g2p_adj_ctas": 5, "p2g_adj_ctas": 5, "grid_ctas_per_sm": 32, "g2p_ctas": 10,
            "grid_op_adj_ctas": 6}
    rng = np.random.default_rng(0)
    calls = []

    def measure(shapes):
        calls.append(dict(shapes))
        # each kernel's time depends on its own field only (+ 0.2 % noise)
        def t(f, base):
            return base * (1 + 0.05 * abs(shapes[f] - best[f])) * (1 + 0.002 * rng.standard_normal())
        return {"p2g": t("p2g_ctas", 100.0), "g2p_adj": t("g2p_adj_ctas", 120.0),
                "p2g_adj": t("p2g_adj_ctas", 110.0), "grid_op": t("grid_ctas_per_sm", 10.0),
                "grid_op_adj": t("grid_ctas_per_sm", 25.0) * t("grid_op_adj_ctas", 1.0),
                "g2p": t("g2p_ctas", 50.0), "clear": 9.0}

    start = at.Tuning().shapes()
    shapes, seen = at.coordinate_descent(measure, start, reps=3, margin=0.01)
    assert shapes == best
    assert set(seen) == set(at.CANDIDATES)
    n_cand = sum(len(c) for c in at.CANDIDATES.values())
    assert len(calls) == 3 * n_cand


def test_coordinate_descent_leaves_defaults_when_nothing_is_faster():
    shapes, _ = at.coordinate_descent(lambda s: {"p2g": 1.0, "g2p_adj": 1.0, "p2g_adj": 1.0, "grid_op": 1.0},
                                      at.Tuning().shapes(), reps=2)
    assert shapes == at.Tuning().shapes()


def test_resort_candidates_respect_the_checkpoint_interval_and_horizon():
    c = at.resort_candidates(50, 1, 1000)
    assert c == [50, 100, 250, 25, 10, 0]
    c = at.resort_candidates(50, 10, 1000)
    assert all(r % 10 == 0 for r in c) and c[0] == 50 and c[-1] == 0 and 30 in c
    c = at.resort_candidates(50, 10, 100)  # a two-action horizon: one interior boundary at most
    assert c == [50, 30, 10, 0]


def test_tuning_cache_round_trip(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("DIFFSKILL_GB300_TUNE_CACHE", str(path))
    t = at.Tuning(p2g_ctas=8, resort_every=100, measured={"p2g_ctas": {"7": 1.0, "8": 0.9}})
    at._store_cache(at._cache_path(), "key", t)
    back = at.Tuning(**at._load_cache(at._cache_path())["key"])
    assert back == t
