"""Host logic of the engine autotuner (no GPU): the search over a knob grid,
the tie rule that keeps the defaults, and applying a stored table only to
graphs of the size it was tuned on."""
import numpy as np

from wedge_gb300 import autotune as A
from wedge_gb300 import engine as W

DEFAULTS = {"hub_bytes": 65536, "probe_edges": 16, "sssp_tile": 512, "sssp_narrow": 1}  # graphs of 2^23+ in-edges


class FakeGraph:
    """a handle whose run time is a function of its knobs"""

    def __init__(self, cost):
        self.cost = cost
        self.set = {}
        self.calls = []

    def set_knob(self, k, v):
        self.calls.append((k, v))
        if v is None:
            self.set.pop(k, None)
        else:
            self.set[k] = v

    def knob(self, k):
        return self.set.get(k, DEFAULTS[k])

    def run(self, app, params):
        return {"running_ms": self.cost({k: self.knob(k) for k in DEFAULTS})}


def test_tune_engine_finds_the_fastest_and_restores_defaults():
    g = FakeGraph(lambda k: 10.0 + abs(k["hub_bytes"] - 32768) / 32768 + abs(k["probe_edges"] - 32) / 16)
    default, best, results = A.tune_engine(g, W.APP_BFS, None, A.ENGINE_SPACE["bfs"], reps=3, log=lambda *_: None)
    assert len(results) == len(A.ENGINE_SPACE["bfs"]["hub_bytes"]) * len(A.ENGINE_SPACE["bfs"]["probe_edges"])
    assert (best["hub_bytes"], best["probe_edges"]) == (32768, 32)
    assert best["ms"] == min(r["ms"] for r in results) < default["ms"]
    assert g.set == {}  # every knob back to its default


def test_tune_engine_keeps_the_defaults_on_a_tie():
    g = FakeGraph(lambda k: 5.0)
    default, best, _ = A.tune_engine(g, W.APP_SSSP, None, A.ENGINE_SPACE["sssp"], reps=2, log=lambda *_: None)
    assert best is default
    assert {k: best[k] for k in ("hub_bytes", "sssp_tile", "sssp_narrow")} == {"hub_bytes": 65536, "sssp_tile": 512,
                                                                              "sssp_narrow": 1}


def test_apply_engine_tuning_only_on_matching_graphs():
    table = {"scale": 26, "edge_factor": 16,
             "apps": {"sssp": {"best": {"hub_bytes": 32768, "sssp_tile": 512, "sssp_narrow": 1, "ms": 1.0}}}}
    g = FakeGraph(lambda k: 1.0)
    assert A.apply_engine_tuning(g, "sssp", 24, 16, table) == {}
    assert A.apply_engine_tuning(g, "bfs", 26, 16, table) == {}
    assert g.calls == []
    got = A.apply_engine_tuning(g, "sssp", 26, 16, table)
    assert got == {"hub_bytes": 32768, "sssp_tile": 512, "sssp_narrow": 1}
    assert g.set == got


def test_knob_names_match_the_header():
    text = open(W.__file__.replace("wedge_gb300/engine.py", "include/wedge_cuda.h")).read()
    for name, k in W.KNOB_NAMES.items():
        assert f"WEDGE_KNOB_{name.upper()} = {k}," in text
    assert W.KNOB_DEFAULT == np.iinfo(np.uint64).max
