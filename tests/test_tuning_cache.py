"""The launch-shape autotuner's persistent cache (no GPU): a result stored for a
mechanism's content, GPU and options is returned without measuring, and a changed
mechanism file misses."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


class FakeSolution:
    def __init__(self, path, h=12345):
        self._h = h
        self.source = (path, "gas")

    def structure(self):
        return {"K": 10, "R": 29}


def test_cache_hit_and_miss(tmp_path, monkeypatch):
    from cantera_gb300 import tuning
    mech = tmp_path / "m.yaml"
    mech.write_text("phases: []\n")
    cache = tmp_path / "shapes.json"
    monkeypatch.setenv("GBCHEM_TUNING_CACHE", str(cache))
    tuning._cache.clear()
    sol = FakeSolution(str(mech))
    key = "|".join([tuning.mechanism_key(sol), tuning.gpu_key(), "lu64", "w3", "p8192", "t0.001",
                    "r1e-08", "a1e-15"])
    cache.write_text(json.dumps({key: {"pick": {"matrix_placement": 2, "warps_per_block": 8},
                                       "log": [{"seconds": 1e-4}]}}))
    pick, log = tuning.autotune(sol, None, None, None, 1e-3)
    assert pick == {"matrix_placement": 2, "warps_per_block": 8} and log == [{"seconds": 1e-4}]
    # another mechanism content is another key: the tuner would measure (here: fails without
    # arrays, which shows it did not take the stored entry)
    tuning._cache.clear()
    mech.write_text("phases: [x]\n")
    try:
        tuning.autotune(FakeSolution(str(mech), h=999), None, None, None, 1e-3)
        raise AssertionError("expected a measurement attempt")
    except AttributeError:
        pass
    # the Krylov path's shapes are stored under their own key: the dense entry is not taken
    tuning._cache.clear()
    mech.write_text("phases: []\n")
    try:
        tuning.autotune(sol, None, None, None, 1e-3, linear_solver="gmres")
        raise AssertionError("expected a measurement attempt")
    except AttributeError:
        pass
    # an empty setting turns the file off
    monkeypatch.setenv("GBCHEM_TUNING_CACHE", "")
    assert tuning.cache_path() is None
