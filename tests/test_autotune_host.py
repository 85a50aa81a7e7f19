"""Host logic of the tile autotuner's cache (no GPU): keys, lookup and selection."""
import json

from se2dr_fork_gb300 import autotune as A
from se2dr_fork_gb300 import gpu as G
from se2dr_fork_gb300 import host as H
from se2dr_fork_gb300 import spec as S


class FakeSolver:
    """The part of gpu.Solver the cache lookup uses."""

    def __init__(self, setup, precision):
        self.setup, self.precision = setup, G.PRECISIONS[precision]
        self.selected = None

    def tile_configs(self):
        return [(7, 320), (7, 320), (6, 256)]

    def set_tile_config(self, c):
        self.selected = c


def test_apply_selects_the_cached_configuration(tmp_path, monkeypatch):
    monkeypatch.setattr(A, "CACHE", str(tmp_path / "tuning.json"))
    setup = H.Setup(S.explosion64(16, 12, p=4))
    db = {A.key(setup, "fp32_kahan"): {"config": 2}, A.key(setup, "fp32"): {"config": 1}}
    A.save(db)
    assert json.load(open(A.CACHE)) == db
    sol = FakeSolver(setup, "fp32_kahan")
    assert A.apply(sol) == 2 and sol.selected == 2          # precision from the solver
    sol = FakeSolver(setup, "fp32_kahan")
    assert A.apply(sol, "fp32") == 1 and sol.selected == 1  # or given
    other = FakeSolver(H.Setup(S.explosion64(16, 12, p=3)), "fp32_kahan")
    assert A.apply(other) == 0 and other.selected is None   # nothing cached: configuration 0


def test_cached_configuration_outside_the_table_is_ignored(tmp_path, monkeypatch):
    monkeypatch.setattr(A, "CACHE", str(tmp_path / "tuning.json"))
    setup = H.Setup(S.explosion64(16, 12, p=4))
    A.save({A.key(setup, "fp32_kahan"): {"config": 9}})
    sol = FakeSolver(setup, "fp32_kahan")
    assert A.apply(sol) == 0 and sol.selected is None


def test_key_separates_degree_precision_and_size_class():
    a = H.Setup(S.explosion64(16, 12, p=4))
    b = H.Setup(S.explosion64(64, 64, p=4))
    c = H.Setup(S.explosion64(16, 12, p=5))
    keys = {A.key(a, "fp32_kahan"), A.key(b, "fp32_kahan"), A.key(c, "fp32_kahan"), A.key(a, "fp32")}
    assert len(keys) == 4
