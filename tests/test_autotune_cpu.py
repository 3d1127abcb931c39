"""The tuning cache's host logic (flint_gb300.autotune): where the file lives,
atomic stores, unreadable files read as empty, and how a stored entry is put
into effect on a handle."""
import os

from flint_gb300 import autotune


def test_cache_path_precedence(tmp_path, monkeypatch):
    monkeypatch.delenv("FLINT_TUNING_CACHE", raising=False)
    assert autotune.cache_path() == autotune.DEFAULT_CACHE
    monkeypatch.setenv("FLINT_TUNING_CACHE", str(tmp_path / "env.json"))
    assert autotune.cache_path() == str(tmp_path / "env.json")
    assert autotune.cache_path(str(tmp_path / "arg.json")) == str(tmp_path / "arg.json")


def test_store_and_load(tmp_path):
    p = str(tmp_path / "sub" / "tuning.json")
    assert autotune._load(p) == {}                     # missing file
    data = {"k1": {"reactor_layout": 2, "wdot_threads": 128}}
    autotune._store(p, data)
    assert autotune._load(p) == data
    assert [f for f in os.listdir(os.path.dirname(p)) if f.endswith(".tmp")] == []   # replaced atomically
    with open(p, "w") as f:
        f.write("{not json")
    assert autotune._load(p) == {}                     # unreadable: retuned, not fatal


class FakeChem:
    def __init__(self):
        self.calls = []

    def set_tuning(self, layout, wdot_threads, jac_threads):
        self.calls.append(("set_tuning", layout, wdot_threads, jac_threads))

    def use_generated(self, on, jac=False):
        self.calls.append(("use_generated", on, jac))


def test_apply_puts_the_entry_into_effect():
    c = FakeChem()
    autotune.apply(c, {"reactor_layout": 3, "wdot_threads": 64, "jac_threads": 256,
                       "wdot_kernel": "generated", "jac_kernel": "data-driven"})
    assert c.calls == [("set_tuning", 3, 64, 256), ("use_generated", True, False)]
    c = FakeChem()
    autotune.apply(c, {})                              # an empty entry restores the defaults
    assert c.calls == [("set_tuning", 0, 0, 0), ("use_generated", False, False)]
