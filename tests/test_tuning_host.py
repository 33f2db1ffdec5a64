"""The table of kernel parameters by system size (sep_gpu_set_tuning,
include/sepgpu.h): host-side checks that need no device."""
import ctypes as C

import pytest

from seplib_gb300 import Tuning, tune


@pytest.fixture
def saved(lib):
    old = Tuning()
    lib.sep_gpu_get_tuning(C.byref(old))
    yield lib
    assert lib.sep_gpu_set_tuning(C.byref(old)) == 0


def test_default_table(saved):
    cur = tune.current(saved)
    assert cur[-1]["nmax"] is None
    assert all(c["team"] in (1, 2) and c["groups"] in (1, 2) and 1.0 <= c["cellf"] <= 2.0 for c in cur)


def test_set_get_roundtrip(saved):
    chosen = [(2, 1, 1.2), (1, 2, 1.0), (2, 2, 1.2)]
    tune.apply(saved, [1024, 8192], chosen)
    cur = tune.current(saved)
    assert [c["nmax"] for c in cur] == [1024, 8192, None]
    assert [(c["team"], c["groups"], c["cellf"]) for c in cur] == chosen


@pytest.mark.parametrize("bad", [
    dict(team=3), dict(team=0), dict(groups=4), dict(cellf=0.9), dict(cellf=2.5),
    dict(cellf=float("nan")), dict(order=True), dict(nclass=0), dict(nclass=9)])
def test_rejected_tables(saved, bad):
    before = tune.current(saved)
    t = tune.table([1024, 8192], [(1, 2, 1.0)] * 3)
    if "team" in bad:
        t.team[1] = bad["team"]
    if "groups" in bad:
        t.groups[0] = bad["groups"]
    if "cellf" in bad:
        t.cellf[2] = bad["cellf"]
    if "order" in bad:
        t.nmax[1] = 512
    if "nclass" in bad:
        t.nclass = bad["nclass"]
    assert saved.sep_gpu_set_tuning(C.byref(t)) == -1
    assert tune.current(saved) == before                      # a rejected table changes nothing
    with pytest.raises(ValueError):
        tune.apply(saved, [1024], [(5, 1, 1.0), (1, 1, 1.0)])


def test_driver_words():
    words = tune.as_args([1024, 8192], [(1, 2, 1.0), (2, 1, 1.2), (2, 2, 1.0)])
    assert words == ["3", "1024", "1", "2", "1.0", "8192", "2", "1", "1.2", "0", "2", "2", "1.0"]


CHOSEN = [(2, 2, 1.0), (1, 2, 1.2), (2, 1, 1.0), (1, 1, 1.0), (2, 2, 1.2), (1, 1, 1.2), (2, 1, 1.2),
          (1, 2, 1.0)]


def test_cache_roundtrip(saved, tmp_path, monkeypatch):
    """load_or_tune times once, writes the table next to the library (here a
    temporary path) and later calls load it for the same GPU and build."""
    calls = []

    def fake_tune(lib, **kw):
        calls.append(kw)
        chosen = CHOSEN[:len(tune.CLASSES) + 1]
        tune.apply(lib, list(tune.CLASSES), chosen)
        return dict(classes=list(tune.CLASSES), chosen=[list(c) for c in chosen], trials=[], seconds=0.0)

    monkeypatch.setattr(tune, "tune", fake_tune)
    path = str(tmp_path / "tuning.json")
    rec = tune.load_or_tune(saved, path=path)
    assert rec["source"] == "tuned" and len(calls) == 1
    tune.apply(saved, [], [(1, 2, 1.0)])                     # something else in between
    rec2 = tune.load_or_tune(saved, path=path)
    assert rec2["source"] == "cache" and len(calls) == 1
    cur = tune.current(saved)
    assert [(c["team"], c["groups"], c["cellf"]) for c in cur] == CHOSEN[:len(tune.CLASSES) + 1]
    # a different build (key) is timed again
    import json
    with open(path) as fh:
        d = json.load(fh)
    d["key"] = "another|0|0"
    with open(path, "w") as fh:
        json.dump(d, fh)
    rec3 = tune.load_or_tune(saved, path=path)
    assert rec3["source"] == "tuned" and len(calls) == 2
