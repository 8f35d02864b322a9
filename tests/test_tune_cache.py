"""The batched mat-vec autotuner's cache (richmol_gb300.tune), on the host: a
choice is timed once per operator shape and vector-block count, stored in the
JSON file and read back without timing; other shapes or block counts are
tuned afresh; a damaged file is ignored. CPU only (a fake timer)."""
import json
from types import SimpleNamespace

import numpy as np

from richmol_gb300 import tune

KINDS = ["tensor", "tensor_tmem", "fp32"]


def _plan(dm=(1, 3, 5), nterm=7):
    a = dict(out_dm=np.array(dm, np.int32), out_dk=np.ones(len(dm), np.int32), t_out=np.arange(nterm, dtype=np.int32))
    return SimpleNamespace(tables=SimpleNamespace(arrays=a), dim_out=int(sum(dm)), nterm=nterm)


class FakeTimer:
    def __init__(self, ms):
        self.ms, self.calls = ms, 0

    def __call__(self, run, kinds, reps):
        self.calls += 1
        return {k: self.ms[k] for k in kinds}


def test_choice_is_timed_once_then_read_from_the_file(tmp_path):
    path = str(tmp_path / "tune.json")
    timer = FakeTimer({"tensor": 3.0, "tensor_tmem": 1.5, "fp32": 4.0})
    kind, ms, cached = tune.choose(_plan(), 4096, KINDS, None, "GB300", path=path, timer=timer)
    assert (kind, cached, timer.calls) == ("tensor_tmem", False, 1)
    entry = json.load(open(path))
    assert list(entry.values())[0]["kind"] == "tensor_tmem"
    # the same shape and vector blocks: from the file, nothing timed
    kind2, ms2, cached2 = tune.choose(_plan(), 4000, KINDS, None, "GB300", path=path, timer=timer)
    assert (kind2, cached2, timer.calls) == ("tensor_tmem", True, 1)
    assert ms2["fp32"] == 4.0


def test_other_shapes_and_vector_blocks_are_tuned_afresh(tmp_path):
    path = str(tmp_path / "tune.json")
    timer = FakeTimer({"tensor": 1.0, "tensor_tmem": 2.0, "fp32": 3.0})
    tune.choose(_plan(), 4096, KINDS, None, "GB300", path=path, timer=timer)
    tune.choose(_plan(), 512, KINDS, None, "GB300", path=path, timer=timer)          # other vector blocks
    tune.choose(_plan(dm=(1, 3, 7)), 4096, KINDS, None, "GB300", path=path, timer=timer)  # other slabs
    tune.choose(_plan(), 4096, KINDS, None, "other GPU", path=path, timer=timer)     # other device
    assert timer.calls == 4 and len(json.load(open(path))) == 4


def test_damaged_cache_file_is_ignored_and_replaced(tmp_path):
    path = tmp_path / "tune.json"
    path.write_text("{not json")
    timer = FakeTimer({"tensor": 2.0, "tensor_tmem": 2.5, "fp32": 1.0})
    kind, _, cached = tune.choose(_plan(), 128, KINDS, None, "GB300", path=str(path), timer=timer)
    assert (kind, cached) == ("fp32", False)
    assert list(json.load(open(path)).values())[0]["kind"] == "fp32"


def test_cache_path_from_environment(tmp_path, monkeypatch):
    monkeypatch.setenv(tune.CACHE_ENV, str(tmp_path / "x.json"))
    assert tune.cache_path() == str(tmp_path / "x.json")
