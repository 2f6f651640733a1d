"""The engine-settings autotuner's host logic: buckets, keys, the JSON cache and
the choice of the fastest candidate (the timing itself is replaced by a fake)."""

from __future__ import annotations

import json

import pytest

from galaxy_collision_gb300 import autotune


def test_buckets_and_keys():
    assert [autotune.bucket(n) for n in (1, 2, 3, 4, 1023, 1024, 250_000, 4_000_000)] == [0, 1, 1, 2, 9, 10, 17, 21]
    assert autotune.key("GB300", 128, 1_500_000) == "GB300/G128/N2^20"
    with pytest.raises(ValueError):
        autotune.bucket(0)


def test_tune_picks_the_fastest_and_caches_it(tmp_path):
    path = tmp_path / "tune.json"
    times = {(False, 20): 3.0, (True, 20): 2.0, (False, 10): 2.5, (True, 10): 2.0}
    seen = []

    def measure(c):
        seen.append(c)
        return times[(c["phase_launches"], c["sort_every"])]

    e = autotune.tune(64, 300_000, None, None, 0.005, device="dev", measure=measure, path=path)
    assert len(seen) == len(autotune.CANDIDATES)
    # the first of the two fastest as listed
    assert e["settings"] == {"phase_launches": True, "sort_every": 20}
    saved = json.loads(path.read_text())
    assert saved["dev/G64/N2^18"]["settings"] == e["settings"]

    def never(c):
        raise AssertionError("a cached entry must not be re-timed")

    # same bucket (2^18 .. 2^19 - 1): served from the cache
    assert autotune.settings_for(64, 500_000, None, None, 0.005, device="dev", path=path, measure=never) == \
        {"phase_launches": True, "sort_every": 20}
    # another grid or bucket is tuned and added next to it
    autotune.settings_for(128, 2_000_000, None, None, 0.005, device="dev", path=path, measure=measure)
    assert set(json.loads(path.read_text())) == {"dev/G64/N2^18", "dev/G128/N2^20"}


def test_unreadable_cache_is_empty(tmp_path):
    p = tmp_path / "bad.json"
    p.write_text("{not json")
    assert autotune.load(p) == {}
    assert autotune.load(tmp_path / "missing.json") == {}
