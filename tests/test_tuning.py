"""Autotuner host logic: candidate radix plans and the on-disk cache (CPU)."""

import math

import pytest

from pyturb_gb300 import tuning


@pytest.mark.parametrize("n", [384, 96, 768, 1449, 37, 1000, 4096 * 2, 12])
def test_radix_plans_factor_n(n):
    plans = tuning.radix_plans(n)
    assert plans
    for p in plans:
        assert math.prod(p) == n and all(r >= 2 for r in p)
    assert len(set(plans)) == len(plans)


def test_cache_round_trip(tmp_path, monkeypatch):
    monkeypatch.setenv("PYTURB_GB300_TUNE_CACHE", str(tmp_path / "sub" / "tune.json"))
    tuning._store("dev|k", [8, 8, 2, 3])
    tuning._store("dev|b", 3)
    data = tuning._load()
    assert data["dev|k"] == [8, 8, 2, 3] and data["dev|b"] == 3


def test_unreadable_cache_is_empty(tmp_path, monkeypatch):
    p = tmp_path / "tune.json"
    p.write_text("not json")
    monkeypatch.setenv("PYTURB_GB300_TUNE_CACHE", str(p))
    assert tuning._load() == {}
