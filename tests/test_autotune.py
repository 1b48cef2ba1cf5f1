"""The autotuner's selection and cache logic, and the C library's tile
registry (host code only: no kernel runs here)."""

import json

import pytest

from mbem_gb300 import autotune as at


@pytest.fixture(autouse=True)
def _reset():
    yield
    for fam in at.FAMILIES:
        at.select(fam, 0)


def test_registry_counts_and_descriptions():
    for fam in at.FAMILIES:
        n = at.count(fam)
        assert n >= 4
        descs = [at.describe(fam, c) for c in range(n)]
        assert len(set(descs)) == n                  # every configuration is distinct
        assert at.current(fam) == 0
    assert at.describe("mixed_matvec", 0) == "rows=16 ch=1024 stages=3"
    assert at.describe("gemm_split", 0) == "splits=model"
    with pytest.raises(ValueError):
        at.select("mixed_matvec", at.count("mixed_matvec"))
    with pytest.raises(ValueError):
        at.count("no_such_family")


def test_tuner_selects_fastest_and_reuses_cache(tmp_path):
    fam = "bf16_matvec"
    n = at.count(fam)
    fake = [5.0, 3.0, 4.0, 3.0, 9.0, 7.0, 8.0, 6.0][:n]
    timed = []

    def timer(run):
        run()
        timed.append(at.current(fam))
        return fake[at.current(fam)]

    path = tmp_path / "tune.json"
    t = at.Autotuner(cache_path=str(path), timer=timer, device="fake-gpu")
    runs = []
    r = t.tune(fam, "n=99", lambda: runs.append(1))
    assert r.best == 1 and not r.cached          # ties go to the lower configuration
    assert at.current(fam) == 1
    assert timed == list(range(n)) and len(runs) == n
    data = json.loads(path.read_text())
    assert data["fake-gpu|bf16_matvec|n=99"]["best"] == 1

    at.select(fam, 0)

    def no_timer(run):
        raise AssertionError("a cached workload is not timed again")
    t2 = at.Autotuner(cache_path=str(path), timer=no_timer, device="fake-gpu")
    r2 = t2.tune(fam, "n=99", lambda: None)
    assert r2.cached and r2.best == 1 and at.current(fam) == 1
    # another workload key or device is timed afresh
    t3 = at.Autotuner(cache_path=str(path), timer=timer, device="other-gpu")
    assert not t3.tune(fam, "n=99", lambda: None).cached


def test_in_process_cache_writes_no_file(tmp_path):
    t = at.Autotuner(cache_path="", timer=lambda run: 1.0, device="fake-gpu")
    t.tune("gemm_split", "k=1", lambda: None)
    assert list(tmp_path.iterdir()) == []
