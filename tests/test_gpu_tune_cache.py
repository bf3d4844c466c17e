"""The radius-pipeline autotuner caches its timings per device, box size and
batch size, and a later context reuses them instead of timing again."""
import pytest

pytestmark = pytest.mark.gpu


def test_tuning_is_cached_and_reused(hii, tmp_path, monkeypatch):
    cache = tmp_path / "tune.jsonl"
    monkeypatch.setenv("SF21_TUNE_CACHE", str(cache))
    monkeypatch.delenv("SF21_RETUNE", raising=False)
    fb = hii.FilterBank(128, 100.0, 0.7, [(30.0, 25.0, 30)])
    path1, ms1 = fb.path()
    fb.close()
    lines = cache.read_text().splitlines()
    assert len(lines) == 1 and "|N=128|" in lines[0]
    fb = hii.FilterBank(128, 100.0, 0.7, [(30.0, 25.0, 30)])
    path2, ms2 = fb.path()
    fb.close()
    assert path2 == path1
    assert [ms2[p] for p in sorted(ms2)] == pytest.approx([ms1[p] for p in sorted(ms1)], rel=1e-5)
    assert len(cache.read_text().splitlines()) == 1  # reused, not appended
    monkeypatch.setenv("SF21_RETUNE", "1")
    fb = hii.FilterBank(128, 100.0, 0.7, [(30.0, 25.0, 30)])
    fb.close()
    assert len(cache.read_text().splitlines()) == 2  # timed again and stored
