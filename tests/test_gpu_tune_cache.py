"""The radius-pipeline autotuner (pipeline and radii per spectrum read)
caches its timings per device, box size and batch size, and a later context
reuses them instead of timing again."""
import pytest

pytestmark = pytest.mark.gpu


def test_tuning_is_cached_and_reused(hii, tmp_path, monkeypatch):
    cache = tmp_path / "tune.jsonl"
    monkeypatch.setenv("SF21_TUNE_CACHE", str(cache))
    monkeypatch.delenv("SF21_RETUNE", raising=False)
    fb = hii.FilterBank(128, 100.0, 0.7, [(30.0, 25.0, 30)])
    path1, ms1 = fb.path()
    k1 = fb.batch_radii()
    fb.close()
    assert k1 in (4, 6, 8)
    lines = cache.read_text().splitlines()
    assert len(lines) == 3 and all("|N=128|" in ln for ln in lines)  # batch sizes 8, 6, 4
    assert sorted(ln.split("|K=")[1].split('"')[0] for ln in lines) == ["4", "6", "8"]
    fb = hii.FilterBank(128, 100.0, 0.7, [(30.0, 25.0, 30)])
    path2, ms2 = fb.path()
    assert fb.batch_radii() == k1
    fb.close()
    assert path2 == path1
    assert [ms2[p] for p in sorted(ms2)] == pytest.approx([ms1[p] for p in sorted(ms1)], rel=1e-5)
    assert len(cache.read_text().splitlines()) == 3  # reused, not appended
    fb = hii.FilterBank(128, 100.0, 0.7, [(30.0, 25.0, 30)], kmax=6)  # a fixed batch size: only its timings
    assert fb.batch_radii() == 6
    fb.close()
    assert len(cache.read_text().splitlines()) == 3
    monkeypatch.setenv("SF21_RETUNE", "1")
    fb = hii.FilterBank(128, 100.0, 0.7, [(30.0, 25.0, 30)])
    fb.close()
    assert len(cache.read_text().splitlines()) == 6  # timed again and stored
