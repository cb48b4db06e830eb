"""The autotuner's cache (include/fsg.h, fsg_tune_cache_*): host-only functions,
so they run without a GPU.  Entries are stored and found by workload class,
survive a round trip through the cache file, and malformed launches or file
lines are refused."""
import pytest

from fake_spectra_gb300 import _lib


def _key(**kw):
    k = _lib.TuneKey(sms=152, precision=1, compute_tau=1, kernel=1, nbins_b=26, pairs_med_b=18,
                     pairs_p99_b=26, lines_b=15, damp_b=-7)
    for name, v in kw.items():
        setattr(k, name, v)
    return k


@pytest.fixture()
def fresh(tmp_path):
    _lib.tune_cache_file(None)
    _lib.tune_cache_clear()
    yield tmp_path
    _lib.tune_cache_file(None)
    _lib.tune_cache_clear()


def test_store_and_lookup_by_class(fresh):
    assert _lib.tune_cache_lookup(_key()) is None
    _lib.tune_cache_store(_key(), 384, 4, 1, ms_default=10.0, ms_best=9.0, candidates=7,
                          sample_lines=608, records=1)
    e = _lib.tune_cache_lookup(_key())
    assert (e["threads"], e["chunk"], e["persistent"], e["records"]) == (384, 4, 1, 1)
    assert e["ms_default"] == 10.0 and e["ms_best"] == 9.0 and e["candidates"] == 7
    # another class (other nbins bucket, other line) is a miss
    assert _lib.tune_cache_lookup(_key(nbins_b=20)) is None
    assert _lib.tune_cache_lookup(_key(damp_b=-5)) is None


def test_file_round_trip(fresh):
    path = str(fresh / "tune.txt")
    _lib.tune_cache_file(path)
    _lib.tune_cache_store(_key(), 256, 16, 0, 5.0, 4.5, 6, 100)
    _lib.tune_cache_store(_key(compute_tau=0), 512, 32, 1, 2.0, 2.0, 6, 100)
    # a line that does not parse, and one with an invalid launch, are skipped on load
    with open(path, "a") as f:
        f.write("garbage line\n")
        f.write("fsg-tune-v2 152 1 1 1 26 18 26 15 -9 100 4 1 0 7 608 1.0 1.0\n")
        f.write("fsg-tune-v2 152 1 1 1 26 18 26 15 -9 512 4 1 2 7 608 1.0 1.0\n")
    _lib.tune_cache_file(None)
    _lib.tune_cache_clear()
    assert _lib.tune_cache_lookup(_key()) is None
    _lib.tune_cache_file(path)
    e = _lib.tune_cache_lookup(_key())
    assert (e["threads"], e["chunk"], e["persistent"]) == (256, 16, 0)
    e = _lib.tune_cache_lookup(_key(compute_tau=0))
    assert (e["threads"], e["chunk"], e["persistent"]) == (512, 32, 1)
    assert _lib.tune_cache_lookup(_key(damp_b=-9)) is None


@pytest.mark.parametrize("threads,chunk,persistent,records", [
    (100, 8, 1, 0), (512, 0, 1, 0), (512, 33, 1, 0), (2048, 8, 1, 0), (512, 8, 2, 0),
    (512, 8, 1, 2)])
def test_invalid_launch_refused(fresh, threads, chunk, persistent, records):
    with pytest.raises(ValueError):
        _lib.tune_cache_store(_key(), threads, chunk, persistent, records=records)
    assert _lib.tune_cache_lookup(_key()) is None
