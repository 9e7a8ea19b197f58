"""Host logic of the batched launch's autotune cache (meshlib_gb300.Batch.autotune): lookups reject
stale or damaged entries, and concurrent writers never leave a file that does not parse."""
import json
import multiprocessing as mp

import meshlib_gb300 as M

NAMES = ["4x4x2/128", "4x4x2/256", "8x4x1/128", "8x4x1/256", "2x4x4/128", "2x4x4/256"]


def test_lookup_missing_and_roundtrip(tmp_path):
    path = str(tmp_path / "sub" / "autotune.json")
    assert M._autotune_cache_lookup(path, "k", NAMES) is None
    rec = {"config": 5, "name": NAMES[5], "times_ms": [1.0] * 6}
    M._autotune_cache_store(path, "k", rec)
    assert M._autotune_cache_lookup(path, "k", NAMES) == rec
    M._autotune_cache_store(path, "k2", dict(rec, config=0, name=NAMES[0]))
    assert M._autotune_cache_lookup(path, "k", NAMES) == rec  # other keys are kept
    assert M._autotune_cache_lookup(path, "k2", NAMES)["config"] == 0


def test_stale_and_damaged_entries_are_ignored(tmp_path):
    path = str(tmp_path / "autotune.json")
    M._autotune_cache_store(path, "renamed", {"config": 1, "name": "old-variant"})
    M._autotune_cache_store(path, "range", {"config": 9, "name": "x"})
    M._autotune_cache_store(path, "junk", {"cfg": 1})
    assert M._autotune_cache_lookup(path, "renamed", NAMES) is None
    assert M._autotune_cache_lookup(path, "range", NAMES) is None
    assert M._autotune_cache_lookup(path, "junk", NAMES) is None
    with open(path, "w") as fh:
        fh.write("{not json")
    assert M._autotune_cache_lookup(path, "renamed", NAMES) is None
    M._autotune_cache_store(path, "k", {"config": 2, "name": NAMES[2]})  # a damaged file is replaced
    assert M._autotune_cache_lookup(path, "k", NAMES)["config"] == 2


def _writer(path, w):
    for i in range(40):
        M._autotune_cache_store(path, f"w{w}_{i}", {"config": i % 6, "name": NAMES[i % 6]})


def test_concurrent_writers_leave_a_valid_file(tmp_path):
    path = str(tmp_path / "autotune.json")
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_writer, args=(path, w)) for w in range(4)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    with open(path) as fh:
        cache = json.load(fh)
    # read-modify-write without a lock: keys of interleaved writers may be lost, the file never is
    assert isinstance(cache, dict) and cache
    assert all(M._autotune_cache_lookup(path, k, NAMES) is not None for k in cache)
    assert not [f for f in tmp_path.iterdir() if f.name.startswith(".autotune.")]
