"""The autotune cache file (solrt_tune_cache_lookup / _store): host-only,
so these run without a GPU. The GPU side (solrt_batch_autotune_cached:
a miss times and stores, a hit re-plans without timing) is in
test_gpu_batch.py."""
import pytest


def test_store_lookup_replace(solrt, tmp_path):
    api = solrt.api
    path = str(tmp_path / "tune.jsonl")
    assert api.tune_cache_lookup(path, "gpu=X|h=1") is None          # no file yet
    api.tune_cache_store(path, "gpu=X|h=1", 128, 32, 0, 12.5)
    api.tune_cache_store(path, "gpu=X|h=2", 256, 16, 1 << 20, 3.0)
    assert api.tune_cache_lookup(path, "gpu=X|h=1") == dict(block_size=128, smem_stack=32, pass_paths=0,
                                                            best_ms=pytest.approx(12.5))
    api.tune_cache_store(path, "gpu=X|h=1", 64, 16, 4096, 9.0)       # replaced in place
    assert api.tune_cache_lookup(path, "gpu=X|h=1")["block_size"] == 64
    assert api.tune_cache_lookup(path, "gpu=X|h=2")["pass_paths"] == 1 << 20
    assert api.tune_cache_lookup(path, "gpu=Y|h=1") is None
    lines = open(path).read().splitlines()
    assert len(lines) == 2 and all(l.startswith('{"key": ') for l in lines)
    assert not (tmp_path / "tune.jsonl.tmp").exists()


def test_bad_lines_and_shapes_are_skipped(solrt, tmp_path):
    api = solrt.api
    path = tmp_path / "tune.jsonl"
    path.write_text('not json\n'
                    '{"key": "a", "block_size": 96, "smem_stack": 32, "pass_paths": 0}\n'   # no such kernel
                    '{"key": "b", "block_size": 128}\n'                                    # fields missing
                    '{"key": "c", "block_size": 64, "smem_stack": 16, "pass_paths": 7, "best_ms": 1.5}\n')
    assert api.tune_cache_lookup(str(path), "a") is None
    assert api.tune_cache_lookup(str(path), "b") is None
    assert api.tune_cache_lookup(str(path), "c") == dict(block_size=64, smem_stack=16, pass_paths=7,
                                                         best_ms=pytest.approx(1.5))
    api.tune_cache_store(str(path), "d", 128, 32)                    # rewrites with the parsable entries
    assert [l.split('"')[3] for l in path.read_text().splitlines()] == ["c", "d"]


def test_argument_checks(solrt, tmp_path):
    api = solrt.api
    path = str(tmp_path / "tune.jsonl")
    for bad in ('has"quote', "back\\slash", "ctl\nchar", "", "k" * 300):
        with pytest.raises(solrt.SolrtError):
            api.tune_cache_store(path, bad, 128, 32)
    with pytest.raises(solrt.SolrtError):
        api.tune_cache_store(path, "ok", 96, 32)                      # no extend kernel of that shape
    with pytest.raises(solrt.SolrtError):
        api.tune_cache_store(str(tmp_path / "no_dir" / "tune.jsonl"), "ok", 128, 32)
