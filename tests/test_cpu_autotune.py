"""Host side of the grouped-GEMM autotuner (lofloat_gb300/autotune.py): the
schedule codes it hands to lofgb_gemm_grouped_prepare, the shape signatures
that key its cache, and the cache file's read-modify-write under threads.
The timing itself needs a GPU (tests/test_gpu_grouped_gemm.py)."""
import json
import threading

import pytest

from lofloat_gb300 import autotune


def test_choice_codes():
    assert len(autotune.CHOICES) == len(set(autotune.CHOICES)) == 9
    assert autotune._code("task") == 0 and autotune._code("lpt_snake") == 2
    assert autotune._code("128x128/task") == 0
    assert autotune._code("128x64/lpt") == 16 | 1           # LOFGB_GROUPED_TILE_N64
    assert autotune._code("128x256/lpt_snake") == 32 | 2    # LOFGB_GROUPED_TILE_N256
    for c in autotune.CHOICES:
        code = autotune._code(c)
        assert code & 15 in (0, 1, 2) and code & ~15 in (0, 16, 32)
        assert autotune.TILE_N[c.split("/")[0]] in (64, 128, 256)
    with pytest.raises(KeyError):
        autotune._code("96x96/lpt")
    with pytest.raises(KeyError):
        autotune._code("128x64/zigzag")


def test_signature_buckets_and_order():
    assert [autotune._bucket(v) for v in (1, 2, 3, 4096, 4097)] == [1, 2, 4, 4096, 8192]
    a = autotune.signature([(256, 300, 512, 32), (4096, 257, 1, 16)])
    b = autotune.signature([(4096, 512, 1, 16), (200, 512, 400, 32)])
    assert a == b
    assert json.loads(a) == [[256, 512, 512, 32], [4096, 512, 1, 16]]
    assert autotune.signature([(256, 256, 256, 32)]) != autotune.signature([(256, 256, 256, 64)])
    r = autotune.round_signature([(1000, 3), (5, 0)])
    assert r.startswith("round:") and json.loads(r[6:]) == [[8, 0], [1024, 3]]


def test_cache_round_trip_and_concurrent_writers(tmp_path, monkeypatch):
    path = tmp_path / "sub" / "tune.json"
    monkeypatch.setattr(autotune, "CACHE_PATH", str(path))
    assert autotune._load_cache() == {}
    autotune._store_cache("a", {"schedule": "lpt", "ms": {"lpt": 1.0}})
    assert autotune._load_cache()["a"]["schedule"] == "lpt"
    writers = [threading.Thread(target=autotune._store_cache, args=(f"s{i}", {"schedule": "task"}))
               for i in range(16)]
    for t in writers:
        t.start()
    for t in writers:
        t.join()
    assert set(autotune._load_cache()) == {"a"} | {f"s{i}" for i in range(16)}
    assert not [p for p in path.parent.iterdir() if ".tmp" in p.name]
    path.write_text("{not json")
    assert autotune._load_cache() == {}
