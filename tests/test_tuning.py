"""Autotuner: the JSON tuning store (CPU) and the coordinate-descent tuner plus every
threshold setting giving identical products (GPU)."""
import numpy as np
import pytest

import oracle
import opsparse_gb300 as ops
from opsparse_gb300 import gen


def test_tuning_store_roundtrip(tmp_path):
    path = tmp_path / "tuning.json"
    assert ops.tuning_lookup(path, "gpu/x") is None
    ops.tuning_store(path, "gpu/x", [8, 16, 0, 64, 512, 13312])
    ops.tuning_store(path, "gpu/y", [8, 0, 32, 128, 1024, 4096])
    ops.tuning_store(path, "gpu/x", [8, 16, 32, 32, 256, 13312])
    assert ops.tuning_lookup(path, "gpu/x") == [8, 16, 32, 32, 256, 13312]
    assert ops.tuning_lookup(path, "gpu/y") == [8, 0, 32, 128, 1024, 4096]
    import json
    assert json.loads(path.read_text())["gpu/y"][4] == 1024


def test_tuning_record_store_roundtrip(tmp_path):
    """Whole tuning records (thresholds, hash slots, batch plan, warp/CTA split) keep every
    field; a thresholds-only record reads back with the other fields at their defaults, and
    the thresholds of a whole record read back through the thresholds-only lookup."""
    path = tmp_path / "tuning.json"
    rec = {"thresholds": [8, 16, 32, 64, 512, 4096], "hash_slots": 2, "batch_persistent": 0, "batch_warp_max": 256}
    ops.tuning_store_record(path, "gpu/batch", rec)
    ops.tuning_store(path, "gpu/plain", [8, 16, 32, 128, 1024, 13312])
    assert ops.tuning_lookup_record(path, "gpu/batch") == rec
    assert ops.tuning_lookup(path, "gpu/batch") == rec["thresholds"]
    assert ops.tuning_lookup_record(path, "gpu/plain") == {"thresholds": [8, 16, 32, 128, 1024, 13312],
                                                           "hash_slots": 4, "batch_persistent": 1,
                                                           "batch_warp_max": 512}
    assert ops.tuning_lookup_record(path, "gpu/none") is None


@pytest.mark.gpu
def test_every_threshold_setting_gives_the_same_product(cuda):
    a = gen.web_powerlaw(40000, lmax=3000)
    n = 40000
    A = ops.csr_to_device(*a, n, n)
    ref = oracle.spgemm(*a, *a, n)
    for th in ([8, 16, 32, 128, 1024, 13312], [0, 0, 0, 0, 0, 0], [8, 0, 0, 32, 256, 4096], [0, 16, 32, 0, 1024, 0]):
        h = ops.Handle()
        h.set_thresholds(th)
        assert h.get_thresholds() == th
        rpt, col, val = h.spgemm(A, A).to_host()
        assert np.array_equal(col, ref[1]) and np.array_equal(val.view(np.uint64), ref[2].view(np.uint64)), th
        h.close()


@pytest.mark.gpu
def test_autotune_installs_valid_thresholds(cuda):
    rng = np.random.default_rng(2)
    pairs = []
    for b in range(12):
        n = int(np.exp(rng.uniform(np.log(64), np.log(8192))))
        pairs.append((ops.csr_to_device(*gen.erdos_renyi(n, rng.uniform(4, 32), seed=b), n, n),
                      ops.csr_to_device(*gen.erdos_renyi(n, rng.uniform(4, 32), seed=100 + b), n, n)))
    h = ops.Handle()
    best, ms = ops.autotune(h, pairs, reps=1)
    assert len(best) == 6 and ms > 0
    assert h.get_thresholds() == best
    t = h.get_tuning()  # every field the tuner searched holds one of its candidates
    assert t["hash_slots"] in (2, 4) and t["batch_persistent"] in (0, 1) and t["batch_warp_max"] in (128, 256, 512)
    batch = ops.Batch(h, pairs)
    batch.execute(True)
    batch.check()
    single = ops.Handle()
    for i in range(len(pairs)):
        r = batch.result(i)
        s = single.spgemm(*pairs[i]).to_host()
        assert np.array_equal(r[1], s[1]) and np.array_equal(r[2].view(np.uint64), s[2].view(np.uint64))
