"""Null-distribution compliance harness on the CPU: the KS distance, the
critical value, the `.es` dump reader and the per-set comparison of the null
columns (permutations 1..P-1), against scipy and hand-made dumps."""
import numpy as np
import pytest

from cudagsea_gb300 import compliance


def test_ks_distance_matches_scipy():
    stats = pytest.importorskip("scipy.stats")
    rng = np.random.default_rng(7)
    for n, m, shift in ((50, 80, 0.0), (400, 400, 0.3), (1000, 37, -0.5)):
        a = rng.normal(size=n)
        b = rng.normal(shift, 1.0, size=m)
        assert compliance.ks_distance(a, b) == pytest.approx(stats.ks_2samp(a, b).statistic, abs=1e-12)


def test_ks_distance_edge_cases():
    a = np.array([0.1, 0.2, np.nan, 0.3])
    assert compliance.ks_distance(a, a) == 0.0
    assert compliance.ks_distance(np.array([np.nan]), np.array([np.nan])) == 0.0
    assert compliance.ks_distance(np.array([1.0]), np.array([np.nan])) == 1.0
    assert compliance.ks_distance(np.array([0.0, 0.0]), np.array([1.0, 1.0])) == 1.0


def test_critical_value():
    n = m = 1000
    c = np.sqrt(-0.5 * np.log(0.005))
    assert compliance.critical_value(n, m) == pytest.approx(c * np.sqrt(2 / 1000))
    assert compliance.critical_value(n, m, alpha=0.05) < compliance.critical_value(n, m)


def test_es_dump_round_trip_and_null_columns(tmp_path):
    rng = np.random.default_rng(3)
    K, P = 4, 257
    es = rng.normal(size=(K, P)).astype(np.float32)
    path = tmp_path / f"run_{K}_{P}_32.es"
    es.tofile(path)
    got = compliance.read_es_dump(str(path))
    assert got.dtype == np.float32 and np.array_equal(got, es)
    # the observed column 0 is not part of the null
    other = es.copy()
    other[:, 0] = 100.0
    assert np.all(compliance.null_distances(es, other) == 0.0)
    shifted = es + np.float32(10.0)
    assert np.all(compliance.null_distances(es, shifted) == 1.0)
    es64 = es.astype(np.float64)
    p64 = tmp_path / f"run_{K}_{P}_64.es"
    es64.tofile(p64)
    assert np.array_equal(compliance.read_es_dump(str(p64)), es64)


def test_es_dump_rejects_bad_names_and_sizes(tmp_path):
    bad = tmp_path / "run.es"
    bad.write_bytes(b"\0" * 16)
    with pytest.raises(ValueError):
        compliance.read_es_dump(str(bad))
    short = tmp_path / "run_2_3_32.es"
    short.write_bytes(b"\0" * 20)  # 5 floats, not 6
    with pytest.raises(ValueError):
        compliance.read_es_dump(str(short))
    with pytest.raises(ValueError):
        compliance.null_distances(np.zeros((2, 5)), np.zeros((3, 5)))
