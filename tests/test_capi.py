"""The C ABI without a GPU: exported symbols, metadata, argument checking,
the .es dump writer, host-side fault injection and the R-style input checks."""
import ctypes
import os
import re

import numpy as np
import pytest

from cudagsea_gb300 import _native as N
from cudagsea_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "gsea103.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gsea_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = N.lib()
    names = header_functions()
    assert len(names) >= 25
    for name in names:
        assert hasattr(L, name), name
    # and the bindings cover the whole header
    assert set(names) == {s[0] for s in N.SIGNATURES}


def test_proxy_header_symbols_exported():
    out = os.popen(f"nm -DC --defined-only {N.LIB_PATH}").read()
    for sym in ("gsea_single_proxy", "gsea_double_proxy", "listCudaDevices_proxy", "getCudaDevice_proxy",
                "setCudaDevice_proxy"):
        assert sym in out, sym


def test_metric_ids_follow_reference_dispatch_order():
    L = N.lib()
    for i, name in enumerate(api.METRICS):
        assert L.gsea_metric_id(name.encode()) == i
        assert L.gsea_metric_name(i).decode() == name
    assert L.gsea_metric_id(b"") == -1
    assert L.gsea_metric_id(b"signal2noise") == -1
    assert L.gsea_metric_name(14) is None


def test_status_strings():
    L = N.lib()
    assert L.gsea_status_string(0) == b"success"
    assert L.gsea_status_string(2) == b"unknown metric"


def _cfg(**kw):
    c = N.Config()
    N.lib().gsea_config_init(ctypes.byref(c))
    c.num_genes, c.num_samples, c.num_sets, c.num_perms = 100, 10, 3, 8
    for k, v in kw.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("field,value,status", [
    ("num_samples", 1, 1), ("num_genes", 0, 1), ("num_sets", 0, 1), ("num_perms", 0, 1),
    ("metric", 14, 2), ("metric", -1, 2), ("precision", 16, 1), ("form", 5, 1), ("perm_offset", -1, 1),
])
def test_plan_create_rejects_bad_config(field, value, status):
    c = _cfg(**{field: value})
    h = ctypes.c_void_p()
    assert N.lib().gsea_plan_create(ctypes.byref(c), ctypes.byref(h)) == status
    assert not h.value
    assert N.lib().gsea_last_error()


def test_config_defaults_follow_reference():
    c = N.Config()
    N.lib().gsea_config_init(ctypes.byref(c))
    assert c.seed == 42 and c.precision == 32 and c.ascending == 0
    assert c.metric == 6  # onepass_signal2noise, the CLI default


def test_injected_allocation_failure(monkeypatch):
    monkeypatch.setenv("GSEA_FAULT", "alloc")
    c = _cfg()
    h = ctypes.c_void_p()
    assert N.lib().gsea_plan_create(ctypes.byref(c), ctypes.byref(h)) == 8
    assert b"injected" in N.lib().gsea_last_error()


def test_es_dump_layout_and_name(tmp_path):
    es = np.arange(12, dtype=np.float32).reshape(3, 4)
    buf = ctypes.create_string_buffer(4096)
    prefix = str(tmp_path / "run")
    N.check(N.lib().gsea_write_es_dump(prefix.encode(), N.ptr(es), 3, 4, 32, buf, 4096))
    path = buf.value.decode()
    assert path == prefix + "_3_4_32.es"
    np.testing.assert_array_equal(np.fromfile(path, np.float32).reshape(3, 4), es)
    es64 = es.astype(np.float64)
    N.check(N.lib().gsea_write_es_dump(prefix.encode(), N.ptr(es64), 3, 4, 64, buf, 4096))
    assert buf.value.decode().endswith("_3_4_64.es")
    assert N.lib().gsea_write_es_dump(b"", N.ptr(es), 3, 4, 32, None, 0) == 1


def _table():
    vals = np.abs(np.random.RandomState(0).normal(8, 2, size=(6, 4)))
    return api.ExpressionTable(vals, [f"g{i}" for i in range(6)], [f"p{i}" for i in range(4)])


@pytest.mark.parametrize("case", ["labels_len", "labels_value", "nan", "no_sets", "empty_set", "rownames"])
def test_GSEA_input_checks_return_false(case, capsys):
    t = _table()
    labels = [0, 0, 1, 1]
    sets = {"a": ["g0", "g1"], "b": ["g2"]}
    if case == "labels_len":
        labels = [0, 1]
    elif case == "labels_value":
        labels = [0, 2, 1, 1]
    elif case == "nan":
        t.values[1, 1] = np.nan
    elif case == "no_sets":
        sets = {}
    elif case == "empty_set":
        sets = {"a": []}
    elif case == "rownames":
        t = api.ExpressionTable(t.values, t.genes[:-1], t.patients)
    assert api.GSEA(t, labels, sets, 10, "twopass_signal2noise") is False
    assert "INVALID DATA" in capsys.readouterr().out


def test_no_cpu_fallback_without_gpu():
    n = ctypes.c_int(0)
    if N.lib().gsea_device_count(ctypes.byref(n)) == 0 and n.value > 0:
        pytest.skip("a GPU is present")
    t = _table()
    with pytest.raises(N.GseaError) as e:
        api.GSEA(t, [0, 0, 1, 1], {"a": ["g0", "g1"]}, 10, "twopass_signal2noise")
    assert e.value.status in (3, 5)


def test_new_entry_points_check_arguments_without_a_gpu():
    """Host-side validation of the batch, set-mapping, tuning and allocator
    entry points (no device touched)."""
    L = N.lib()
    cfgs = (N.Config * 2)()
    for c in cfgs:
        L.gsea_config_init(ctypes.byref(c))
        c.num_genes, c.num_samples, c.num_sets, c.num_perms = 100, 10, 3, 5
    cfgs[1].precision = 64
    h = ctypes.c_void_p()
    assert L.gsea_batch_create(2, cfgs, 0, ctypes.byref(h)) == 1       # mixed precision
    cfgs[1].precision = 32
    cfgs[1].num_genes = 70000
    assert L.gsea_batch_create(2, cfgs, 0, ctypes.byref(h)) == 7       # G > 65,536: unsupported
    assert L.gsea_batch_create(0, cfgs, 0, ctypes.byref(h)) == 1
    assert L.gsea_batch_execute(None, None) == 1
    # set mapping: bad offsets are rejected before any device work
    genes = (ctypes.c_char_p * 2)(b"a", b"b")
    mem = (ctypes.c_char_p * 2)(b"a", b"x")
    off = np.array([0, 2, 1], np.int64)
    out = np.empty(3, np.int64)
    assert L.gsea_map_sets(2, genes, 2, N.ptr(off), mem, N.ptr(out), None, 0, None) == 9
    assert L.gsea_map_sets(0, genes, 0, None, None, N.ptr(out), None, 0, None) == 1
    # tuning / adaptive defaults
    t = N.Tuning()
    L.gsea_tuning_init(ctypes.byref(t))
    assert (t.metric_pb, t.chosen_tile, t.sort_variant, t.es_warps, t.es_stage) == (0, 0, 0, 0, -1)
    assert L.gsea_plan_set_tuning(None, ctypes.byref(t)) == 1
    ap = N.AdaptiveParams()
    L.gsea_adaptive_params_init(ctypes.byref(ap))
    assert ap.pilot_perms == 1000 and ap.growth == 2.0 and ap.z == 3.0 and ap.q_call == 0.25
    assert ap.q_margin == 1.5
    assert L.gsea_fdr_lower_bound(None, 1, 1, None, 1, None, 0.0, 32, None, None, None) == 1
    assert L.gsea_plan_execute_adaptive(None, None, ctypes.byref(ap), None, None) == 1
    assert L.gsea_model_train(None, None, None, 0, 1, 1, ctypes.c_float(1e-3), None) == 1
