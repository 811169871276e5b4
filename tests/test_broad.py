"""Broad file formats through libgsea103 (no GPU needed): round trips, the
reference's error cases, and the reference CLI's RESULT lines reproduced by
the oracle on the parsed data."""
import os

import numpy as np
import pytest

import oracle
from cudagsea_gb300 import broad, synthetic
from cudagsea_gb300 import _native as N
from tests import helpers as H


def test_round_trip(tmp_path):
    d = synthetic.make(300, 17, 9, 4, seed=3, n_class_b=8, set_min=5, set_max=30)
    gct, cls, gmt = broad.write_dataset(str(tmp_path / "x"), d)
    ds = broad.Dataset(gct, cls, gmt)
    x, labels, off, genes = ds.arrays(32)
    np.testing.assert_array_equal(x, d.exprs)
    np.testing.assert_array_equal(labels, d.labels)
    np.testing.assert_array_equal(off, d.set_offsets)
    np.testing.assert_array_equal(genes, d.set_genes)
    assert ds.gene_symbols() == d.gene_symbols()
    assert ds.set_names() == [f"SET_{k}" for k in range(d.num_sets)]
    x64, *_ = ds.arrays(64)
    np.testing.assert_array_equal(x64.astype(np.float32), d.exprs)


def test_symbols_unknown_and_duplicate_members(tmp_path):
    d = synthetic.make(50, 6, 2, 2, seed=4, n_class_b=3, set_min=5, set_max=8)
    genes = d.gene_symbols()
    p = str(tmp_path / "y")
    broad.write_gct(p + ".gct", d.exprs.T, genes, [f"P{s}" for s in range(6)])
    broad.write_cls(p + ".cls", d.labels, names=("ctrl", "case"))
    broad.write_gmt(p + ".gmt", ["S1", "S2"], [["G3", "  G3 ", "NOPE", "G7"], ["G1"]])
    ds = broad.Dataset(p + ".gct", p + ".cls", p + ".gmt")
    _, labels, off, members = ds.arrays()
    np.testing.assert_array_equal(labels, d.labels)
    assert off.tolist() == [0, 2, 3]
    assert members.tolist() == [3, 7, 1]


@pytest.mark.parametrize("case,msg", [
    ("header", "not a valid gct header"), ("dup", "duplicate symbol"), ("label", "Unknown label"),
    ("classes", "exactly two"), ("missing", "Unable to open"),
])
def test_reference_error_cases(tmp_path, case, msg):
    d = synthetic.make(20, 4, 1, 2, seed=5, n_class_b=2, set_min=3, set_max=5)
    p = str(tmp_path / "z")
    gct, cls, gmt = broad.write_dataset(p, d)
    if case == "header":
        open(gct, "w").write("#1.3\n1\t1\n")
    elif case == "dup":
        lines = open(gct).read().splitlines()
        lines[4] = "G0" + lines[4][lines[4].index("\t"):]
        open(gct, "w").write("\n".join(lines) + "\n")
    elif case == "label":
        open(cls, "w").write("4 2 1\n# A B\nA B C A\n")
    elif case == "classes":
        open(cls, "w").write("4 3 1\n# A B C\nA B C A\n")
    elif case == "missing":
        gct = p + ".nothere"
    with pytest.raises(N.GseaError) as e:
        broad.Dataset(gct, cls, gmt)
    assert e.value.status == 6 and msg in str(e.value)


@pytest.mark.parametrize("prec,order", [("single", "descending"), ("double", "descending"),
                                        ("single", "ascending")])
def test_oracle_reproduces_reference_cli(tmp_path, prec, order):
    """The reference CLI's RESULT lines (golden) from the oracle on our parse;
    `-order ascending` sorts the keys ascending and keeps the labels."""
    d = synthetic.small(num_perms=256)
    gct, cls, gmt = broad.write_dataset(str(tmp_path / "s"), d)
    ds = broad.Dataset(gct, cls, gmt)
    double = prec == "double"
    x, labels, off, genes = ds.arrays(64 if double else 32)
    es, st = oracle.gsea(8, x, labels, off, genes, 256, double=double, ascending=order == "ascending")
    fname = f"cli_result_{prec}.txt" if order == "descending" else f"cli_result_{order}_{prec}.txt"
    names, ref = broad.parse_result_lines(open(os.path.join(H.GOLDEN, fname)).read())
    assert names == ds.set_names()
    K = d.num_sets
    ours = np.stack([st[:K], st[K:2 * K], st[2 * K:3 * K], st[3 * K:4 * K]], axis=1)
    np.testing.assert_allclose(ours[:, :2], ref[:, :2], atol=2e-6)   # printed with 6 decimals
    np.testing.assert_allclose(ours[:, 2:], ref[:, 2:], atol=1.5e-6)
