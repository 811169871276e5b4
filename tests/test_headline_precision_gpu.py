"""The headline workload's accuracy condition: 20,000 genes x 200 samples,
1,000 sets, 1,000 permutations, twopass_signal2noise.  Both tensor-core
forms (the error-free FP32 variance and the FP64 variance finalisation)
against the plain form in FP64, same inputs and permutations:

* FDR < 0.25 calls identical to FP64's;
* every set with |dNES| > 1e-4 tie-explained: each of its moved scores is
  reproduced by the FP64 keys walked in the tensor-core form's own rank
  order (only the order of near-tied genes differs), and its NES with those
  scores put back to FP64 is within 1e-4.

The FP64 run itself is spot-checked against the FP64 oracle (keys bit for
bit, scores to 1e-12)."""
import numpy as np
import pytest

import oracle
from cudagsea_gb300 import precision_check as PC
from cudagsea_gb300 import synthetic
from cudagsea_gb300 import _native as N
from tests import helpers as H

pytestmark = pytest.mark.gpu

METRIC = 8  # twopass_signal2noise


@pytest.fixture(scope="module")
def headline():
    d = synthetic.full()
    ref = PC.run_form(d, METRIC, 64, N.FORM_PLAIN)
    yield d, ref
    ref.close()


def test_fp64_reference_run_matches_oracle(gpu, headline):
    d, ref = headline
    for p in (0, 777):
        k1 = oracle.metric(METRIC, d.exprs.astype(np.float64), d.labels, 1, shift=p, double=True)
        np.testing.assert_array_equal(ref.keys.rows([p])[0].view(np.uint64), k1[0].view(np.uint64))
        sk, o = oracle.sort(k1)
        np.testing.assert_array_equal(ref.order.rows([p])[0], o[0])
        e1 = oracle.es(sk, o, d.set_offsets, d.set_genes)
        assert H.es_close(ref.es[:, p], e1[:, 0], True).all()


@pytest.mark.parametrize("form", [N.FORM_CHOSEN, N.FORM_CHOSEN_FP64], ids=["fp32eft", "fp64var"])
def test_headline_nes_within_1e4_or_tie_explained(gpu, headline, form):
    d, ref = headline
    cur = PC.run_form(d, METRIC, 32, form)
    try:
        rep = PC.compare(d, cur, ref)
    finally:
        cur.close()
    assert rep["fdr_call_diffs"] == 0, rep
    assert rep["all_tie_explained"], rep["exceedances"]
    # the scores that did not move are within the fp32 rounding tolerance
    assert rep["max_abs_dNES"] < 1e-2
