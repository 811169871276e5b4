"""The gsea103 command line against the reference CLI's RESULT lines."""
import os
import subprocess

import numpy as np
import pytest

from cudagsea_gb300 import broad, build, synthetic
from tests import helpers as H

pytestmark = pytest.mark.gpu

CLI = os.path.join(os.path.dirname(build.LIB), "gsea103")


@pytest.mark.parametrize("prec,order", [("single", "descending"), ("double", "descending"),
                                        ("single", "ascending")])
def test_cli_matches_reference_result_lines(gpu, tmp_path, prec, order):
    d = synthetic.small(num_perms=256)
    gct, cls, gmt = broad.write_dataset(str(tmp_path / "s"), d)
    dump = str(tmp_path / "dump")
    out = subprocess.run([CLI, "-res", gct, "-cls", cls, "-gmx", gmt, "-nperm", "256", "-metric",
                          "twopass_signal2noise", "-precision", prec, "-order", order, "-dump", dump],
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    names, ours = broad.parse_result_lines(out.stdout)
    fname = f"cli_result_{prec}.txt" if order == "descending" else f"cli_result_{order}_{prec}.txt"
    rnames, ref = broad.parse_result_lines(open(os.path.join(H.GOLDEN, fname)).read())
    assert names == rnames
    np.testing.assert_allclose(ours[:, :2], ref[:, :2], atol=1e-5)   # ES, NES
    np.testing.assert_allclose(ours[:, 2:], ref[:, 2:], atol=2.0 / 256)  # NP, FWER
    bits = 64 if prec == "double" else 32
    assert os.path.getsize(f"{dump}_{d.num_sets}_256_{bits}.es") == d.num_sets * 256 * bits // 8


def test_cli_errors(gpu, tmp_path):
    assert subprocess.run([CLI], capture_output=True).returncode == 1
    r = subprocess.run([CLI, "-res", "a", "-cls", "b", "-gmx", "c", "-metric", "nope"], capture_output=True)
    assert r.returncode == 1
    r = subprocess.run([CLI, "-res", "a", "-cls", "b", "-gmx", "c", "-order", "sideways"], capture_output=True)
    assert r.returncode == 18
    r = subprocess.run([CLI, "-res", "a", "-cls", "b", "-gmx", "c", "-cpu"], capture_output=True)
    assert r.returncode == 22
