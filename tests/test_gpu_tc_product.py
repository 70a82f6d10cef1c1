"""The tensor-core split-precision product itself (mm_tc, dqmc_tc.cuh),
through a one-CTA harness built with nvcc: its error relative to
sum_k |a_ik b_kj| stays below the double-float product's class (1e-13) for
n = 16 .. 256 with rows and columns spanning scales of 2^+-12, untransposed
and transposed, and no mbarrier wait times out."""
import os
import re
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def harness(tmp_path_factory, lib):
    from montecarlo_gb300 import build
    out = str(tmp_path_factory.mktemp("tc") / "tc_product_harness")
    subprocess.run([build.nvcc(), *build.ARCH, "-O3", "-std=c++17", "-o", out,
                    os.path.join(HERE, "tc_product_harness.cu")], check=True,
                   capture_output=True, text=True)
    return out


def test_tc_product_accuracy(harness):
    r = subprocess.run([harness], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = re.findall(r"^(tc\S*|dfx|fp64)\s+(?:TA|TB)?\s*n=\s*(\d+) status=(\d+)\s+err/sum\|ab\| = (\S+)",
                      r.stdout, flags=re.M)
    assert rows
    for name, n, status, err in rows:
        assert int(status) == 0
        if name.startswith("tc"):
            assert float(err) < 1e-13, (name, n, err)
