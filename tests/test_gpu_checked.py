"""The checked build (every gathered index of the step kernels and of the
adjoint's reverse kernels range-checked on the device, a bad one setting an
error bit instead of faulting) runs the same steps and the same adjoint as
the product build without raising: the same bits for states and traces, the
same gradients to round-off."""
import json
import os
import subprocess
import sys

import pytest

from swe_fvm_gb300.build import build

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(checked: bool) -> dict:
    env = dict(os.environ, SWE_GB300_CHECKED="1" if checked else "0", PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "checked_run.py")], capture_output=True,
                       text=True, env=env, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_checked_build_matches_the_product_build(gpu):
    build(checked=True)
    a, b = _run(False), _run(True)
    assert not a.pop("checked") and b.pop("checked")
    assert a.pop("library") != b.pop("library")
    ga, gb = a.pop("adjoint_grads"), b.pop("adjoint_grads")
    assert a == b
    for x, y in zip(ga, gb):
        assert x > 0 and abs(x - y) <= 1e-12 * x
