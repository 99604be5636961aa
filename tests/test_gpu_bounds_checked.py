"""The bounds-checked build (libgpumesh_gb300_checked.so, GM_BOUNDS_CHECK) on
in-range inputs: the cases of tests/bounds_cases.py run in a child process
that loads the checked library must record no out-of-range index in any
mesh's status word, and must give the ordinary library's results bit for
bit (the checks only compare; an index in range is read unchanged).  No
input here is out of range: the checks exist so that one would be reported
instead of read, and no test plants one on the GPU."""

import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

pytestmark = pytest.mark.gpu


def test_checked_build_matches_and_reports_clean(tmp_path):
    from gpumesh_gb300 import build

    build.build(checked=True)
    import bounds_cases

    plain = bounds_cases.run_cases()
    assert int(plain["checked"]) == 0
    out = tmp_path / "checked.npz"
    env = dict(os.environ, GPUMESH_GB300_LIB="checked")
    r = subprocess.run([sys.executable, os.path.join(HERE, "bounds_cases.py"), str(out)], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    checked = dict(np.load(out, allow_pickle=False))
    assert int(checked["checked"]) == 1
    assert not checked["bounds_words"].any(), checked["bounds_words"]
    assert int(checked["batch_status"]) == 0
    for k, v in plain.items():
        if k in ("checked",):
            continue
        assert np.array_equal(np.asarray(v), checked[k], equal_nan=True), k
