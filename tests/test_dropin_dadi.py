"""dadi's own model code through the drop-in boundary (no GPU): after
dadi_gb300.install() and dadi.cuda_enabled(True), dadi's make_extrap_func
over Demographics2D.IM / split_mig, and its one_pop, two_pops, three_pops,
four_pops and five_pops (temporal, and constant with enable_cuda_cached),
reach dadi_gb300's drivers and give dadi's own results and Demes records
(tests/dropin_dadi.py runs them in a subprocess with the kernel launches
replaced by the oracle; dadi is built from the reference tree as
tests/golden/make_golden.py builds it).  Skipped where the reference tree is
absent."""
import json
import os
import subprocess
import sys
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference():
    sys.path.insert(0, ROOT)
    import __graft_entry__
    return __graft_entry__.REFERENCE


def test_dadi_through_the_dropin():
    ref = _reference()
    if not os.path.isdir(os.path.join(ref, "dadi")):
        pytest.skip("reference tree absent")
    build = os.path.join(tempfile.gettempdir(), "dadi_ref")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "dropin_dadi.py"), ref,
                        build], capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert out["cuda_module"] == "dadi_gb300.cuda"
    for name, c in out["cases"].items():
        assert c["through_dropin"], name
        if c["exact_expected"]:
            assert c["bitwise"] and c["records_equal"] is True, (name, c)
        else:
            # dadi's CPU path takes its constant-parameter loop, dadi's CUDA
            # path the temporal one (dadi/Integration.py:214-216, 318-345)
            assert c["max_rel"] < 1e-9, (name, c)
            got, ref_types = c["records_equal"]
            assert got[:len(ref_types)] == ref_types and got[-1] == "IntegrationNonConst"
