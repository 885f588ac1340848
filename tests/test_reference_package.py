"""The reference's own Python tests, unchanged, through the drop-in (on the CPU).

tests/golden/make_dropin.py imports the reference's `costal` package with `costal._costal` bound to
costal_gb300._costal (device entry points answered by the oracle here, where there is no GPU) and runs
the reference's Python test files under pytest; check mode also re-records every call the package
makes and compares it with the committed record that tests/test_dropin_replay.py replays on a GB300.
It needs the reference checkout (oracle/reference_py.py) and skips without it.
"""

import json
import subprocess
import sys
from pathlib import Path

import pytest

import dropin_trace as T
from oracle import reference_py

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_committed_record_has_no_failed_reference_test():
    doc, _ = T.load()
    rt = doc["meta"]["reference_tests"]
    assert rt["failed"] == [] and rt["pytest_exit"] == 0
    assert len(rt["passed"]) >= 48
    # the only skips are the comparisons with packages this image lacks (igraph, leidenalg)
    for name, reason in rt["skipped"]:
        assert any(p in reason for p in ("igraph", "leidenalg", "pandas")), (name, reason)


def test_reference_python_tests_pass_through_the_drop_in():
    if reference_py.locate() is None:
        pytest.skip("the reference checkout is not on this machine (set COSTAL_REFERENCE)")
    r = subprocess.run([sys.executable, str(GOLDEN / "make_dropin.py"), "--check"], capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-4000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["check"] == "ok" and out["passed"] >= 48
