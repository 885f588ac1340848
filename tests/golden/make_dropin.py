"""Record what the reference's own Python package asks of `costal._costal` (tests/golden/dropin_*).

    python tests/golden/make_dropin.py           # write tests/golden/dropin_trace.json + dropin_arrays.npz
    python tests/golden/make_dropin.py --check   # re-record and compare with the committed files

Runs only where the reference checkout is (oracle/reference_py.py finds it). It imports the
reference's unchanged `costal` package (python/costal of CosTaL 2.1.0) with `costal._costal` bound to
costal_gb300._costal — the drop-in — whose device entry points are answered by the CPU oracle
(oracle/device_stub.py), because this machine has no GPU. Through that it runs

  * the reference's Python tests (oracle.reference_py.TEST_FILES) under pytest, unchanged; igraph,
    leidenalg and pandas are not installed, so the tests that compare with them skip;
  * `costal.find_communities(X, k=10, leiden="fast", resolution=0.8, seed=0)` and
    `costal.find_communities_multiscale(X, leiden="fast")` on the 20,000 x 32 mixture (the
    reference-runnable configuration), `costal.build_graph` on 100,000 rows of the rare-population
    generator, and `costal.knn(..., 30)` on 40,000 rows of the duplicate-heavy generator;

and records every call the package made into the module. tests/test_dropin_replay.py replays the
record on a GB300 through the real library; tests/test_reference_package.py re-runs this script in
check mode on the CPU.
"""

from __future__ import annotations

import argparse
import json
import sys
import types
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
for p in (ROOT, ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

import numpy as np  # noqa: E402

import dropin_trace as T  # noqa: E402
from oracle import reference_py  # noqa: E402

# End-to-end inputs: (workload generator, rows); None = the workload's full size.
INPUTS = {"mixture": ("mixture_20k", None), "rare": ("rare_400k", 100_000), "dup": ("dense_dup_160k", 40_000)}


class Outcomes:
    """pytest plugin: the outcome of every reference test."""

    def __init__(self):
        self.passed, self.skipped, self.failed = [], [], []

    def pytest_runtest_logreport(self, report):
        name = report.nodeid.split("::", 1)[-1]
        fname = Path(report.nodeid.split("::", 1)[0]).name
        if report.when == "call" and report.passed:
            self.passed.append(f"{fname}::{name}")
        elif report.skipped and report.when in ("setup", "call"):
            reason = report.longrepr[2] if isinstance(report.longrepr, tuple) else str(report.longrepr)
            self.skipped.append([f"{fname}::{name}", reason])
        elif report.failed:
            self.failed.append([f"{fname}::{name}", report.longreprtext[-2000:]])


def record():
    ref = reference_py.locate()
    if ref is None:
        raise SystemExit("the reference checkout was not found (set COSTAL_REFERENCE)")
    from costal_gb300 import _costal as drop_in
    from costal_gb300 import workloads
    from oracle import device_stub

    device_stub.install()
    inputs = {key: workloads.make(name, n)[0] for key, (name, n) in INPUTS.items()}
    known = {T.digest(x): {"workload": name, "n": n if n is not None else len(x)}
             for (name, n), x in zip(INPUTS.values(), inputs.values())}
    from conftest import clustered, scaled_clusters

    rec = T.Recorder(known, {"clustered": clustered, "scaled_clusters": scaled_clusters})
    mod = types.ModuleType("costal._costal")
    mod.__dict__.update({k: v for k, v in vars(drop_in).items() if not k.startswith("__") or k == "__version__"})
    for name in T.FUNCTIONS:
        setattr(mod, name, rec.wrap(name, getattr(drop_in, name)))
    sys.modules["costal._costal"] = mod
    # seed=None draws a Leiden seed from `secrets` (_api.py:_seed64); a seeded stand-in keeps the
    # record reproducible without touching the package
    import random
    import secrets

    draws = random.Random(20241204)
    secrets.randbits = draws.getrandbits
    sys.path.insert(0, str(ref / "python"))
    sys.dont_write_bytecode = True

    import pytest

    outcomes = Outcomes()
    files = [str(ref / "tests" / f) for f in reference_py.TEST_FILES]
    rc = pytest.main([*files, "-q", "-p", "no:cacheprovider", "-o", "addopts=", "-W", "ignore::DeprecationWarning"],
                     plugins=[outcomes])
    n_test_calls = len(rec.calls)

    import costal

    assert sys.modules["costal._api"]._ext is mod, "the reference package did not bind the drop-in"
    finals = {}
    x = inputs["mixture"]
    finals["find_communities_mixture_20k"] = T.digest(
        costal.find_communities(x, k=10, leiden="fast", resolution=0.8, seed=0))
    finals["find_communities_multiscale_mixture_20k"] = T.digest(costal.find_communities_multiscale(x, leiden="fast"))
    finals["build_graph_rare_100k"] = [T.digest(a) for a in costal.build_graph(inputs["rare"], 10)]
    g = costal.knn(inputs["dup"], 30)
    finals["knn_dense_dup_40k_k30"] = [T.digest(g.idx), T.digest(g.cos)]
    meta = {
        "reference": "CosTaL 2.1.0 python/costal (unchanged), costal._costal = costal_gb300._costal",
        "reference_tests": {"files": list(reference_py.TEST_FILES), "pytest_exit": int(rc),
                            "passed": outcomes.passed, "skipped": outcomes.skipped, "failed": outcomes.failed},
        "calls_from_reference_tests": n_test_calls,
        "end_to_end": finals,
    }
    return rec, meta


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--check", action="store_true", help="compare with the committed record instead of writing")
    args = ap.parse_args()
    rec, meta = record()
    if meta["reference_tests"]["failed"]:
        for name, text in meta["reference_tests"]["failed"]:
            print(f"FAILED {name}\n{text}", file=sys.stderr)
        raise SystemExit(1)
    if not args.check:
        rec.save(meta)
        print(f"recorded {len(rec.calls)} calls, {len(rec.arrays)} stored arrays; "
              f"{len(meta['reference_tests']['passed'])} reference tests passed, "
              f"{len(meta['reference_tests']['skipped'])} skipped")
        return
    doc, arrays = T.load()
    fresh = json.loads(json.dumps({"meta": meta, "calls": rec.calls}))
    assert fresh["calls"] == doc["calls"], "the reference package's calls differ from the committed record"
    assert fresh["meta"]["end_to_end"] == doc["meta"]["end_to_end"], "end-to-end answers differ from the record"
    # stored arrays are keyed by their digest (NaN inputs included, which never compare equal)
    assert sorted(arrays) == sorted(rec.arrays) and all(T.digest(arrays[k]) == k[1:] for k in arrays)
    print(json.dumps({"check": "ok", "calls": len(rec.calls), "passed": len(meta["reference_tests"]["passed"]),
                      "skipped": len(meta["reference_tests"]["skipped"])}))


if __name__ == "__main__":
    main()
