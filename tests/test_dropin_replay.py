"""The reference's own Python package on the GB300: its recorded calls into `costal._costal`, replayed.

tests/golden/make_dropin.py ran the reference's unchanged `costal` package (CosTaL 2.1.0's
python/costal) with `costal._costal` bound to costal_gb300._costal: the reference's Python tests
(test_smoke, test_knn, test_leiden_native, test_leiden_api, test_multiscale) and
`costal.find_communities(..., leiden="fast", resolution=0.8, seed=0)`,
`costal.find_communities_multiscale` (the Leiden ensemble, `_leiden_many`), `costal.build_graph` and
`costal.knn(..., 30)` on the benchmark generators. Every call the package made into the module was
recorded with the answer of the CPU oracle. Here the same calls, with the same arguments and keywords
(`_api.py:203,257,321,462-465`, `_leiden.py:111`, `_multiscale.py:170-175` of the reference), run in
order through the real library on the GPU; each array a call returned is fed to the later calls that
took it, as the package would, and every answer must be the recorded one bit for bit (errors: the
same exception type and the message text the reference's tests match).

The second pass repeats everything with the module's default backend switched to the certified
split-BF16 tensor-core path (DEFAULT_MATMUL = "bf16", what COSTAL_GB300_MATMUL=bf16 does for an
unchanged caller): the answers must not change.
"""

import numpy as np
import pytest

import dropin_trace as T
from conftest import clustered, scaled_clusters

pytestmark = pytest.mark.gpu

GENERATORS = {"clustered": clustered, "scaled_clusters": scaled_clusters}


def _inputs(name, n, d=None, seed=None):
    if d is None:
        from costal_gb300 import workloads

        return workloads.make(name, n)[0]
    return GENERATORS[name](n, d, seed)


@pytest.mark.parametrize("default", ["fp32", "bf16"])
def test_reference_package_calls_give_the_recorded_answers(ext, monkeypatch, default):
    monkeypatch.setattr(ext, "DEFAULT_MATMUL", default)
    doc, arrays = T.load()
    assert not doc["meta"]["reference_tests"]["failed"]
    produced, replayed, raised = {}, 0, 0
    for i, call in enumerate(doc["calls"]):
        if not call["replay"]:
            continue
        args = [T.make_input(a, arrays, produced, _inputs) for a in call["args"]]
        kwargs = {k: T.make_input(v, arrays, produced, _inputs) for k, v in call["kwargs"].items()}
        where = f"call {i} {call['fn']}"
        fn = getattr(ext, call["fn"])
        if "raises" in call:
            want = call["raises"]
            with pytest.raises(Exception) as info:
                fn(*args, **kwargs)
            assert type(info.value).__name__ == want["type"], f"{where}: {info.value!r}"
            for s in T.MATCHED:
                assert (s in want["msg"]) <= (s in str(info.value)), f"{where}: {info.value} lacks {s!r}"
            raised += 1
        else:
            got = fn(*args, **kwargs)
            if default == "bf16" and call["fn"] == "_knn_exact":
                # the tensor-core pass may re-run uncertified rows in FP32 before any regather, so
                # only the answer, not the fallback count, is the reference's
                got = (got[0], {**got[1], "fallback_rows": 0})
                want = call["result"]
                want = {"tuple": [want["tuple"][0], {"stats": {**want["tuple"][1]["stats"], "fallback": False}}]}
                T.compare_output(got, want, produced, where)
            else:
                T.compare_output(got, call["result"], produced, where)
        replayed += 1
    assert replayed > 100 and raised > 0
    print(f"replayed {replayed} calls of the reference package ({raised} expected errors), default {default}")
