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
took it, as the package would. Every answer must equal the oracle's on the same inputs (the same
calls replayed with the oracle answering the device entry points), and the recorded answer wherever
this machine rebuilt the recorded inputs bit for bit (the generators' arcsinh need not round alike on
every CPU).

The last pass repeats everything with the module's default backend switched to the certified
split-BF16 tensor-core path (DEFAULT_MATMUL = "bf16", what COSTAL_GB300_MATMUL=bf16 does for an
unchanged caller): the answers must not change.
"""

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


def _replay(ext, doc, arrays):
    rp = T.Replay(arrays, _inputs)
    return [rp.call(ext, c) if c["replay"] else None for c in doc["calls"]]


@pytest.fixture(scope="module")
def record_and_oracle(ext):
    from oracle import device_stub

    doc, arrays = T.load()
    remove = device_stub.install()
    try:
        oracle_pass = _replay(ext, doc, arrays)
    finally:
        remove()
    return doc, arrays, oracle_pass


def test_oracle_pass_reproduces_the_record(record_and_oracle):
    """Where the inputs were rebuilt bit for bit, the oracle's answers on this machine are the record's."""
    doc, _, oracle_pass = record_and_oracle
    assert not doc["meta"]["reference_tests"]["failed"]
    checked = 0
    for i, (call, got) in enumerate(zip(doc["calls"], oracle_pass)):
        if got is None or not got[1]:
            continue
        want = {"raises": call["raises"]} if "raises" in call else {"result": call["result"]}
        assert T.same_answer(got[0], want), f"call {i} {call['fn']}: {got[0]} instead of {want}"
        checked += 1
    print(f"{checked} of {sum(c['replay'] for c in doc['calls'])} replayed calls had their recorded inputs")


@pytest.mark.parametrize("default", ["fp32", "bf16"])
def test_reference_package_calls_give_the_oracle_answers_on_the_gpu(ext, monkeypatch, record_and_oracle, default):
    doc, arrays, oracle_pass = record_and_oracle
    monkeypatch.setattr(ext, "DEFAULT_MATMUL", default)
    gpu_pass = _replay(ext, doc, arrays)
    replayed = raised = 0
    for i, (call, g, o) in enumerate(zip(doc["calls"], gpu_pass, oracle_pass)):
        if g is None:
            continue
        # on the tensor-core pass, rows the certificate sends back are re-run in FP32 before any
        # regather, so only the answer, not whether a row fell back, is the oracle's
        assert T.same_answer(g[0], o[0], with_fallback=default == "fp32"), \
            f"call {i} {call['fn']}: GPU {g[0]} oracle {o[0]}"
        replayed += 1
        raised += "raises" in g[0]
    assert replayed > 100 and raised > 0
    print(f"replayed {replayed} calls of the reference package on the GPU ({raised} expected errors), "
          f"default backend {default}")
