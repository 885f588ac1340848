"""The record of what the reference's own Python package asks of `costal._costal`, and its replay.

tests/golden/make_dropin.py imports the reference's unchanged `costal` package with `costal._costal`
bound to a recording wrapper of costal_gb300._costal, runs the reference's Python tests and the
end-to-end calls of the benchmark configurations through it, and writes every call the package made:
the function, its arguments and keywords as the package passed them, and what came back.
tests/test_dropin_replay.py makes the same calls, in order, on a GB300 and asserts the same answers.

Arrays are stored by content: an argument that an earlier call returned is named by that return's
digest (so the replay feeds the GPU's own outputs forward, as the package would); a benchmark input
by its workload generator; anything else is saved in an .npz beside the record. Returned arrays are
kept as digests (dtype, shape and bytes); exceptions as their type and message.
"""

from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
TRACE_JSON = GOLDEN / "dropin_trace.json"
TRACE_NPZ = GOLDEN / "dropin_arrays.npz"

# The functions of the reference module (crates/costal-py/src/lib.rs:448-465) that the package calls.
FUNCTIONS = ("hello", "core_version", "row_l2_norms", "_knn_exact", "_knn_bruteforce", "_reweight", "_fuzzy_union",
             "_leiden", "_leiden_many", "_leiden_coo", "_modularity", "l2_bytes_per_thread", "tile_budget_bytes",
             "default_matmul")

# Functions that run on the host in the library too (the Leiden consumer and module constants). A call
# of one whose array arguments all come from the reference's test data, not from an earlier call, is
# fully exercised where it is recorded; the replay only repeats those fed by device results.
HOST_FUNCTIONS = ("hello", "core_version", "_leiden", "_leiden_many", "_leiden_coo", "_modularity",
                  "l2_bytes_per_thread", "tile_budget_bytes", "default_matmul")

# Substrings that the reference's tests match in error messages (tests/test_knn.py:159,
# tests/test_leiden_native.py:96-101, tests/test_leiden_api.py): a replayed error must carry the same.
MATCHED = ("NaN", "out of range", "n_iterations", "resolution", "objective", "unknown", "contiguous")


def digest(a) -> str:
    a = np.asarray(a)
    h = hashlib.sha256(f"{a.dtype.str}|{a.shape}|".encode())
    h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:24]


def _layout(a):
    if a.flags.c_contiguous:
        return "C"
    if a.flags.f_contiguous:
        return "F"
    return "strided"


class Recorder:
    """Wraps the module's functions; collects calls (JSON-ready) and the input arrays to store."""

    def __init__(self, known_inputs=None, generators=None):
        self.calls = []
        self.arrays = {}
        self.produced = set()
        self.known = dict(known_inputs or {})  # digest -> {"workload": name, "n": n}
        self.generators = generators or {}  # name -> f(n, d, seed): test-data generators to recognise
        self._pending = {}
        self._fed = False

    # --- encoding -------------------------------------------------------------------------------
    def enc_in(self, v):
        if isinstance(v, np.ndarray):
            dg = digest(v)
            lay = _layout(v)
            if lay == "C" and dg in self.produced:
                self._fed = True
                return {"out": dg}
            if lay == "C" and dg in self.known:
                return {**self.known[dg], "digest": dg}
            gen = self._generated(v, dg) if lay == "C" else None
            if gen is not None:
                return gen
            key = f"d{dg}"
            self._pending[key] = np.ascontiguousarray(v)
            return {"npz": key, "digest": dg, "layout": lay}
        if isinstance(v, (list, tuple)):
            return {"tuple" if isinstance(v, tuple) else "list": [self.enc_in(u) for u in v]}
        if isinstance(v, np.generic):
            return v.item()
        if v is None or isinstance(v, (bool, int, float, str)):
            return v
        raise TypeError(f"cannot record an argument of type {type(v).__name__}")

    def _generated(self, v, dg):
        """A 2-D float32 argument that one of the test-data generators makes (seeds 0-39)."""
        if v.dtype != np.float32 or v.ndim != 2:
            return None
        for name, gen in self.generators.items():
            for seed in range(40):
                if digest(gen(v.shape[0], v.shape[1], seed)) == dg:
                    spec = {"gen": name, "n": v.shape[0], "d": v.shape[1], "seed": seed, "digest": dg}
                    self.known[dg] = spec
                    return spec
        return None

    def enc_out(self, v, fn):
        if isinstance(v, np.ndarray):
            dg = digest(v)
            self.produced.add(dg)
            return {"arr": dg, "dtype": v.dtype.str, "shape": list(v.shape)}
        if isinstance(v, dict):
            # _knn_exact's stats: the reference's keys that do not depend on the machine
            # (lib.rs:152-166); fallback_rows as "any row fell back" (tests/test_knn.py:43,92)
            return {"stats": {"select": v.get("select"), "margin": v.get("margin"),
                              "fallback": bool(v.get("fallback_rows", 0) > 0)}}
        if isinstance(v, (list, tuple)):
            return {"tuple" if isinstance(v, tuple) else "list": [self.enc_out(u, fn) for u in v]}
        if isinstance(v, np.generic):
            return v.item()
        return v

    def wrap(self, name, fn):
        def recorded(*args, **kwargs):
            self._pending, self._fed = {}, False
            entry = {"fn": name, "args": [self.enc_in(a) for a in args],
                     "kwargs": {k: self.enc_in(v) for k, v in kwargs.items()}}
            entry["replay"] = name not in HOST_FUNCTIONS or self._fed
            if entry["replay"]:
                self.arrays.update(self._pending)
            try:
                out = fn(*args, **kwargs)
            except Exception as e:  # recorded, then re-raised to the package as it was
                entry["raises"] = {"type": type(e).__name__, "msg": str(e)}
                self.calls.append(entry)
                raise
            entry["result"] = self.enc_out(out, name)
            self.calls.append(entry)
            return out

        recorded.__name__ = name
        recorded.__doc__ = fn.__doc__
        return recorded

    def save(self, meta):
        TRACE_JSON.write_text(json.dumps({"meta": meta, "calls": self.calls}, indent=1) + "\n")
        np.savez_compressed(TRACE_NPZ, **self.arrays)


# --- replay ------------------------------------------------------------------------------------
#
# The inputs are rebuilt on the machine that replays: the test-data generators' transcendental
# functions (arcsinh) need not round alike on every CPU, so a rebuilt input can differ in a last bit
# from the recorded one. The replay therefore makes every call twice on the same rebuilt inputs —
# once through the library, once with its device entry points answered by the oracle — and requires
# the two answers to be identical; and wherever the rebuilt inputs equal the recorded ones, also equal
# to the recorded answer.

def load():
    doc = json.loads(TRACE_JSON.read_text())
    arrays = dict(np.load(TRACE_NPZ))
    return doc, arrays


class Replay:
    """One pass over the record. `bound` maps a recorded array digest to this pass's array."""

    def __init__(self, arrays, workloads):
        self.arrays = arrays
        self.workloads = workloads
        self.bound = {}
        self.rebuilt_differs = False  # some input of the current call was rebuilt with other bits

    def make_input(self, spec):
        if isinstance(spec, dict):
            if "out" in spec:
                if spec["out"] not in self.bound:
                    raise AssertionError(f"the replay never produced the array {spec['out']} the package passed on")
                a, same = self.bound[spec["out"]]
                self.rebuilt_differs |= not same
                return a
            if "gen" in spec or "workload" in spec:
                if "gen" in spec:
                    x = self.workloads(spec["gen"], spec["n"], spec["d"], spec["seed"])
                else:
                    x = self.workloads(spec["workload"], spec["n"])
                self.rebuilt_differs |= digest(x) != spec["digest"]
                return x
            if "npz" in spec:
                a = self.arrays[spec["npz"]]
                if spec["layout"] == "F":
                    a = np.asfortranarray(a)
                elif spec["layout"] == "strided":
                    a = np.repeat(a, 2, axis=-1)[..., ::2]
                return a
            if "tuple" in spec:
                return tuple(self.make_input(u) for u in spec["tuple"])
            if "list" in spec:
                return [self.make_input(u) for u in spec["list"]]
        return spec

    def bind(self, want, got, same):
        """Name this pass's returned arrays by the recorded digests they stand for."""
        if isinstance(want, dict) and "arr" in want and isinstance(got, np.ndarray):
            self.bound[want["arr"]] = (got, same and digest(got) == want["arr"])
        elif isinstance(want, dict) and ("tuple" in want or "list" in want) and isinstance(got, (tuple, list)):
            for w, g in zip(want.get("tuple", want.get("list")), got):
                self.bind(w, g, same)

    def call(self, ext, call):
        """Make one recorded call; returns (answer encoded like the record, inputs equal the recorded)."""
        self.rebuilt_differs = False
        args = [self.make_input(a) for a in call["args"]]
        kwargs = {k: self.make_input(v) for k, v in call["kwargs"].items()}
        same = not self.rebuilt_differs
        try:
            out = getattr(ext, call["fn"])(*args, **kwargs)
        except Exception as e:  # noqa: BLE001 (compared with the recorded exception)
            return {"raises": {"type": type(e).__name__, "msg": str(e)}}, same
        enc = encode_answer(out)
        if "result" in call:
            self.bind(call["result"], out, same)
        return {"result": enc}, same


def encode_answer(v):
    """An answer as the record encodes it (arrays by digest, stats by their machine-independent keys)."""
    if isinstance(v, np.ndarray):
        return {"arr": digest(v), "dtype": v.dtype.str, "shape": list(v.shape)}
    if isinstance(v, dict):
        return {"stats": {"select": v.get("select"), "margin": v.get("margin"),
                          "fallback": bool(v.get("fallback_rows", 0) > 0)}}
    if isinstance(v, (list, tuple)):
        return {"tuple" if isinstance(v, tuple) else "list": [encode_answer(u) for u in v]}
    if isinstance(v, np.generic):
        return v.item()
    return v


def same_answer(a, b, with_fallback=True):
    """Two encoded answers are the same (exceptions: same type and the message text the reference's
    tests match; stats: select and margin, and whether any row fell back when `with_fallback`)."""
    if "raises" in a or "raises" in b:
        if not ("raises" in a and "raises" in b) or a["raises"]["type"] != b["raises"]["type"]:
            return False
        return all((m in a["raises"]["msg"]) == (m in b["raises"]["msg"]) for m in MATCHED)

    def eq(x, y):
        if isinstance(x, dict) and isinstance(y, dict):
            if "stats" in x and "stats" in y:
                keys = ("select", "margin", "fallback") if with_fallback else ("select", "margin")
                return all(x["stats"].get(k) == y["stats"].get(k) for k in keys)
            return x.keys() == y.keys() and all(eq(x[k], y[k]) for k in x)
        if isinstance(x, list) and isinstance(y, list):
            return len(x) == len(y) and all(eq(u, v) for u, v in zip(x, y))
        if isinstance(x, (int, float)) and isinstance(y, (int, float)) and not isinstance(x, bool):
            return x == y
        return type(x) is type(y) and x == y

    return eq(a["result"], b["result"])
