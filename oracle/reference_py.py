"""TEST INFRASTRUCTURE ONLY — where the reference's own Python package and tests are, when present.

The reference (ike12th/CosTaL 2.1.0) keeps its pure-Python package in `python/costal/` and its Python
tests in `tests/`. This recipe finds that checkout: `$COSTAL_REFERENCE` if set, else a read-only
copy at /root/reference where the fixtures are recorded. Nothing is copied out of it: the
reference package is imported from where it lies, only by tests/golden/make_dropin.py (which records
what that package asks of `costal._costal`) and the CPU test that re-runs it. On a machine without
the reference, `locate()` returns None and those skip.
"""

from __future__ import annotations

import os
from pathlib import Path

DEFAULT = Path("/root/reference")

# The reference's Python test files run through the drop-in (tests/ of the reference checkout). The
# others test the CLI, FCS reading, preprocessing, 1.0 compatibility and the examples, which are not
# on the kNN-graph path and call nothing of `costal._costal` that these do not.
TEST_FILES = ("test_smoke.py", "test_knn.py", "test_leiden_native.py", "test_leiden_api.py", "test_multiscale.py")


def locate() -> Path | None:
    """The reference checkout's root, or None when it is not on this machine."""
    root = Path(os.environ.get("COSTAL_REFERENCE", DEFAULT))
    if (root / "python" / "costal" / "__init__.py").is_file() and (root / "tests").is_dir():
        return root
    return None
