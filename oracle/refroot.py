"""Where the reference's read-only source tree is found (test infrastructure).

Only the recipes that compile the reference into the oracle's pin
(`oracle/build_ref.sh`, `baseline/build_refgpu.sh`), the fixture generators
under `tests/golden/` and the tests that read the reference's own test data ask
for it. Order: the environment variable RFBA_REFERENCE_ROOT, then the caller's
argument, then the default mount point of the development container. None of
the library, the GPU tests or the bench reads the reference at run time.
"""
from __future__ import annotations

import os

ENV = "RFBA_REFERENCE_ROOT"
# default: the development container's mount point of the reference tree
DEFAULT = "/root/reference"


def reference_root(arg: str | None = None) -> str:
    return os.environ.get(ENV) or arg or DEFAULT


def present(arg: str | None = None) -> bool:
    return os.path.isdir(reference_root(arg))
