"""Shared fixtures: the GB300 library, the CPU oracle and (where they were
built from the reference sources) the reference builds."""

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from sunlightlb_gb300 import build as _build  # noqa: E402
from sunlightlb_gb300.binding import Library  # noqa: E402

ORACLE = os.path.join(ROOT, "oracle", "liboracle.so")
REF_STRICT = os.path.join(ROOT, "oracle", "_ref", "libref_strict.so")
REF_SHIPPED = os.path.join(ROOT, "oracle", "_ref", "libref_shipped.so")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the GB300 kernels)")


@pytest.fixture(scope="session")
def orc():
    if not os.path.exists(ORACLE):
        _build.build_oracle(with_reference=False)
    return Library(ORACLE, extended=True)


@pytest.fixture(scope="session")
def gpu():
    import sunlightlb_gb300
    return sunlightlb_gb300.library()


@pytest.fixture(scope="session")
def ref_strict():
    if not os.path.exists(REF_STRICT):
        pytest.skip("reference build not available (built only where the reference sources are)")
    return Library(REF_STRICT, extended=False)


@pytest.fixture(scope="session")
def ref_shipped():
    if not os.path.exists(REF_SHIPPED):
        pytest.skip("reference build not available (built only where the reference sources are)")
    return Library(REF_SHIPPED, extended=False)
