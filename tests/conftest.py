import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "erdos-strauss_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); run with -m gpu")


def golden(*parts):
    return os.path.join(GOLDEN, *parts)


def read(*parts):
    with open(golden(*parts)) as f:
        return f.read()


def split_stream(text):
    """(certificate lines, SUMMARY lines) of a scanner's stdout."""
    lines = text.splitlines(keepends=True)
    return [ln for ln in lines if not ln.startswith("SUMMARY ")], [ln for ln in lines if ln.startswith("SUMMARY ")]


def strip_for_cover_scan(summary):
    """The fields tests/diff3.sh:31 removes before comparing against cover_scan."""
    import re
    return re.sub(r" classes_sha256=[0-9a-f]+", "", re.sub(r" sieved=[0-9]+", "", summary))


@pytest.fixture(scope="session")
def filters():
    import es_sieve
    return {f: es_sieve.load_filters(golden("filters", f)) for f in os.listdir(golden("filters"))}
