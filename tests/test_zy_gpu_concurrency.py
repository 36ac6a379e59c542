"""Concurrent use of one index handle, as the reference tests it
(pqivf/concurrency_test.go, internal/testutil/concurrent.go:19-118), plus
failed updates that keep their entries (pqivf/index_test.go:455-500).

The scenarios (tests/concurrency_scenarios.py) run in one child process: a
crash or a deadlock there fails these tests and leaves the rest of the
session running. The file sorts after the other GPU tests, so they run
first, and before the allocation-free entry point's tests, which run last."""
import json
import os
import subprocess
import sys

import pytest

from tests import concurrency_scenarios as cs

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CHILD_TIMEOUT_S = 300


@pytest.fixture(scope="module")
def results(gpu):
    try:
        p = subprocess.run([sys.executable, "-m", "tests.concurrency_scenarios"], cwd=ROOT, capture_output=True,
                           text=True, timeout=CHILD_TIMEOUT_S)
        out, rc, tail = p.stdout, p.returncode, p.stderr[-2000:]
    except subprocess.TimeoutExpired as e:
        out = e.stdout.decode() if isinstance(e.stdout, bytes) else (e.stdout or "")
        rc, tail = "timeout", ""
    got = {}
    for line in out.splitlines():
        if line.startswith("{"):
            r = json.loads(line)
            got[r["name"]] = r
    return got, rc, tail


@pytest.mark.parametrize("name", sorted(cs.SCENARIOS))
def test_scenario(results, name):
    got, rc, tail = results
    assert name in got, f"the scenario process ended before {name} (exit {rc}): {tail}"
    assert got[name]["ok"], got[name].get("error")
