"""The C++ interface <genie/genie.h> (libgenie.so over the C ABI), driven by
the C++ program tests/cpp/shim_test.cc the way the reference's examples and
tests use the reference library."""
import os
import subprocess

import numpy as np
import pytest

from conftest import golden


def _built():
    from genie_gb300 import build
    build.build()
    build.build_cpp()
    return build.SHIM_TEST


def test_cpp_interface_host_side(tmp_path):
    """Configuration errors, CSV parsing and status-code -> exception mapping
    (no device work)."""
    exe = _built()
    r = subprocess.run([exe, "host", str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr


@pytest.mark.gpu
def test_cpp_interface_search_and_second_level(oracle, tmp_path):
    """genie::Search over sift_20 (test_csv_input_sift_data.cc:65-87), the
    second-level BuildTable/BuildQuery/Match, binary save/load, multi-table
    Match and a query range, against the oracle."""
    exe = _built()
    z = golden("sift20.npz")
    values = z["values"]
    p = tmp_path / "sift_20.csv"
    with open(p, "w") as f:
        for row in values:
            f.write(",".join(str(v) for v in row) + ",\n")
    r = subprocess.run([exe, "gpu", str(p), str(p), str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout[-2000:] + r.stderr
    rows = {}
    for line in r.stdout.splitlines():
        parts = line.split()
        if len(parts) == 5:
            rows.setdefault(parts[0], []).append([int(x) for x in parts[1:]])
    ox = oracle.Index(values)
    q = 5
    for tag, rad in (("search", 0), ("range1", 1)):
        got = np.array(rows[tag])
        qv = values[:q]
        dims = np.tile(np.arange(values.shape[1]), q)
        batch = dict(item_off=np.arange(q + 1) * values.shape[1], dim=dims.astype(np.int32),
                     low=(qv.ravel() - rad).astype(np.int32), up=(qv.ravel() + rad).astype(np.int32),
                     k=np.full(q, 5, np.uint32))
        oid, ocnt, _, _ = ox.search(batch)
        assert np.array_equal(got[:, 2], oid) and np.array_equal(got[:, 3], ocnt), tag
