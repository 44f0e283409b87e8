"""The solver's node update against a plain restatement of it, on the host.

stencil.cuh's fm_update shares each lateral pair's sort between the two
octants that differ in the radial direction, orders keys by min/max and masks
octants outside the grid with a select.  tests/stencil_network_check.cpp
restates the update the direct way (eight octants, each sorted by a full
three-comparator stable network, outside octants skipped) and compares the
two bit for bit on random inputs with ties, unset neighbours and +inf/NaN
outside the grid, in both precisions.  It also checks the main sweep's
upstream-only update (fm_update_upstream) against fm_update with the three
downstream neighbours unset, for every sweep direction.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_update_equals_plain_restatement(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = tmp_path / "stencil_network_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    os.path.join(HERE, "stencil_network_check.cpp"), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe), "200000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "float mismatches 0" in r.stdout and "double mismatches 0" in r.stdout
    assert "upstream float mismatches 0" in r.stdout and "upstream double mismatches 0" in r.stdout
