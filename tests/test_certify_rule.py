"""The certification rule of the rounds' first pass, checked on the host.

tests/certify_check.cpp restates one directional sweep with the solver's
node update (every node computed once, its upstream neighbours first, the
field above the bottom face unset), applies the rule certify_kernel uses,
and recomputes every node the rule clears from the final field: each must
give the same bits.  Random slowness models (3% and 15% perturbations),
plane-wave bottom faces, sweep directions with and against the wave, both
orders and both precisions; the rule must also clear a fair share of the
nodes.  Without its margin and its second-order conditions the same check
finds changed nodes, so it can tell.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_certified_nodes_do_not_change(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = tmp_path / "certify_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "certify_check.cpp"),
                    "-o", str(exe)], check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe), "400"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 changed; double" in r.stdout and r.stdout.strip().endswith("0 changed")
