"""The precision study (fm3dt.precision) on a small slab case: single-precision
offset times against double precision, per source-receiver pair -- receiver
time within 1e-5 relative and 1 ms, ray end point within one
propagation-grid cell; Frechet rows, which follow the slightly shifted ray
paths, within 1e-2 of the row's largest entry and in 2-norm (measured on this
case: 3.2e-3 and 3.7e-3; on the full 256^3 slab with 16 events 2.2e-2 and
9.8e-3 at worst, 2.6e-4 and 1.6e-4 on average)."""
import pytest

pytestmark = pytest.mark.gpu


def test_precision_study_small_slab(gpu_lib):
    from fm3dt import precision
    r = precision.study(cfg=2, scale=40, nev=4, batch64=2)
    assert r["pairs"] == 4 * r["receivers"]
    assert r["traveltime_rel"]["max"] <= 1e-5
    assert r["traveltime_abs_s"]["max"] <= 1e-3
    assert r["ray_endpoint_cells"]["max"] <= 1.0
    assert r["frechet_row_rel"]["max"] <= 1e-2
    assert r["frechet_row_rel_l2"]["max"] <= 1e-2
