"""GPU: SetGeometry on the device (imexlb_device_set_geometry) against the
host set-up (imexlb_host_set_geometry), which the CPU tests pin to the
reference's rules (initialization.f90:167-255, initialization_3d.f90:
170-279): geo over every padded cell and every list, element for element,
on the benchmark lattices, the ensemble's cylinder cases (with the y offset
extension) and odd sizes; and the same IMEXLB_ERR_GEOMETRY where the
reference's obstacle probe leaves the geo array."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LISTS = ("fluid_id", "bl", "br", "bu", "bd", "bf", "bb", "b_user")


def _configs():
    import imexlb as im
    from imexlb import ensemble
    out = [
        im.make_config(2, 1024, 512, charlength=0.0390625, xpos=0.25, re=100.0,
                       ome=1.7857142857142856),
        im.make_config(2, 63, 31, charlength=0.21, xpos=0.37, re=30.0, ome=1.6),
        im.make_config(3, 256, 128, 128, charlength=0.09375, xpos=0.25, re=100.0,
                       ome=1.8910741301059),
        im.make_config(3, 45, 27, 31, charlength=0.3, xpos=0.3, re=20.0, ome=1.7),
    ]
    out += [ensemble.case_config(c) for c in ensemble.draw_cases(6, seed=3)]
    return out


def test_device_geometry_matches_host(built):
    import imexlb as im
    for cfg in _configs():
        t0 = time.perf_counter()
        h = im.Setup(cfg, state=False)
        t1 = time.perf_counter()
        d = im.Setup(cfg, device=0, state=False)
        t2 = time.perf_counter()
        what = "%dD %dx%dx%d" % (cfg.dim, cfg.nx, cfg.ny, cfg.nz)
        assert np.array_equal(h.geo, d.geo), what
        for name in LISTS:
            assert np.array_equal(getattr(h, name), getattr(d, name)), (what, name)
        assert d.fluid_id.size > 0 and d.b_user.size > 0
        print("%s: host %.1f ms, device %.1f ms" % (what, 1e3 * (t1 - t0), 1e3 * (t2 - t1)))


def test_device_geometry_probe_outside_the_array(built):
    """A small 3D lattice with a large sphere, where the reference's obstacle
    probe (offsets of up to 80 planes) leaves the geo array: both set-ups
    refuse it alike."""
    import imexlb as im
    cfg = im.make_config(3, 32, 10, 13, charlength=0.358, xpos=0.246, re=20.0, ome=1.7)
    errs = []
    for dev in (None, 0):
        with pytest.raises(im.ImexlbError) as ei:
            im.Setup(cfg, device=dev, state=False)
        errs.append(ei.value.code)
    assert errs == [im.ERR_GEOMETRY, im.ERR_GEOMETRY]
