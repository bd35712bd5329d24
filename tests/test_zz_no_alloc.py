"""imexlb_monitor_noalloc: the Monitor value without any allocation.

This entry point exists for hosts that cannot let a library call cudaMalloc,
for example a Fortran host whose u and fluid_id live in device memory mapped
by its OpenMP offload runtime, or an application that keeps the device
memory for its own pool. Given those device arrays it computes what the
reference's Monitor reduces (lbm.f90:211-217), using only a fixed scratch
array compiled into the library.

The test calls it through the C ABI on device copies of the state that
imexlb_step holds, twice in a row on two different states, and requires the
same value imexlb_step's own Monitor reports (IEEE equality, as all parity
tests here). The device arrays are created by the test, not by the entry
point.
"""
import ctypes as C

import numpy as np
import pytest

from parity_util import make_case

pytestmark = pytest.mark.gpu


def _monitor_noalloc(im, torch, dim, u_host, fluid_id):
    u = torch.from_numpy(np.ascontiguousarray(u_host)).cuda()
    fid = torch.from_numpy(np.ascontiguousarray(fluid_id, dtype=np.int32)).cuda()
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = im.lib().imexlb_monitor_noalloc(dim, C.c_void_p(u.data_ptr()), C.c_void_p(fid.data_ptr()),
                                         int(fid.numel()), C.c_void_p(out.data_ptr()), None)
    assert rc == im.IMEXLB_OK, im.lib().imexlb_last_error(None).decode()
    torch.cuda.synchronize()
    return float(out.item())


@pytest.mark.parametrize("name", ["3d_32x16x16", "2d_64x32"])
def test_monitor_noalloc_matches_step_monitor(built, name):
    import torch
    import imexlb as im
    cfg, st, o = make_case(name)
    with im.Solver(cfg) as s:
        s.set_geometry(st)
        s.upload(o.f, o.fb, o.p, o.u)
        s.step(0, 6, 0)
        _, _, _, u1 = s.download()
        ref1 = s.step(6, 1, 1)[0]      # Monitor of iteration 6 sees u1
        s.step(7, 4, 0)
        _, _, _, u2 = s.download()
        ref2 = s.step(11, 1, 1)[0]     # Monitor of iteration 11 sees u2
    got1 = _monitor_noalloc(im, torch, cfg.dim, u1, st.fluid_id)
    got2 = _monitor_noalloc(im, torch, cfg.dim, u2, st.fluid_id)
    assert ref1 > 0 and ref2 > 0 and ref1 != ref2
    assert got1 == ref1
    assert got2 == ref2


def test_monitor_noalloc_rejects_lists_beyond_its_scratch(built):
    import imexlb as im
    L = im.lib()
    big = 16777216 + 1
    rc = L.imexlb_monitor_noalloc(3, C.c_void_p(8), C.c_void_p(8), big, C.c_void_p(8), None)
    assert rc == im.ERR_ARG
    assert "IMEXLB_NOALLOC_MAX_FLUID" in L.imexlb_last_error(None).decode()
