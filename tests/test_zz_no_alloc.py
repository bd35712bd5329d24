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


def test_monitor_noalloc_allocates_nothing_large_list_user_stream(built):
    """A synthetic list of 600,000 fluid entries (293 partial blocks, so the
    final reduction loops over more than one block of partials), enqueued on
    a stream the caller created, with the largest |(ux, uy)| in the last
    block. Device free memory is read before and after two calls: a call that
    allocated would lower it (the caching allocator of the test holds its own
    buffers from before the first reading). One call runs before the first
    reading: the first use of the library's kernels on a device loads their
    module, which brings the static scratch array with it."""
    import torch
    import imexlb as im
    L = im.lib()
    rng = np.random.default_rng(7)
    n_cells, dim, n = 1_000_003, 3, 600_000
    u_host = rng.uniform(-0.05, 0.05, n_cells * dim)
    fid_host = rng.choice(n_cells, n, replace=False).astype(np.int32)
    last = fid_host[n - 3]                  # an entry of the last block
    u_host[last * dim] = 0.9
    u_host[last * dim + 1] = -0.4
    u_host[fid_host[0] * dim] = 5.0         # fluid_id(0) is not part of Monitor
    ux, uy = u_host[fid_host[1:] * dim], u_host[fid_host[1:] * dim + 1]
    want = float(np.max(np.sqrt(ux * ux + uy * uy)))
    u = torch.from_numpy(u_host).cuda()
    fid = torch.from_numpy(fid_host).cuda()
    outs = [torch.full((1,), -1.0, dtype=torch.float64, device="cuda") for _ in range(2)]
    stream = torch.cuda.Stream()
    warm = torch.empty(1, dtype=torch.float64, device="cuda")
    assert L.imexlb_monitor_noalloc(dim, C.c_void_p(u.data_ptr()), C.c_void_p(fid.data_ptr()), 2,
                                    C.c_void_p(warm.data_ptr()), None) == im.IMEXLB_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for out in outs:
        rc = L.imexlb_monitor_noalloc(dim, C.c_void_p(u.data_ptr()), C.c_void_p(fid.data_ptr()), n,
                                      C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert rc == im.IMEXLB_OK, L.imexlb_last_error(None).decode()
    stream.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert outs[0].item() == want and outs[1].item() == want
