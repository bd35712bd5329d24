"""GPU: the step kernel that stages tiles in shared memory with bulk copies.

For BF16 and FP16 storage the staged kernel (cp.async.bulk copies of
each tile's pulled runs into shared memory by a producer warp, completion on
mbarriers; consumer warps update two cells per thread with packed f32x2
arithmetic; the boundary groups in a second kernel) and the kernel that loads
every population into registers run the same node update with explicit
rounding, so after many iterations they hold the same bits: f, fb, p, u and
every Monitor value, in both boundary-copy modes, on the small D3Q27 parity
lattices and on the benchmark's sphere (the launch takes the staged kernel
for D3Q27 only).
"""
import numpy as np
import pytest

from parity_util import make_case

pytestmark = pytest.mark.gpu


def _run(im, cfg, st, init, precision, staged, mode, steps, interv):
    with im.Solver(cfg, precision=precision) as s:
        s.set_geometry(st)
        s.set_fill_mode(mode)
        assert im.lib().imexlb_testing_set_staged_kernel(s.h, 1 if staged else 0) == im.IMEXLB_OK
        s.upload(*init)
        mon = s.step(0, steps, interv)
        return mon, s.download()


def _same(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


@pytest.mark.parametrize("name", ["3d_32x16x16", "3d_24x12x14_rho"])
@pytest.mark.parametrize("prec", ["fp16", "bf16"])
def test_staged_kernel_matches_register_kernel(built, name, prec):
    import imexlb as im
    code = {"fp16": im.FP16, "bf16": im.BF16}[prec]
    cfg, st, o = make_case(name)
    init = [x.copy() for x in (o.f, o.fb, o.p, o.u)]
    for mode in (im.FILL_FUSED, im.FILL_KERNEL):
        a = _run(im, cfg, st, init, code, True, mode, 60, 7)
        b = _run(im, cfg, st, init, code, False, mode, 60, 7)
        assert _same(a[0], b[0]), (mode, "Monitor")
        for x, y, w in zip(a[1], b[1], ("f", "fb", "p", "u")):
            assert _same(x, y), (mode, w)


@pytest.mark.parametrize("workload", ["sphere_d3q27_128x64x64"])
@pytest.mark.parametrize("prec,interv", [("fp16", 13), ("bf16", 1)])
def test_staged_kernel_matches_register_kernel_benchmark_lattices(built, workload, prec, interv):
    """interv 1: a Monitor on every iteration (the kernels' Monitor forms)."""
    import bench
    import imexlb as im
    code = {"fp16": im.FP16, "bf16": im.BF16}[prec]
    cfg, st = bench._setup(workload)
    init = (st.f, st.fb, st.p, st.u)
    a = _run(im, cfg, st, init, code, True, im.FILL_FUSED, 40, interv)
    b = _run(im, cfg, st, init, code, False, im.FILL_FUSED, 40, interv)
    assert _same(a[0], b[0])
    for x, y in zip(a[1], b[1]):
        assert _same(x, y)


def test_staged_wait_gives_up_with_a_status(built):
    """Failure injection on the host side of the kernel: the first tile of
    every block starts no copies, so its bounded wait (50 ms here) runs out;
    the step call returns IMEXLB_ERR_TIMEOUT and the device keeps working."""
    import time
    import imexlb as im
    cfg, st, o = make_case("3d_32x16x16")
    init = [x.copy() for x in (o.f, o.fb, o.p, o.u)]
    ref = _run(im, cfg, st, init, im.FP16, True, im.FILL_FUSED, 20, 5)
    with im.Solver(cfg, precision=im.FP16) as s:
        s.set_geometry(st)
        s.upload(*init)
        assert im.lib().imexlb_testing_stage_stall(s.h, 0.05) == im.IMEXLB_OK
        t0 = time.time()
        with pytest.raises(im.ImexlbError) as ei:
            s.step(0, 3, 0)
        assert ei.value.code == im.ERR_TIMEOUT
        assert time.time() - t0 < 10.0
        assert im.lib().imexlb_testing_stage_stall(s.h, 0.0) == im.IMEXLB_OK
        s.upload(*init)
        mon = s.step(0, 20, 5)
        out = s.download()
    assert _same(mon, ref[0])
    for x, y in zip(out, ref[1]):
        assert _same(x, y)
