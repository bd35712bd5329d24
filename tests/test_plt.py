"""WriteBinary (Tecplot #!TDV112) output against the record layout of
lbm.f90:231-413 / lbm_3d.f90:233-449, read back with an independent parser
on an oracle state."""
import struct

import numpy as np
import pytest

from oracle import orc


def _parse(buf, dim):
    o = 0

    def ints(n):
        nonlocal o
        v = struct.unpack_from("<%di" % n, buf, o)
        o += 4 * n
        return list(v)

    def f32(n):
        nonlocal o
        v = struct.unpack_from("<%df" % n, buf, o)
        o += 4 * n
        return list(v)

    def f64(n):
        nonlocal o
        v = np.frombuffer(buf, dtype="<f8", count=n, offset=o)
        o += 8 * n
        return v

    assert buf[:8] == b"#!TDV112"
    o = 8
    numvars = 5 if dim == 2 else 7
    title = "Cylinder" if dim == 2 else "Sphere"
    hdr = ints(4 + numvars + len(title) + sum(len(nm) for nm in
                                             (["x", "y", "p", "ux", "uy"] if dim == 2 else
                                              ["x", "y", "z", "p", "ux", "uy", "uz"])))
    out = {"hdr": hdr}
    out["fmt"] = f32(1)[0]
    out["zone"] = ints(11)
    out["time"] = f64(1)[0]
    out["sizes"] = ints(9)
    out["markers"] = f32(2)
    out["varfmt"] = ints(numvars + 3)
    out["limits"] = f64(2 * numvars)
    out["data_offset"] = o
    return out, numvars


@pytest.mark.parametrize("dim,n", [(2, (40, 20, 0)), (3, (20, 10, 12))])
def test_plt_records(built, tmp_path, dim, n):
    import imexlb as im
    kw = dict(charlength=0.3, xpos=0.3, re=20.0, ome=1.75, dt=1.0, rho0=1.0)
    o = orc.Oracle(orc.make_input(dim, *n, **kw))
    o.init_up(orc.r_vec(3))
    o.init_pdf()
    o.run(0, 7, 0)
    cfg = im.make_config(dim, *n, **kw)
    path = str(tmp_path / "output_003.plt")
    im.write_plt(cfg, path, 3, 7, o.p, o.u, o.lists["fluid_id"])
    buf = open(path, "rb").read()
    r, nv = _parse(buf, dim)
    title = "Cylinder" if dim == 2 else "Sphere"
    hdr = r["hdr"]
    assert hdr[:2] == [1, 0] and "".join(map(chr, hdr[2:2 + len(title)])) == title
    assert hdr[2 + len(title)] == 0 and hdr[3 + len(title)] == nv
    assert r["fmt"] == 299.0 and r["markers"] == [357.0, 299.0]
    assert "".join(map(chr, r["zone"][:8])) == "ZONE 003" and r["zone"][8:] == [0, -1, 0]
    s = o.s
    assert r["time"] == 7 / s.t_intv
    L = [s.nx + 1, s.ny + 1, (s.nz + 1) if dim == 3 else 1]
    assert r["sizes"] == [-1, 0, 0, 0, 0, L[0], L[1], L[2], 0]
    assert r["varfmt"] == [2] * nv + [0, 0, -1]
    # min/max over fluid_id(1:), starting from 0, in the reference's units
    ids = o.lists["fluid_id"][1:]
    u = o.u.reshape(-1, dim)
    cl, ti = s.charlength, s.t_intv
    exp = [0.0, s.nx / cl, 0.0, s.ny / cl] + ([0.0, s.nz / cl] if dim == 3 else [])
    exp += [min(0.0, o.p[ids].min()) * cl / ti ** 2, max(0.0, o.p[ids].max()) * cl / ti ** 2]
    for k in range(dim):
        exp += [min(0.0, u[ids, k].min()) / (cl * ti), max(0.0, u[ids, k].max()) / (cl * ti)]
    assert np.array_equal(r["limits"], np.array(exp))
    # data blocks
    npts = L[0] * L[1] * L[2]
    assert len(buf) == r["data_offset"] + nv * npts * 8
    data = np.frombuffer(buf, dtype="<f8", offset=r["data_offset"]).reshape(nv, L[2], L[1], L[0])
    zz, yy, xx = np.meshgrid(np.arange(L[2]), np.arange(L[1]), np.arange(L[0]), indexing="ij")
    ids3 = (xx + 3) + s.dy * (yy + 3) + (s.dz * (zz + 3) if dim == 3 else 0)
    assert np.array_equal(data[0], xx / cl) and np.array_equal(data[1], yy / cl)
    k0 = 2
    if dim == 3:
        assert np.array_equal(data[2], zz / cl)
        k0 = 3
    assert np.array_equal(data[k0], o.p[ids3] * cl / ti ** 2)
    for k in range(dim):
        assert np.array_equal(data[k0 + 1 + k], u[ids3, k] / (cl * ti))
