"""C-ABI surface of libimexlb, checked without a GPU: the library loads,
exports every function the public headers declare, and rejects bad
descriptors before touching the device."""
import ctypes as C
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(imexlb_\w+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_headers_declare_the_reference_entry_points():
    names = _declared()
    for n in ("imexlb_create", "imexlb_set_geometry", "imexlb_upload", "imexlb_init_pdf",
              "imexlb_step", "imexlb_download", "imexlb_destroy", "imexlb_last_error",
              "imexlb_host_read_input", "imexlb_host_set_geometry", "imexlb_host_init_up"):
        assert n in names


def test_library_exports_every_declared_symbol(built):
    import imexlb as im
    lib = im.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", im.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = _declared() - exported
    assert not missing, missing
    for n in _declared():
        getattr(lib, n)
    # the Python front end binds exactly the declared set
    assert set(im.symbols()) == _declared()


def test_version_string(built):
    import imexlb as im
    assert im.lib().imexlb_version().decode().startswith("1.0")


def test_create_rejects_bad_descriptors(built):
    import imexlb as im
    cfg = im.make_config(3, 16, 8, 8)
    rank_cfg = im.rank_config(cfg, (2, 1, 1), 1)
    L = im.lib()

    def create(d):
        h = C.c_void_p()
        rc = L.imexlb_create(C.byref(h), C.byref(d))
        msg = L.imexlb_last_error(None).decode()
        if rc == 0:
            L.imexlb_destroy(h)
        return rc, msg

    d = im.make_desc(cfg)
    d.ghost = 2
    assert create(d)[0] == im.ERR_ARG
    d = im.make_desc(cfg)
    d.nq = 19
    assert create(d)[0] == im.ERR_ARG
    d = im.make_desc(cfg)
    d.local_start[0] = 4  # box beyond the global lattice
    rc, msg = create(d)
    assert rc == im.ERR_ARG and "outside the global lattice" in msg
    d = im.make_desc(rank_cfg, precision=im.FP32)  # a rank of a multi-rank run
    rc, msg = create(d)
    assert rc == im.ERR_UNSUPPORTED and "IMEXLB_FP64" in msg
    d = im.make_desc(cfg)
    d.e[0] = 1  # direction 0 is (-1,-1,-1) in InitLattice order
    assert create(d)[0] == im.ERR_ARG
    d = im.make_desc(cfg)
    d.precision = 99
    assert create(d)[0] == im.ERR_UNSUPPORTED
    d = im.make_desc(cfg)
    d.dy += 1
    assert create(d)[0] == im.ERR_ARG


def test_null_handle_calls_fail_cleanly(built):
    import imexlb as im
    L = im.lib()
    assert L.imexlb_step(None, 0, 1, 0, None) == im.ERR_ARG
    assert L.imexlb_download(None, None, None, None, None) == im.ERR_ARG
    assert L.imexlb_upload(None, None, None, None, None) == im.ERR_ARG
    assert L.imexlb_set_fill_mode(None, im.FILL_FUSED) == im.ERR_ARG
    assert L.imexlb_get_fill_mode(None, None) == im.ERR_ARG
    L.imexlb_destroy(None)


def test_create_without_gpu_reports_cuda_error(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import imexlb as im
    with pytest.raises(im.ImexlbError) as ei:
        im.Solver(im.make_config(2, 16, 8))
    assert ei.value.code == im.ERR_CUDA
