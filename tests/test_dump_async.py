"""Asynchronous dump: the file written by dump_begin/dump_finish is the
synchronous dump of the state at dump_begin, although steps run between
the two calls; the column diagnostics match asph_column_diag."""
import os

import numpy as np
import pytest

from sph_cuda_gb300 import Asph, dumpfmt, preset


@pytest.mark.gpu
def test_async_dump_equals_sync_dump(tmp_path):
    p = preset("reference", 24, 24, 16)
    a, b = Asph(p), Asph(p)
    a.init()
    b.init()
    a.step(7)
    b.step(7)
    sync = a.dump(str(tmp_path / "sync"))
    diag_sync = a.column_diag()
    b.dump_begin()
    b.step(5)                      # runs while the copy completes
    path, diag = b.dump_finish(str(tmp_path / "async"))
    assert os.path.basename(path) == os.path.basename(sync)
    assert open(path, "rb").read() == open(sync, "rb").read()
    for k in ("cloud_pct", "ql_max", "w_max", "precip_mm"):
        assert diag[k] == pytest.approx(diag_sync[k], rel=1e-6, abs=1e-12), k
    # the later steps did run
    assert b.control()["step"] == 12
    d = dumpfmt.read(path)
    assert d["nx"] == 24 and np.all(np.isfinite(d["data"]))
    a.close()
    b.close()


@pytest.mark.gpu
def test_one_dump_in_flight():
    from sph_cuda_gb300 import AsphError
    p = preset("reference", 16, 16, 8)
    a = Asph(p)
    a.init()
    with pytest.raises(AsphError):
        a.dump_finish("/tmp")
    a.dump_begin()
    with pytest.raises(AsphError):
        a.dump_begin()
    a.close()
