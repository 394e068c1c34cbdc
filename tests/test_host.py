"""Host pieces of the drivers (sfwi_gb300/host): SU records written and read
back, shot indexing (index_shot, sfwi-stage1/main.cpp:76-165) and the
para_stage parameter file."""
import os

import numpy as np
import pytest

from sfwi_gb300 import su


@pytest.fixture(scope="module", autouse=True)
def _built():
    from sfwi_gb300 import build
    build.build_host()


def test_su_round_trip_and_index(tmp_path):
    path = str(tmp_path / "rec.su")
    rng = np.random.default_rng(0)
    shots = [(1000, np.arange(600, 1210, 10)), (1100, np.arange(900, 1500, 20)), (1500, np.arange(1200, 1800, 10))]
    data = []
    for k, (sx, gx) in enumerate(shots):
        d = rng.standard_normal((len(gx), 333)).astype(np.float32)
        su.write(path, sx, gx, d, 1e-3, append=k > 0)
        data.append(d)
    nt, dt, table = su.index(path)
    assert nt == 333 and dt == pytest.approx(1e-3)
    assert [t["no"] for t in table] == [1, 2, 3]
    pos = 0
    for t, (sx, gx), d in zip(table, shots, data):
        assert t["ntr"] == len(gx) and t["sx"] == sx and t["pos"] == pos
        assert t["cx_min"] == min(sx, gx.min()) and t["cx_max"] == max(sx, gx.max())
        r, gc = su.read(path, t["pos"], t["ntr"], nt)
        assert np.array_equal(r, d) and np.array_equal(gc, gx)
        pos += t["ntr"]
    assert os.path.getsize(path) == pos * (240 + 4 * nt)


def test_su_header_offsets(tmp_path):
    """sx at byte 72, gx at 80, ns at 114, dt (microseconds) at 116."""
    path = str(tmp_path / "one.su")
    su.write(path, 123456, np.array([7890]), np.zeros((1, 50), np.float32), 5e-4)
    h = open(path, "rb").read(240)
    assert int.from_bytes(h[72:76], "little", signed=True) == 123456
    assert int.from_bytes(h[80:84], "little", signed=True) == 7890
    assert int.from_bytes(h[114:116], "little") == 50
    assert int.from_bytes(h[116:118], "little") == 500


def test_para_file(tmp_path):
    path = tmp_path / "para_stage1"
    path.write_text("10 10 50 376 201 1 38\n/d/vp.bin\n/d/vs.bin\n/d/rho.bin\n/d/record-z.su\n/d/record-x.su\n"
                    "/d/out\n10 100 0\n0 0\n1 0 0 1000\n")
    p = su.read_para(str(path))
    assert (p["dx"], p["dz"], p["pml"], p["allnx"], p["allnz"], p["minshot"], p["maxshot"]) == (10, 10, 50, 376, 201,
                                                                                              1, 38)
    assert p["vp"] == "/d/vp.bin" and p["rec_x"] == "/d/record-x.su" and p["outdir"] == "/d/out"
    assert (p["f0"], p["maxiter"], p["iter_round1"], p["sy"], p["gy"]) == (10, 100, 0, 0, 0)
    assert (p["light"], p["rbc"], p["cpu_mem"], p["iointerval"]) == (1, 0, 0, 1000)
    bad = tmp_path / "bad"
    bad.write_text("10 10\n")
    with pytest.raises(OSError):
        su.read_para(str(bad))


def test_corrupt_record_files_are_refused(tmp_path):
    """A truncated file, a header without samples and a read past the end
    are reported (OSError from the host library's -1), never crashed on."""
    path = str(tmp_path / "rec.su")
    su.write(path, 1000, np.arange(0, 100, 10), np.ones((10, 64), np.float32), 1e-3)
    good = open(path, "rb").read()
    trunc = str(tmp_path / "trunc.su")
    open(trunc, "wb").write(good[:-17])
    with pytest.raises(OSError):
        su.index(trunc)
    with pytest.raises(OSError):
        su.read(trunc, 9, 1, 64)
    nosamples = bytearray(good)
    nosamples[114:116] = b"\x00\x00"
    bad = str(tmp_path / "ns0.su")
    open(bad, "wb").write(bytes(nosamples))
    with pytest.raises(OSError):
        su.index(bad)
    with pytest.raises(OSError):
        su.read(path, 5, 10, 64)  # traces 5..14 of a 10-trace file
    with pytest.raises(OSError):
        su.index(str(tmp_path / "missing.su"))
