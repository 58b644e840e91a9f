"""Restart files on the host (no GPU): the library's netCDF classic parser against files written by scipy's
independent writer, the checksum restatement's known answers, and the refusals."""
import numpy as np
import pytest

from fv3atm_gb300 import restart as R
from fv3atm_gb300._lib import Fv3gError
from oracle.restart_oracle import mpp_chksum, z16

from ._restart_files import write_fields


def test_mpp_chksum_known_answers():
    assert mpp_chksum(np.array([1.0, 2.0])) == 0x3FF0000000000000 + 0x4000000000000000
    # the 64-bit sum wraps: two patterns with the top bit set
    assert mpp_chksum(np.array([-1.0, -2.0])) == (0xBFF0000000000000 + 0xC000000000000000) % 2 ** 64
    # FP32 patterns are widened with their sign: -1.0f is 0xBF800000, a negative int32
    assert mpp_chksum(np.array([-1.0], dtype=np.float32)) == 0xFFFFFFFFBF800000
    assert mpp_chksum(np.array([1.0, -1.0], dtype=np.float32)) == (0x3F800000 + 0xFFFFFFFFBF800000) % 2 ** 64
    assert mpp_chksum(np.zeros(0)) == 0


def test_z16_is_right_justified_upper_case_hex_in_32_columns():
    assert z16(0x7FF0000000000000) == "7FF0000000000000" + " " * 16
    assert z16(0xFF) == " " * 14 + "FF" + " " * 16
    assert len(z16(0)) == 32


@pytest.mark.parametrize("version", [1, 2])
def test_reader_matches_scipy_written_tracer_file(tmp_path, version):
    rng = np.random.default_rng(7)
    fields = {"sphum": rng.random((5, 6, 6)) * 1e-2, "liq_wat": rng.random((5, 6, 6)).astype(np.float32),
              "o3mr": rng.standard_normal((5, 6, 6))}
    path = str(tmp_path / "fv_tracer.res.tile1.nc")
    write_fields(path, fields, version=version)
    with R.NcFile(path) as f:
        v = f.variables()
        assert list(v) == ["xaxis_1", "yaxis_1", "zaxis_1", "Time", "sphum", "liq_wat", "o3mr"]
        assert v["liq_wat"] == (np.dtype(np.float32), (1, 5, 6, 6), True)
        assert v["zaxis_1"] == (np.dtype(np.float64), (5,), False)
        assert f.field_names() == ["sphum", "liq_wat", "o3mr"]
        for name, a in fields.items():
            assert np.array_equal(f.read(name), a.astype(np.float64))
            assert f.checksum(name) == mpp_chksum(a)
        assert np.array_equal(f.read("yaxis_1"), np.arange(1.0, 7.0))
        assert f.read("Time") == 1.0  # one record of a 1-D record variable


def test_reader_finds_delp_in_a_core_file(tmp_path):
    """fv_core.res: staggered u on (yaxis_1 = n+1, xaxis_1), the cell fields on (yaxis_2, xaxis_1)."""
    rng = np.random.default_rng(8)
    n, npz = 6, 4
    delp = rng.random((npz, n, n)) * 100 + 500
    u = rng.standard_normal((1, npz, n + 1, n))
    path = str(tmp_path / "fv_core.res.tile1.nc")
    write_fields(path, {"delp": delp}, core=True, extra={"u": (u, ("Time", "zaxis_1", "yaxis_1", "xaxis_1"))})
    with R.NcFile(path) as f:
        assert f.variables()["u"][1] == (1, npz, n + 1, n)
        assert np.array_equal(f.read("delp"), delp)
        assert np.array_equal(f.read("u"), u[0])
        assert f.checksum("u") is None


def test_refusals_are_errors_not_crashes(tmp_path):
    hdf5 = tmp_path / "netcdf4.nc"
    hdf5.write_bytes(b"\x89HDF\r\n\x1a\n" + bytes(64))
    with pytest.raises(Fv3gError, match="HDF5"):
        R.NcFile(str(hdf5))
    junk = tmp_path / "junk.nc"
    junk.write_bytes(b"not a netcdf file at all")
    with pytest.raises(Fv3gError, match="not a netCDF"):
        R.NcFile(str(junk))
    with pytest.raises(Fv3gError, match="cannot open"):
        R.NcFile(str(tmp_path / "missing.nc"))
    good = str(tmp_path / "good.nc")
    write_fields(good, {"sphum": np.ones((2, 3, 3))})
    data = open(good, "rb").read()
    cut = tmp_path / "cut.nc"
    cut.write_bytes(data[:40])  # header cut short
    with pytest.raises(Fv3gError):
        R.NcFile(str(cut))
    with R.NcFile(good) as f:
        with pytest.raises(Fv3gError, match="no variable"):
            f.read("rainwat")


def test_reader_parses_a_cdf5_file(tmp_path):
    """64-bit counts, sizes, dimension ids and offsets (CDF-5), FP64 and FP32 fields."""
    from ._restart_files import write_cdf5
    rng = np.random.default_rng(9)
    fields = {"sphum": rng.random((3, 5, 5)), "o3mr": rng.random((3, 5, 5)).astype(np.float32)}
    path = str(tmp_path / "cdf5.nc")
    write_cdf5(path, fields)
    with R.NcFile(path) as f:
        v = f.variables()
        assert list(v) == ["xaxis_1", "yaxis_1", "zaxis_1", "Time", "sphum", "o3mr"]
        assert v["o3mr"] == (np.dtype(np.float32), (1, 3, 5, 5), True)
        for k, a in fields.items():
            assert np.array_equal(f.read(k), a.astype(np.float64))
            assert f.checksum(k) == mpp_chksum(a)
        assert np.array_equal(f.read("zaxis_1"), np.arange(1.0, 4.0))


def test_truncated_data_is_an_error(tmp_path):
    """A file whose header is whole but whose values stop early: the host read reports a short read."""
    good = str(tmp_path / "good.nc")
    write_fields(good, {"sphum": np.ones((4, 6, 6))})
    data = open(good, "rb").read()
    cut = tmp_path / "cut.nc"
    cut.write_bytes(data[:-100])
    with R.NcFile(str(cut)) as f:
        with pytest.raises(Fv3gError, match="short read"):
            f.read("sphum")
