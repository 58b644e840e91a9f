"""Restart files through the GPU: fv_tracer.res / fv_core.res read into and written from a batched state, in
the write component's layout, against scipy's independent netCDF reader and writer and the numpy restatement of
FMS mpp_chksum.  Integer and byte work: everything is compared bit for bit."""
import os

import numpy as np
import pytest

from fv3atm_gb300 import api
from fv3atm_gb300 import restart as R
from fv3atm_gb300 import synth as S
from fv3atm_gb300._lib import Fv3gError
from oracle.restart_oracle import mpp_chksum, z16

from ._helpers import interior
from ._restart_files import read_fields, write_fields

pytestmark = pytest.mark.gpu

NAMES = ["sphum", "liq_wat", "o3mr"]


@pytest.fixture(scope="module")
def prob():
    return S.make_problem(24, 5, 3, seed=31, cmax=0.7)


def _state(P, precision="fp64", upload=True):
    st = api.CubeState(P.n, P.npz, P.nq, precision=precision)
    if upload:
        st.load_problem(P)
    else:
        st.set_grid(P.geoms)
        st.set_levels(P.ak, P.bk)
    return st


@pytest.mark.parametrize("precision,dtype,version", [("fp64", "double", 2), ("fp64", "float", 1),
                                                     ("mixed", "double", 5), ("mixed", "float", 2)])
def test_written_files_read_by_scipy(cuda, prob, tmp_path, precision, dtype, version):
    """Each tile's tracers as the state holds them, converted to the file type, with mpp_chksum in '(Z16)'."""
    P = prob
    st = _state(P, precision)
    q = st.download("Q")
    npdt = np.float64 if dtype == "double" else np.float32
    for t in range(6):
        path = str(tmp_path / f"fv_tracer.res.tile{t + 1}.nc")
        sums = R.write_state(st, "Q", t, path, NAMES, dtype=dtype, version=version)
        if version == 5:  # scipy reads CDF-1/2 only: read CDF-5 back through the library
            with R.NcFile(path) as f:
                got = {k: (f.read(k).astype(npdt), z16(f.checksum(k))) for k in NAMES}
        else:
            got = read_fields(path)
        assert list(got) == NAMES
        for iq, name in enumerate(NAMES):
            data, ck = got[name]
            want = interior(q[t, iq], P.n).astype(npdt)
            assert data.dtype.kind == "f" and data.dtype.itemsize == np.dtype(npdt).itemsize
            assert np.array_equal(data, want)
            assert sums[iq] == mpp_chksum(want)
            assert ck == z16(sums[iq])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_restart_files_load_into_the_state(cuda, prob, tmp_path, precision):
    """scipy-written CDF-2 files (FP64 tracers, FP32 delp) into a fresh state: interiors exact (rounded to FP32
    in a mixed state), halos untouched, checksums verified and returned."""
    P = prob
    q = P.q.numpy()
    dp = P.dp.numpy()
    for t in range(6):
        write_fields(str(tmp_path / f"fv_tracer.res.tile{t + 1}.nc"),
                     {nm: interior(q[t, iq], P.n).copy() for iq, nm in enumerate(NAMES)})
        write_fields(str(tmp_path / f"fv_core.res.tile{t + 1}.nc"),
                     {"delp": interior(dp[t], P.n).astype(np.float32)}, core=True)
    st = _state(P, precision, upload=False)
    names = R.load_restart(st, str(tmp_path))
    assert names == NAMES
    gq, gdp = st.download("Q"), st.download("DELP")
    cast = (lambda a: a) if precision == "fp64" else (lambda a: a.astype(np.float32).astype(np.float64))
    assert np.array_equal(interior(gq, P.n), cast(interior(q, P.n)))
    assert np.array_equal(interior(gdp, P.n), interior(dp, P.n).astype(np.float32).astype(np.float64))
    ring = np.ones(gq.shape[-2:], bool)
    ring[3:3 + P.n, 3:3 + P.n] = False
    assert not gq[..., ring].any() and not gdp[..., ring].any()
    sums = R.read_state(st, "Q", 2, str(tmp_path / "fv_tracer.res.tile3.nc"), NAMES)
    assert sums == [mpp_chksum(interior(q[2, iq], P.n).copy()) for iq in range(3)]


def test_checksum_mismatch_is_an_error_unless_ignored(cuda, prob, tmp_path):
    P = prob
    a = interior(P.q.numpy()[0, 0], P.n).copy()
    path = str(tmp_path / "bad.nc")
    write_fields(path, {"sphum": a}, checksum={"sphum": z16(mpp_chksum(a) ^ 1)})
    st = _state(P, upload=False)
    with pytest.raises(Fv3gError, match="FV3G_E_CHECKSUM"):
        R.read_state(st, "Q", 0, path, ["sphum"])
    assert R.read_state(st, "Q", 0, path, ["sphum"], verify=False) == [mpp_chksum(a)]
    assert np.array_equal(interior(st.download("Q")[0, 0], P.n), a)


def test_slots_pick_tracers_and_others_keep_their_values(cuda, prob, tmp_path):
    P = prob
    src = _state(P)
    path = str(tmp_path / "t.nc")
    R.write_state(src, "Q", 4, path, ["a", "b", "c"])
    dst = _state(P)
    before = dst.download("Q")
    R.read_state(dst, "Q", 4, path, ["c", "a"], slots=[0, 2])
    after = dst.download("Q")
    q = src.download("Q")
    assert np.array_equal(interior(after[4, 0], P.n), interior(q[4, 2], P.n))
    assert np.array_equal(interior(after[4, 2], P.n), interior(q[4, 0], P.n))
    assert np.array_equal(after[4, 1], before[4, 1]) and np.array_equal(after[:4], before[:4])


def test_step_from_restart_equals_step_from_upload(cuda, prob, tmp_path):
    """A state whose tracers and delp come from restart files (interiors only) steps to the same interior as
    one uploaded with halos: the six-tile state rebuilds every halo cell it reads."""
    P = prob
    a = _state(P)
    R.save_restart(a, str(tmp_path), NAMES, delp=True)
    b = _state(P, upload=False)
    for name, val in (("CX", P.cx), ("CY", P.cy), ("MFX", P.mfx), ("MFY", P.mfy)):
        b.upload(name, val.numpy())
    R.load_restart(b, str(tmp_path))
    a.step(3)
    b.step(3)
    qa, qb = a.download("Q_REMAPPED"), b.download("Q_REMAPPED")
    assert np.array_equal(interior(qa, P.n), interior(qb, P.n))  # halos of the output are not part of it


def test_shape_and_argument_errors(cuda, prob, tmp_path):
    P = prob
    st = _state(P, upload=False)
    path = str(tmp_path / "small.nc")
    write_fields(path, {"sphum": np.ones((P.npz, 8, 8))})
    with pytest.raises(Fv3gError, match="is not"):
        R.read_state(st, "Q", 0, path, ["sphum"])
    with pytest.raises(Fv3gError, match="tile"):
        R.write_state(st, "Q", 6, str(tmp_path / "x.nc"), ["sphum"])
    with pytest.raises(Fv3gError, match="slot"):
        R.write_state(st, "Q", 0, str(tmp_path / "x.nc"), ["sphum"], slots=[P.nq])
    assert not os.path.exists(str(tmp_path / "x.nc"))
