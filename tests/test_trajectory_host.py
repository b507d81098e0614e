"""Host side of the trajectory output: the log-spaced save schedule against the oracle's
restatement of logSpacedIntegers, and the NetCDF-3 records read back by an independent reader
(scipy) with the reference's layout (vectorValueNetCDF.cpp:3-36)."""
import numpy as np
import pytest

import oracle
from curvedspacevertexmodel_gb300.trajectory import logSpacedIntegers, vectorValueNetCDF


@pytest.mark.parametrize("first,exponent,count", [(0, 0.05, 150), (0, 0.1, 80), (37, 0.05, 150), (1000, 0.02, 150)])
def test_log_spaced_integers(first, exponent, count):
    """(count keeps the steps inside the int range the reference computes them in)"""
    ref = oracle.log_spaced(first, exponent, count)
    lsi = logSpacedIntegers(first, exponent)
    got = []
    for _ in range(count):
        got.append(lsi.nextSave)
        lsi.update()
    assert np.array_equal(np.array(got), ref)
    assert np.all(np.diff(ref) > 0)


def test_netcdf_records_read_back(tmp_path):
    netcdf = pytest.importorskip("scipy.io")
    fn = str(tmp_path / "cellPositions.nc")
    rng = np.random.default_rng(2)
    w = vectorValueNetCDF(fn, 12)
    recs = [(rng.normal(size=12), float(rng.normal())) for _ in range(5)]
    for vec, val in recs:
        w.writeState(vec, val)
    with netcdf.netcdf_file(fn, "r", mmap=False) as f:
        assert f.dimensions["record"] is None and f.dimensions["unit"] == 1 and f.dimensions["N"] == 12
        assert f.variables["vector"].dimensions == ("record", "N")
        assert f.variables["value"].dimensions == ("record", "unit")
        vec = np.array(f.variables["vector"][:])
        val = np.array(f.variables["value"][:])
    assert vec.shape == (5, 12) and val.shape == (5, 1)
    for i, (v, x) in enumerate(recs):
        assert np.array_equal(vec[i], v) and val[i, 0] == x
