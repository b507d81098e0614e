"""Trajectory output and dynamical observables around the Brownian step, as the reference's
trajectory driver produces them (runTrajectory.cpp:104-169):

* ``logSpacedIntegers`` -- the save schedule of inc/simpleUtilities.h:5-41;
* ``vectorValueNetCDF`` -- records of (value, vector[N]) in a NetCDF-3 classic file with the layout
  of src/databases/vectorValueNetCDF.cpp:3-36 (dimensions record (unlimited), unit = 1, N; double
  variables value(record, unit) and vector(record, N)), written directly in the classic format so
  that no NetCDF library is needed;
* ``dynamicalFeatures`` -- the mean squared geodesic displacement and the overlap function of the
  cell positions (src/analysis/dynamicalFeatures.cpp:6-53), reduced on the device
  (svm_model_dynamics);
* ``run_trajectory`` -- the driver: stabilisation, initialisation, then states, MSD and overlap at
  log-spaced steps.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import struct

import numpy as np

from ._lib import call


class logSpacedIntegers:
    """Integers round(10^(k exponent)), each once, starting after `firstSave`."""

    def __init__(self, firstSave: int = 0, exponent: float = 0.05):
        self.nextSave = int(firstSave)
        self.exponent = float(exponent)
        self.base = math.pow(10.0, self.exponent)
        self.logSaveIdx = 0
        if self.nextSave != 0:
            cur = 0
            while cur < self.nextSave:
                self.logSaveIdx += 1
                cur = int(_round_half_away(math.pow(self.base, self.logSaveIdx)))

    def update(self):
        self.logSaveIdx += 1
        cur = int(_round_half_away(math.pow(self.base, self.logSaveIdx)))
        while cur == self.nextSave:
            self.logSaveIdx += 1
            cur = int(_round_half_away(math.pow(self.base, self.logSaveIdx)))
        self.nextSave = cur


def _round_half_away(x: float) -> float:
    """C's round(): halves away from zero (Python's round() rounds them to even)."""
    return math.floor(x + 0.5) if x >= 0 else math.ceil(x - 0.5)


# ---- NetCDF-3 classic (CDF-1), big-endian ---------------------------------------------------------
_NC_DIMENSION, _NC_VARIABLE, _NC_DOUBLE = 0x0A, 0x0B, 6


def _name(s: str) -> bytes:
    b = s.encode()
    return struct.pack(">i", len(b)) + b + b"\0" * ((4 - len(b) % 4) % 4)


class vectorValueNetCDF:
    """Records (value, vector[N]) appended to a NetCDF-3 classic file; mode "replace" starts a new
    file (NcFile::Replace)."""

    def __init__(self, filename: str, N: int, mode: str = "replace"):
        if mode != "replace":
            raise ValueError("only mode='replace' is supported")
        self.filename, self.N = filename, int(N)
        dims = [("record", 0), ("unit", 1), ("N", self.N)]
        head = b"CDF\x01" + struct.pack(">i", 0)
        head += struct.pack(">ii", _NC_DIMENSION, len(dims))
        for nm, ln in dims:
            head += _name(nm) + struct.pack(">i", ln)
        head += struct.pack(">ii", 0, 0)  # no global attributes
        # two record variables: value(record, unit), vector(record, N); begin offsets filled below
        self._vsize = [8, 8 * self.N]
        var_part_len = 8
        for nm, ndim in (("value", 2), ("vector", 2)):
            var_part_len += len(_name(nm)) + 4 + 4 * ndim + 8 + 4 + 4 + 4
        self.header_size = len(head) + var_part_len
        begin = [self.header_size, self.header_size + self._vsize[0]]
        head += struct.pack(">ii", _NC_VARIABLE, 2)
        for i, (nm, dimids) in enumerate((("value", (0, 1)), ("vector", (0, 2)))):
            head += _name(nm) + struct.pack(">i", len(dimids)) + struct.pack(">%di" % len(dimids), *dimids)
            head += struct.pack(">ii", 0, 0)  # no variable attributes
            head += struct.pack(">iii", _NC_DOUBLE, self._vsize[i], begin[i])
        assert len(head) == self.header_size
        self.recsize = sum(self._vsize)
        self.records = 0
        with open(filename, "wb") as f:
            f.write(head)

    def writeState(self, vec, val: float):
        v = np.ascontiguousarray(vec, dtype=">f8").reshape(-1)
        if v.size != self.N:
            raise ValueError(f"vector of {v.size} values for a file of N = {self.N}")
        with open(self.filename, "r+b") as f:
            f.seek(self.header_size + self.records * self.recsize)
            f.write(struct.pack(">d", float(val)) + v.tobytes())
            self.records += 1
            f.seek(4)
            f.write(struct.pack(">i", self.records))


class dynamicalFeatures:
    """MSD and overlap of the model's cell positions against those at construction (the first
    floor(N fractionAnalyzed) cells), reduced on the device."""

    def __init__(self, model, fractionAnalyzed: float = 1.0):
        self.model = model
        self.fraction = float(fractionAnalyzed)
        call("svm_model_set_dynamics_reference", model.handle)

    def _both(self, cutoff: float):
        msd, ov = C.c_double(), C.c_double()
        call("svm_model_dynamics", self.model.handle, self.fraction, float(cutoff), C.byref(msd), C.byref(ov))
        return msd.value, ov.value

    def computeMSD(self) -> float:
        return self._both(0.5)[0]

    def computeOverlapFunction(self, cutoff: float = 0.5) -> float:
        return self._both(cutoff)[1]


def run_trajectory(N: int = 100, maximumIterations: int = 0, fIdx: int = -1, temperature: float = 0.001,
                   p0: float = 3.78, a0: float = 1.0, kr: float = 1.0, dt: float = 0.001, outdir: str = "data",
                   seed: int | None = None, verbose: bool = False):
    """runTrajectory.cpp's main path with the GPU model: 10/dt stabilisation steps at T = 0,
    P0 = 1 and timestep dt/100; min(maximumIterations, 1000/dt) steps at (T, a0, p0, dt); then, for
    fIdx >= 0, maximumIterations steps with, at log-spaced steps, the cell positions and energy,
    the MSD and the overlap appended to data/{cellPositions,msd,overlap}_N..._fidx...nc.  Returns the
    list of (step, energy, msd, overlap) written."""
    from .model import Simulation, brownianDynamics, noiseSource, sphericalVertexModel
    reproducible = fIdx <= 0
    noise = noiseSource(reproducible)
    if seed is not None:
        noise.setReproducibleSeed(seed)
    model = sphericalVertexModel(N, noise, a0, p0)
    model.setScalarModelParameter(kr)
    bd = brownianDynamics(reproducible)
    if seed is not None:
        bd.noise.setReproducibleSeed(seed + 1)
    sim = Simulation()
    sim.setConfiguration(model)
    sim.addUpdater(bd, model)
    steps_per_tau = int(math.floor(1.0 / dt))
    sim.setIntegrationTimestep(0.01 * dt)
    bd.setT(0.0)
    model.setPreferredParameters(1.0, 1.0)
    for _ in range(10 * steps_per_tau):
        sim.performTimestep()
    sim.setIntegrationTimestep(dt)
    bd.setT(temperature)
    model.setPreferredParameters(a0, p0)
    for _ in range(min(maximumIterations, 1000 * steps_per_tau)):
        sim.performTimestep()
    out = []
    if fIdx < 0:
        return out
    dyn = dynamicalFeatures(model)
    lsi = logSpacedIntegers(0, 0.05)
    lsi.update()
    tag = f"N{N}_p{p0:.4f}_T{temperature:.5f}_kr{kr:.3f}_fidx{fIdx}"
    os.makedirs(outdir, exist_ok=True)
    vv = vectorValueNetCDF(os.path.join(outdir, f"cellPositions_{tag}.nc"), N * 3)
    msd_f = vectorValueNetCDF(os.path.join(outdir, f"msd_{tag}.nc"), 2)
    ov_f = vectorValueNetCDF(os.path.join(outdir, f"overlap_{tag}.nc"), 2)
    for ii in range(maximumIterations):
        if ii == lsi.nextSave:
            lsi.update()
            e = sim.computeEnergy()
            vv.writeState(model.cellPositions().reshape(-1), e)
            msd, overlap = dyn._both(0.5)
            msd_f.writeState([ii * dt, msd], ii)
            ov_f.writeState([ii * dt, overlap], ii)
            out.append((ii, e, msd, overlap))
            if verbose:
                print(f"wrote state at timestep {ii}  {msd}  {overlap}")
        sim.performTimestep()
    return out
