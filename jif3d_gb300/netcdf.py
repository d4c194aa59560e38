"""jif3D's netCDF data and model files, read and written by the library's own
NetCDF reader / writer (``capi.NcFile`` / ``capi.NcWriter``; no NetCDF or
HDF5 library): the same variable names, units, dimensions and layouts as

* Gravity/ReadWriteGravityData.cpp (scalar and FTG data),
* Magnetics/ReadWriteMagneticData.cpp (total-field and three-component data),
* ModelBase/NetCDFModelTools.cpp (the rectilinear mesh and a 3-D cell array),
* Gravity/ThreeDGravityModel.cpp:75-162, Magnetics/ThreeDSusceptibilityModel.h:
  112-190, Magnetics/ThreeDMagnetizationModel.cpp:28-160 (models with their
  background layers or magnetisation components).

Files are written as NetCDF classic (CDF-2); jif3D's own netCDF-4 files are
read as they are.  Positions are in m, gravity in m/s^2, tensors in 1/s^2,
magnetic fields in nT.
"""
from __future__ import annotations

import numpy as np

from . import capi

SCALAR_GRAVITY, TENSOR_NAMES = "Scalar_gravity", ("Uxx", "Uxy", "Uxz", "Uyx", "Uyy", "Uyz",
                                                  "Uzx", "Uzy", "Uzz")
SCALAR_ERROR = "dGz"
MAG_COMPONENTS, MAG_COMPONENT_ERRORS = ("Bx", "By", "Bz"), ("dBx", "dBy", "dBz")
TOTAL_FIELD, TOTAL_FIELD_ERROR = "T", "dT"
MEAS_POS = ("MeasPosX", "MeasPosY", "MeasPosZ")
STATION_NUMBER = "StationNumber"
# GravityDataType (Gravity/ReadWriteGravityData.h)
scalar, ftg, unknown = "scalar", "ftg", "unknown"


class FatalException(RuntimeError):
    """jif3D::FatalException for file problems."""


def _open(filename):
    try:
        return capi.NcFile(filename)
    except capi.J3GError as e:
        raise FatalException(str(e)) from e


def _positions(f):
    return tuple(f.read(n).reshape(-1) for n in MEAS_POS)


def _write_positions(w, PosX, PosY, PosZ):
    w.add_dim(STATION_NUMBER, len(PosX))
    for name, v in zip(MEAS_POS, (PosX, PosY, PosZ)):
        w.add_var(name, (STATION_NUMBER,), values=v, units="m")


def _check_sizes(n, *vs):
    for v in vs:
        if len(v) != n:
            raise FatalException("inconsistent sizes of data and positions")


# -- gravity data (Gravity/ReadWriteGravityData.cpp) ---------------------------
def IdentifyGravityDatafileType(filename):
    """:75-90: 'scalar' if the file has Scalar_gravity, 'ftg' if it has Uxx."""
    with _open(filename) as f:
        if f.has_var(SCALAR_GRAVITY):
            return scalar
        if f.has_var("Uxx"):
            return ftg
    return unknown


def SaveScalarGravityMeasurements(filename, Data, PosX, PosY, PosZ, Error):
    """:100-122."""
    _check_sizes(len(Data), PosX, PosY, PosZ, Error)
    with capi.NcWriter(filename) as w:
        _write_positions(w, PosX, PosY, PosZ)
        w.add_var(SCALAR_GRAVITY, (STATION_NUMBER,), values=Data, units="m/s2")
        w.add_var(SCALAR_ERROR, (STATION_NUMBER,), values=Error, units="m/s2")


def ReadScalarGravityMeasurements(filename):
    """:132-155: (Data, PosX, PosY, PosZ, Error); zero errors if the file has none."""
    with _open(filename) as f:
        PosX, PosY, PosZ = _positions(f)
        Data = f.read(SCALAR_GRAVITY).reshape(-1)
        Error = f.read(SCALAR_ERROR).reshape(-1) if f.has_var(SCALAR_ERROR) else \
            np.zeros(Data.size)
    return Data, PosX, PosY, PosZ, Error


def SaveTensorGravityMeasurements(filename, Data, PosX, PosY, PosZ, Error):
    """:215-240: nine components per station, one variable per component
    (Uxx ... Uzz) and its error (dUxx ... dUzz), units 1/s2."""
    n = len(PosX)
    _check_sizes(n, PosY, PosZ)
    D = np.asarray(Data, dtype=float).reshape(n, 9)
    E = np.asarray(Error, dtype=float).reshape(n, 9)
    with capi.NcWriter(filename) as w:
        _write_positions(w, PosX, PosY, PosZ)
        for i, name in enumerate(TENSOR_NAMES):
            w.add_var(name, (STATION_NUMBER,), values=D[:, i], units="1/s2")
        for i, name in enumerate(TENSOR_NAMES):
            w.add_var("d" + name, (STATION_NUMBER,), values=E[:, i], units="1/s2")


def ReadTensorGravityMeasurements(filename):
    """:166-205: (Data, PosX, PosY, PosZ, Error), nine values per station;
    components without an error variable get zero errors."""
    with _open(filename) as f:
        PosX, PosY, PosZ = _positions(f)
        n = PosX.size
        Data = np.zeros((n, 9))
        Error = np.zeros((n, 9))
        for i, name in enumerate(TENSOR_NAMES):
            Data[:, i] = f.read(name).reshape(-1)
            if f.has_var("d" + name):
                Error[:, i] = f.read("d" + name).reshape(-1)
    return Data.reshape(-1), PosX, PosY, PosZ, Error.reshape(-1)


# -- magnetic data (Magnetics/ReadWriteMagneticData.cpp) -------------------------
def SaveTotalFieldMagneticMeasurements(filename, Data, PosX, PosY, PosZ, Error):
    _check_sizes(len(Data), PosX, PosY, PosZ)
    with capi.NcWriter(filename) as w:
        _write_positions(w, PosX, PosY, PosZ)
        w.add_var(TOTAL_FIELD, (STATION_NUMBER,), values=Data, units="nT")
        w.add_var(TOTAL_FIELD_ERROR, (STATION_NUMBER,), values=Error, units="nT")


def ReadTotalFieldMagneticMeasurements(filename):
    """(Data, PosX, PosY, PosZ, Error).  Without a dT variable the error
    vector is empty, as the reference's resize-then-clear leaves it."""
    with _open(filename) as f:
        PosX, PosY, PosZ = _positions(f)
        Data = f.read(TOTAL_FIELD).reshape(-1)
        Error = f.read(TOTAL_FIELD_ERROR).reshape(-1) if f.has_var(TOTAL_FIELD_ERROR) else \
            np.zeros(0)
    return Data, PosX, PosY, PosZ, Error


def SaveMagneticComponentMeasurements(filename, Data, PosX, PosY, PosZ, Error):
    """Bx, By, Bz and dBx, dBy, dBz per station (three values per station)."""
    n = len(PosX)
    _check_sizes(n, PosY, PosZ)
    D = np.asarray(Data, dtype=float).reshape(n, 3)
    E = np.asarray(Error, dtype=float).reshape(n, 3)
    with capi.NcWriter(filename) as w:
        _write_positions(w, PosX, PosY, PosZ)
        for i, name in enumerate(MAG_COMPONENTS):
            w.add_var(name, (STATION_NUMBER,), values=D[:, i], units="nT")
        for i, name in enumerate(MAG_COMPONENT_ERRORS):
            w.add_var(name, (STATION_NUMBER,), values=E[:, i], units="nT")


def ReadMagneticComponentMeasurements(filename):
    with _open(filename) as f:
        PosX, PosY, PosZ = _positions(f)
        n = PosX.size
        Data = np.zeros((n, 3))
        Error = np.zeros((n, 3))
        for i, name in enumerate(MAG_COMPONENTS):
            Data[:, i] = f.read(name).reshape(-1)
        for i, name in enumerate(MAG_COMPONENT_ERRORS):
            if f.has_var(name):
                Error[:, i] = f.read(name).reshape(-1)
    return Data.reshape(-1), PosX, PosY, PosZ, Error.reshape(-1)


def ReadMeasPosNetCDF(filename):
    """ModelBase/NetCDFModelTools.cpp ReadMeasPosNetCDF: (PosX, PosY, PosZ)."""
    with _open(filename) as f:
        return _positions(f)


# -- models (ModelBase/NetCDFModelTools.cpp) -------------------------------------
_AXES = ("Northing", "Easting", "Depth")


def _write_axis(w, name, corners):
    """WriteCoordinatesToNetCDF: the upper corner of each cell, the cell
    bounds and the origin as a scalar variable."""
    c = np.asarray(corners, dtype=float)
    n = c.size - 1
    w.add_dim(name, n)
    w.add_var(name, (name,), values=c[1:], units="m", long_name=name + " coordinate",
              bounds=name + "_bnds")
    w.add_var(name + "_bnds", (name, "nbound"), values=np.stack([c[:-1], c[1:]], axis=1),
              units="m")
    w.add_var(name + "_Origin", (), values=c[:1])


def Write3DModelToNetCDF(w, DataName, UnitsName, XCellCoords, YCellCoords, ZCellCoords, Data,
                         extra=()):
    """Write3DModelToNetCDF: the mesh and one cell array, stored
    [Depth][Easting][Northing] (Northing fastest); ``extra`` adds more cell
    arrays (name, units, values) on the same mesh."""
    w.add_dim("nbound", 2)
    w.add_var("nbound", ("nbound",), type=capi.NC_INT, values=[1, 2],
              long_name="Boundary index variable")
    for name, c in zip(_AXES, (XCellCoords, YCellCoords, ZCellCoords)):
        _write_axis(w, name, c)
    for name, units, values in ((DataName, UnitsName, Data),) + tuple(extra):
        w.add_var(name, ("Depth", "Easting", "Northing"),
                  values=np.asarray(values, dtype=float).transpose(2, 1, 0), units=units,
                  long_name=name)
    w.put_att(None, "Conventions", "CF-1.3")


def _read_axis(f, name):
    """ReadCoordinatesFromNetCDF: n + 1 corners (origin first), increasing."""
    n = f.dim(name)
    if n == 0:
        raise FatalException("Cell coordinate is empty: " + name)
    c = np.empty(n + 1)
    c[1:] = f.read(name).reshape(-1)[:n]
    c[0] = float(f.read(name + "_Origin").reshape(-1)[0]) if f.has_var(name + "_Origin") else 0.0
    if np.any(np.diff(c) < 0):
        raise FatalException("Cell coordinates in netcdf file are not in increasing order: " +
                             name)
    return c


def Read3DModelFromNetCDF(f, DataName, UnitsName):
    """(XCellCoords, YCellCoords, ZCellCoords, Data[x][y][z]); the units of the
    cell array must be UnitsName."""
    if not f.has_var(DataName):
        raise FatalException("Cannot read variable: " + DataName)
    X, Y, Z = (_read_axis(f, a) for a in _AXES)
    if (f.att(DataName, "units") or "") != UnitsName:
        raise FatalException("Units in file do not match expected units !")
    return X, Y, Z, _cells(f, DataName, X, Y, Z)


def _cells(f, name, X, Y, Z):
    v = f.read(name)
    shape = (Z.size - 1, Y.size - 1, X.size - 1)
    if v.size != int(np.prod(shape)):
        raise FatalException("Cell size specification does not match data !")
    return v.reshape(shape).transpose(2, 1, 0).copy()


def _model_geometry(M, X, Y, Z, data):
    M.SetMeshSize(X.size - 1, Y.size - 1, Z.size - 1)
    M.SetXCoordinates(X)
    M.SetYCoordinates(Y)
    M.SetZCoordinates(Z)
    M.SetData()[...] = data


def WriteLayeredModel(M, filename, name, units, bg_name, bg_long):
    """ThreeDGravityModel::WriteNetCDF / ThreeDSusceptibilityModel::WriteNetCDF:
    the cell array and, if any, the background layers (bg_layers dimension)."""
    with capi.NcWriter(filename) as w:
        Write3DModelToNetCDF(w, name, units, M.GetXCoordinates(), M.GetYCoordinates(),
                             M.GetZCoordinates(), M.GetData())
        bg = M.GetBackgroundValues()
        if bg.size:
            th = M.GetBackgroundThicknesses()
            if th.size != bg.size:
                raise FatalException("background values and thicknesses differ in number")
            w.add_dim("bg_layers", bg.size)
            w.add_var(bg_name, ("bg_layers",), values=bg, long_name=bg_long, units=units)
            w.add_var("bg_thicknesses", ("bg_layers",), values=th,
                      long_name="Background Thicknesses", units="m")


def ReadLayeredModel(M, filename, name, units, bg_name, old_units=None, old_factor=1.0):
    """ThreeDGravityModel::ReadNetCDF (old "g/cm3" densities are scaled by
    1000) / ThreeDSusceptibilityModel::ReadNetCDF."""
    with _open(filename) as f:
        if not f.has_var(name):
            raise FatalException("Cannot read variable: " + name)
        factor = 1.0
        unit = units
        if old_units is not None and f.att(name, "units") == old_units:
            factor, unit = old_factor, old_units
        X, Y, Z, data = Read3DModelFromNetCDF(f, name, unit)
        _model_geometry(M, X, Y, Z, factor * data)
        if f.has_dim("bg_layers"):
            M.SetBackgroundValues(factor * f.read(bg_name).reshape(-1))
            M.SetBackgroundThicknesses(f.read("bg_thicknesses").reshape(-1))


def WriteMagnetizationModel(M, filename):
    """ThreeDMagnetizationModel::WriteNetCDF: Mx, My, Mz in A/m."""
    with capi.NcWriter(filename) as w:
        Write3DModelToNetCDF(w, "Mx", "A/m", M.GetXCoordinates(), M.GetYCoordinates(),
                             M.GetZCoordinates(), M.GetMagnetization_X(),
                             extra=(("My", "A/m", M.GetMagnetization_Y()),
                                    ("Mz", "A/m", M.GetMagnetization_Z())))


def ReadMagnetizationModel(M, filename):
    with _open(filename) as f:
        X, Y, Z, mx = Read3DModelFromNetCDF(f, "Mx", "A/m")
        _model_geometry(M, X, Y, Z, mx)
        M.SetMagnetization_Y()[...] = _cells(f, "My", X, Y, Z)
        M.SetMagnetization_Z()[...] = _cells(f, "Mz", X, Y, Z)
