"""jif3D's netCDF data and model files through the library's own reader and
writer (host code, no GPU): the netCDF-4 files of jif3D's Tutorial 5 against
the values the tutorial notebook printed, classic files cross-checked with
scipy's independent NetCDF-3 reader and writer, and the jif3D layouts
(variable names, units, dimensions, [Depth][Easting][Northing] order, upper
cell corners plus an origin) round-tripped through the model and data
classes.  Reading and writing are exact (values compare bit for bit)."""
import json
import os

import numpy as np
import pytest

from jif3d_gb300 import capi, gravmag as G, netcdf as N

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
scipy_io = pytest.importorskip("scipy.io")


def golden(name):
    return os.path.join(GOLDEN, name)


def test_tutorial_files_are_netcdf4_and_match_the_notebook():
    meta = json.load(open(golden("netcdf_tutorial.json")))
    Data, X, Y, Z, Err = N.ReadTotalFieldMagneticMeasurements(golden("tutorial5_magdata.nc"))
    p = meta["magdata_printed"]
    assert X.min() == float(p["min_x"]) and X.max() == float(p["max_x"])
    assert Y.min() == float(p["min_y"]) and Y.max() == float(p["max_y"])
    spacing = np.sqrt((X[0] - X[1]) ** 2 + (Y[0] - Y[1]) ** 2)
    assert abs(spacing - float(p["spacing"])) <= 1e-12 * spacing
    assert Data.size == X.size == Y.size == Z.size == Err.size == 748
    with capi.NcFile(golden("tutorial5_magdata.nc")) as f:
        assert f.format == 4  # HDF5
        assert sorted(f.variables()) == ["MeasPosX", "MeasPosY", "MeasPosZ", "T", "dT"]
        assert f.dim("StationNumber") == 748
        assert f.att("T", "units") == "nT" and f.att("MeasPosX", "units") == "m"
    assert N.IdentifyGravityDatafileType(golden("tutorial5_gravdata.nc")) == N.scalar
    assert N.IdentifyGravityDatafileType(golden("tutorial5_magdata.nc")) == N.unknown
    g, gx, gy, gz, ge = N.ReadScalarGravityMeasurements(golden("tutorial5_gravdata.nc"))
    assert g.size == gx.size == 760 and np.all(ge == 1e-5) and np.all(gz == -0.3)
    # the two surveys cover the same area
    assert abs(gx.min() - X.min()) < 1e3 and abs(gy.max() - Y.max()) < 1e3
    D = G.ScalarGravityData()
    D.ReadNetCDF(golden("tutorial5_gravdata.nc"))
    assert np.array_equal(D.GetData(), g) and np.array_equal(D.GetMeasPosX(), gx)


def test_data_files_roundtrip_and_scipy_reads_them(tmp_path):
    rng = np.random.default_rng(1)
    n = 17
    X, Y, Z = rng.normal(size=(3, n)) * 1e3
    d, e = rng.normal(size=n) * 1e-5, np.full(n, 1e-7)
    f = str(tmp_path / "scalar.nc")
    N.SaveScalarGravityMeasurements(f, d, X, Y, Z, e)
    back = N.ReadScalarGravityMeasurements(f)
    for a, b in zip(back, (d, X, Y, Z, e)):
        assert np.array_equal(a, b)
    with scipy_io.netcdf_file(f, "r", mmap=False) as s:
        assert s.version_byte == 2
        assert s.dimensions == {"StationNumber": n}
        assert np.array_equal(s.variables["Scalar_gravity"][:], d)
        assert s.variables["dGz"].units == b"m/s2" and s.variables["MeasPosZ"].units == b"m"
        assert s.variables["MeasPosX"].dimensions == ("StationNumber",)
    # tensor: nine variables and nine errors, nine values per station
    t, te = rng.normal(size=9 * n), rng.uniform(size=9 * n)
    f = str(tmp_path / "ftg.nc")
    N.SaveTensorGravityMeasurements(f, t, X, Y, Z, te)
    assert N.IdentifyGravityDatafileType(f) == N.ftg
    back = N.ReadTensorGravityMeasurements(f)
    assert np.array_equal(back[0], t) and np.array_equal(back[4], te)
    with scipy_io.netcdf_file(f, "r", mmap=False) as s:
        assert np.array_equal(s.variables["Uyz"][:], t.reshape(n, 9)[:, 5])
        assert np.array_equal(s.variables["dUzx"][:], te.reshape(n, 9)[:, 6])
        assert s.variables["Uxx"].units == b"1/s2"
    # magnetics
    f = str(tmp_path / "tf.nc")
    N.SaveTotalFieldMagneticMeasurements(f, d, X, Y, Z, e)
    assert all(np.array_equal(a, b) for a, b in
               zip(N.ReadTotalFieldMagneticMeasurements(f), (d, X, Y, Z, e)))
    b3, e3 = rng.normal(size=3 * n), rng.uniform(size=3 * n)
    f = str(tmp_path / "b3.nc")
    N.SaveMagneticComponentMeasurements(f, b3, X, Y, Z, e3)
    back = N.ReadMagneticComponentMeasurements(f)
    assert np.array_equal(back[0], b3) and np.array_equal(back[4], e3)
    D = G.ThreeComponentMagneticData()
    D.ReadNetCDF(f)
    f2 = str(tmp_path / "b3_again.nc")
    D.WriteNetCDF(f2)
    assert np.array_equal(N.ReadMagneticComponentMeasurements(f2)[0], b3)


def test_files_written_by_scipy_are_read(tmp_path):
    """Classic files from an independent writer: CDF-1 and CDF-2, a record
    (unlimited) dimension, int / float / double variables, global text."""
    rng = np.random.default_rng(2)
    for version in (1, 2):
        f = str(tmp_path / f"v{version}.nc")
        with scipy_io.netcdf_file(f, "w", version=version) as s:
            s.history = "made by scipy"
            s.createDimension("time", None)
            s.createDimension("StationNumber", 5)
            for name in ("MeasPosX", "MeasPosY", "MeasPosZ", "T", "dT"):
                v = s.createVariable(name, "d", ("StationNumber",))
                v[:] = rng.normal(size=5)
                v.units = "nT" if name.endswith("T") else "m"
            iv = s.createVariable("count", "i", ("StationNumber",))
            iv[:] = np.arange(5, dtype=np.int32) - 2
            fv = s.createVariable("half", "f", ("StationNumber",))
            fv[:] = np.linspace(0, 1, 5, dtype=np.float32)
            rv = s.createVariable("rec", "d", ("time", "StationNumber"))
            rv[0, :] = np.arange(5.0)
            rv[1, :] = np.arange(5.0) * 10
            rv2 = s.createVariable("rec2", "i", ("time",))
            rv2[:2] = [7, 8]
            expect = {n: s.variables[n][:].copy() for n in s.variables}
        with capi.NcFile(f) as r:
            assert r.format == version
            assert r.att(None, "history") == "made by scipy"
            for name, val in expect.items():
                assert np.array_equal(r.read(name), np.asarray(val, dtype=float)), name
            assert r.dim("time") == 2 and r.shape("rec") == (2, 5)
        data = N.ReadTotalFieldMagneticMeasurements(f)
        assert np.array_equal(data[0], expect["T"])


def test_cdf5_file_is_read(tmp_path):
    """A CDF-5 (64-bit data) file built byte by byte from the format
    specification: one dimension, one int64 and one double variable."""
    def be32(v):
        return int(v).to_bytes(4, "big")

    def be64(v):
        return int(v).to_bytes(8, "big", signed=True)

    def name(s):
        b = s.encode()
        return be64(len(b)) + b + b"\0" * (-len(b) % 4)
    vals = np.array([1.5, -2.25, 3.0])
    ints = [-(2 ** 40), 5, 2 ** 50]
    header = b"CDF\x05" + be64(0)
    header += be32(0x0A) + be64(1) + name("n") + be64(3)
    header += be32(0) + be64(0)  # no global attributes
    var_i = name("big") + be64(1) + be64(0) + be32(0) + be64(0) + be32(10) + be64(24)
    var_d = name("x") + be64(1) + be64(0) + be32(0) + be64(0) + be32(6) + be64(24)
    size = len(header) + 4 + 8 + len(var_i) + 8 + len(var_d) + 8
    body = be32(0x0B) + be64(2) + var_i + be64(size) + var_d + be64(size + 24)
    data = b"".join(be64(v) for v in ints) + vals.astype(">f8").tobytes()
    f = tmp_path / "cdf5.nc"
    f.write_bytes(header + body + data)
    with capi.NcFile(str(f)) as r:
        assert r.format == 5
        assert np.array_equal(r.read("x"), vals)
        assert np.array_equal(r.read("big"), np.array(ints, dtype=float))


def make_model(cls, rng, nx=4, ny=3, nz=5, bg=True):
    M = cls()
    M.SetMeshSize(nx, ny, nz)
    M.SetXCellSizes(rng.uniform(10, 30, nx).round(1))
    M.SetYCellSizes(rng.uniform(10, 30, ny).round(1))
    M.SetZCellSizes(rng.uniform(5, 20, nz))
    M.SetOrigin(100.5, -20.25, 0.0)
    M.SetData()[...] = rng.normal(size=(nx, ny, nz))
    if bg:
        M.SetBackgroundThicknesses([100.0, 200.0])
        M.SetBackgroundValues([2.5, 2.7])
    return M


def test_gravity_model_layout_and_roundtrip(tmp_path):
    rng = np.random.default_rng(3)
    M = make_model(G.ThreeDGravityModel, rng)
    f = str(tmp_path / "grav.nc")
    M.WriteNetCDF(f)
    with scipy_io.netcdf_file(f, "r", mmap=False) as s:
        assert s.Conventions == b"CF-1.3"
        dens = s.variables["Density"]
        assert dens.dimensions == ("Depth", "Easting", "Northing")
        assert dens.units == b"kg/m3"
        assert np.array_equal(dens[:], M.GetData().transpose(2, 1, 0))
        assert np.array_equal(s.variables["Northing"][:], M.GetXCoordinates()[1:])
        assert s.variables["Northing"].bounds == b"Northing_bnds"
        assert float(s.variables["Easting_Origin"].getValue()) == -20.25
        assert np.array_equal(s.variables["Depth_bnds"][:, 0], M.GetZCoordinates()[:-1])
        assert np.array_equal(s.variables["nbound"][:], [1, 2])
        assert np.array_equal(s.variables["bg_densities"][:], [2.5, 2.7])
        assert s.variables["bg_thicknesses"].units == b"m"
    R = G.ThreeDGravityModel()
    R.ReadNetCDF(f)
    for get in ("GetXCoordinates", "GetYCoordinates", "GetZCoordinates", "GetData",
                "GetBackgroundValues", "GetBackgroundThicknesses"):
        assert np.array_equal(getattr(R, get)(), getattr(M, get)()), get
    # old files in g/cm3 are scaled to kg/m3 (ThreeDGravityModel.cpp:111-124)
    f2 = str(tmp_path / "old.nc")
    with scipy_io.netcdf_file(f, "r", mmap=False) as s, \
            scipy_io.netcdf_file(f2, "w", version=2) as o:
        for k, v in s.dimensions.items():
            o.createDimension(k, v)
        for k, v in s.variables.items():
            w = o.createVariable(k, v.typecode(), v.dimensions)
            w[...] = v[...]
            for a, val in v._attributes.items():
                setattr(w, a, val)
        o.variables["Density"].units = "g/cm3"
    R2 = G.ThreeDGravityModel()
    R2.ReadNetCDF(f2)
    assert np.array_equal(R2.GetData(), 1000.0 * M.GetData())
    assert np.array_equal(R2.GetBackgroundValues(), 1000.0 * M.GetBackgroundValues())


def test_susceptibility_and_magnetization_models(tmp_path):
    rng = np.random.default_rng(4)
    S = make_model(G.ThreeDSusceptibilityModel, rng, bg=False)
    f = str(tmp_path / "sus.nc")
    S.WriteNetCDF(f)
    with capi.NcFile(f) as r:
        assert r.att("Susceptibility", "units") == " " and not r.has_dim("bg_layers")
    R = G.ThreeDSusceptibilityModel()
    R.ReadNetCDF(f)
    assert np.array_equal(R.GetData(), S.GetData())
    with pytest.raises(N.FatalException):  # wrong units for a density model
        G.ThreeDGravityModel().ReadNetCDF(f)
    M = G.ThreeDMagnetizationModel()
    M.SetMeshSize(3, 2, 4)
    M.SetXCellSizes([10.0, 20.0, 30.0])
    M.SetYCellSizes([5.0, 5.0])
    M.SetZCellSizes([1.0, 2.0, 3.0, 4.0])
    for arr in (M.SetMagnetization_X(), M.SetMagnetization_Y(), M.SetMagnetization_Z()):
        arr[...] = rng.normal(size=arr.shape)
    f = str(tmp_path / "mag.nc")
    M.WriteNetCDF(f)
    R = G.ThreeDMagnetizationModel()
    R.ReadNetCDF(f)
    for get in ("GetMagnetization_X", "GetMagnetization_Y", "GetMagnetization_Z",
                "GetXCoordinates", "GetZCoordinates"):
        assert np.array_equal(getattr(R, get)(), getattr(M, get)()), get


def test_errors(tmp_path):
    with pytest.raises(N.FatalException):
        N.ReadScalarGravityMeasurements(str(tmp_path / "missing.nc"))
    bad = tmp_path / "bad.nc"
    bad.write_bytes(b"not a netcdf file at all")
    with pytest.raises(capi.J3GError):
        capi.NcFile(str(bad))
    f = str(tmp_path / "t.nc")
    N.SaveTotalFieldMagneticMeasurements(f, [1.0], [0.0], [0.0], [0.0], [0.1])
    with pytest.raises(capi.J3GError):  # no such variable
        N.ReadScalarGravityMeasurements(f)
    with pytest.raises(capi.J3GError):  # a variable defined but never written
        with capi.NcWriter(str(tmp_path / "w.nc")) as w:
            w.add_dim("n", 2)
            w.add_var("a", ("n",))
    with pytest.raises(ValueError):  # the writer is discarded, no file appears
        with capi.NcWriter(str(tmp_path / "never.nc")) as w:
            w.add_dim("n", 2)
            raise ValueError("stop")
    assert not (tmp_path / "never.nc").exists()
