"""Python host layer mirroring jif3D's gravity / magnetic plugin interface.

Names, argument meaning and error behaviour follow the reference classes so
that code (and tests) written against jif3D read the same here:

* models  -- ``ThreeDGravityModel`` / ``ThreeDSusceptibilityModel``
  (ModelBase/ThreeDModelBase.h, Gravity/ThreeDGravityModel.h,
  Magnetics/ThreeDSusceptibilityModel.h)
* data    -- ``ScalarGravityData``, ``TensorGravityData``,
  ``TotalFieldMagneticData`` (DataBase/GeneralData.h)
* transforms -- ``FTGInvariant``, ``TotalField``, ``TotalFieldAnomaly``
  (Gravity/GravityTransforms.h, Magnetics/MagneticTransforms.h)
* implementations -- ``ScalarGB300GravityImp``, ``TensorGB300GravityImp``,
  ``GB300MagneticSusceptibilityImp``, ``JointGB300GravityImp``: the GB300
  counterparts of the ThreeDGravMagImplementation subclasses
  (GravMag/ThreeDGravMagImplementation.h:39-84)
* calculators -- ``MinMemGravMagCalculator``, ``FullSensitivityGravMagCalculator``
  (GravMag/MinMemGravMagCalculator.h, GravMag/FullSensitivityGravMagCalculator.h),
  unchanged in behaviour: they drive the implementation exactly as the
  reference calculators drive theirs.

Every computation runs on the GPU through the C ABI (``capi``); the
calculators' cached products (J m, 2 J^T r) are the reference's host-side
products, as in FullSensitivityGravMagCalculator.
"""
from __future__ import annotations

import numpy as np

from . import capi


class FatalException(RuntimeError):
    """jif3D::FatalException (Global/FatalException.h:27)."""


# ---------------------------------------------------------------------------
# Models and data
class ThreeDModelBase:
    """Rectilinear mesh, z fastest, z positive down (ModelBase/ThreeDModelBase.h)."""

    def __init__(self):
        self._xs = np.zeros(0)
        self._ys = np.zeros(0)
        self._zs = np.zeros(0)
        self._origin = np.zeros(3)
        self._data = np.zeros((0, 0, 0))
        self._bg_values = np.zeros(0)
        self._bg_thick = np.zeros(0)
        # corner coordinates set as such (SetXCoordinates, e.g. read from a
        # file) are kept as given; otherwise they are the running sums
        self._corners = [None, None, None]

    # mesh -------------------------------------------------------------------
    def SetMeshSize(self, nx, ny, nz):
        self._xs = np.resize(self._xs, nx).astype(float)
        self._ys = np.resize(self._ys, ny).astype(float)
        self._zs = np.resize(self._zs, nz).astype(float)
        self._corners = [None, None, None]
        self._data = np.zeros((nx, ny, nz))

    def SetXCellSizes(self, v):
        self._xs = np.array(v, dtype=float)
        self._corners[0] = None

    def SetYCellSizes(self, v):
        self._ys = np.array(v, dtype=float)
        self._corners[1] = None

    def SetZCellSizes(self, v):
        self._zs = np.array(v, dtype=float)
        self._corners[2] = None

    def _set_corners(self, axis, c):
        """ThreeDModelBase::SetXCoordinates (ThreeDModelBase.h:92-108): the
        corners as given, the sizes their differences (CalcSizes)."""
        c = np.array(c, dtype=float)
        self._corners[axis] = c
        self._origin[axis] = c[0] if c.size else 0.0
        sizes = np.diff(c)
        if axis == 0:
            self._xs = sizes
        elif axis == 1:
            self._ys = sizes
        else:
            self._zs = sizes

    def SetXCoordinates(self, c):
        self._set_corners(0, c)

    def SetYCoordinates(self, c):
        self._set_corners(1, c)

    def SetZCoordinates(self, c):
        self._set_corners(2, c)

    def SetOrigin(self, x, y, z):
        self._origin = np.array([x, y, z], dtype=float)
        self._corners = [None, None, None]

    def GetXCellSizes(self):
        return self._xs

    def GetYCellSizes(self):
        return self._ys

    def GetZCellSizes(self):
        return self._zs

    @staticmethod
    def _coords(origin, sizes):
        # ThreeDModelBase::CalcCoords (ModelBase/ThreeDModelBase.cpp:96-113):
        # running sum of the sizes, in order, starting at the origin
        c = np.empty(sizes.size + 1)
        c[0] = origin
        s = origin
        for i, v in enumerate(sizes):
            s = s + v
            c[i + 1] = s
        return c

    def GetXCoordinates(self):
        c = self._corners[0]
        return c.copy() if c is not None else self._coords(self._origin[0], self._xs)

    def GetYCoordinates(self):
        c = self._corners[1]
        return c.copy() if c is not None else self._coords(self._origin[1], self._ys)

    def GetZCoordinates(self):
        c = self._corners[2]
        return c.copy() if c is not None else self._coords(self._origin[2], self._zs)

    def GetXOrigin(self):
        return float(self._origin[0])

    def GetYOrigin(self):
        return float(self._origin[1])

    def GetZOrigin(self):
        return float(self._origin[2])

    # values -----------------------------------------------------------------
    def SetData(self):
        return self._data

    def GetData(self):
        return self._data

    def SetBackgroundThicknesses(self, v):
        self._bg_thick = np.array(v, dtype=float)

    def GetBackgroundThicknesses(self):
        return self._bg_thick

    def SetBackgroundValues(self, v):
        self._bg_values = np.array(v, dtype=float)

    def GetBackgroundValues(self):
        return self._bg_values

    def GetModelParameters(self):
        """Grid values followed by the background values (ThreeDGravityModel.h:91-99)."""
        return np.concatenate([self._data.reshape(-1), self._bg_values])

    def GetNModelParm(self):
        return self._data.size + self._bg_values.size

    def GetNModelElements(self):
        return self._data.size


class ThreeDGravityModel(ThreeDModelBase):
    SetDensities = ThreeDModelBase.SetData
    GetDensities = ThreeDModelBase.GetData
    SetBackgroundDensities = ThreeDModelBase.SetBackgroundValues
    GetBackgroundDensities = ThreeDModelBase.GetBackgroundValues

    def WriteNetCDF(self, filename):
        """Gravity/ThreeDGravityModel.cpp:75-101: Density (kg/m3) and the
        background layers."""
        from . import netcdf
        netcdf.WriteLayeredModel(self, filename, "Density", "kg/m3", "bg_densities",
                                 "Background Densities")

    def ReadNetCDF(self, filename):
        """Gravity/ThreeDGravityModel.cpp:103-162 (g/cm3 files are scaled to kg/m3)."""
        from . import netcdf
        netcdf.ReadLayeredModel(self, filename, "Density", "kg/m3", "bg_densities",
                                old_units="g/cm3", old_factor=1000.0)


class ThreeDSusceptibilityModel(ThreeDModelBase):
    SetSusceptibilities = ThreeDModelBase.SetData
    GetSusceptibilities = ThreeDModelBase.GetData
    SetBackgroundSusceptibilities = ThreeDModelBase.SetBackgroundValues
    GetBackgroundSusceptibilities = ThreeDModelBase.GetBackgroundValues

    def WriteNetCDF(self, filename):
        """Magnetics/ThreeDSusceptibilityModel.h:112-148 (units " ")."""
        from . import netcdf
        netcdf.WriteLayeredModel(self, filename, "Susceptibility", " ",
                                 "bg_susceptibilities", "Background Susceptibilities")

    def ReadNetCDF(self, filename):
        """Magnetics/ThreeDSusceptibilityModel.h:150-190."""
        from . import netcdf
        netcdf.ReadLayeredModel(self, filename, "Susceptibility", " ", "bg_susceptibilities")


class ThreeDMagnetizationModel(ThreeDModelBase):
    """Remanent magnetisation: three cell arrays, model parameters x block, y
    block, z block and no background parameters
    (Magnetics/ThreeDMagnetizationModel.h:53-70)."""

    def __init__(self):
        super().__init__()
        self._my = np.zeros((0, 0, 0))
        self._mz = np.zeros((0, 0, 0))

    def SetMeshSize(self, nx, ny, nz):
        super().SetMeshSize(nx, ny, nz)
        self._my = np.zeros((nx, ny, nz))
        self._mz = np.zeros((nx, ny, nz))

    def SetMagnetization_X(self):
        return self._data

    def GetMagnetization_X(self):
        return self._data

    def SetMagnetization_Y(self):
        return self._my

    def GetMagnetization_Y(self):
        return self._my

    def SetMagnetization_Z(self):
        return self._mz

    def GetMagnetization_Z(self):
        return self._mz

    def GetModelParameters(self):
        return np.concatenate([self._data.reshape(-1), self._my.reshape(-1),
                               self._mz.reshape(-1)])

    def WriteNetCDF(self, filename):
        """Magnetics/ThreeDMagnetizationModel.cpp:28-103: Mx, My, Mz (A/m)."""
        from . import netcdf
        netcdf.WriteMagnetizationModel(self, filename)

    def ReadNetCDF(self, filename):
        """Magnetics/ThreeDMagnetizationModel.cpp:105-145."""
        from . import netcdf
        netcdf.ReadMagnetizationModel(self, filename)

    def GetNModelParm(self):
        return 3 * self._data.size


class GeneralData:
    """Measurement positions, data and errors (DataBase/GeneralData.h)."""

    def __init__(self):
        self._x, self._y, self._z = [], [], []
        self._data, self._err = np.zeros(0), np.zeros(0)

    def SetDataAndErrors(self, D, E):
        """GeneralData.h:117-126: data and errors of equal length."""
        D, E = np.array(D, dtype=float), np.array(E, dtype=float)
        if D.size != E.size:
            raise FatalException("Data and Errors do not have the same size !")
        self._data, self._err = D, E

    def SetErrors(self, E):
        E = np.array(E, dtype=float)
        if E.size != self._data.size:
            raise FatalException("Data and Errors do not have the same size !")
        self._err = E

    def GetData(self):
        return self._data

    def GetErrors(self):
        return self._err

    def AddMeasurementPoint(self, x, y, z):
        self._x.append(float(x))
        self._y.append(float(y))
        self._z.append(float(z))

    def GetMeasPosX(self):
        return np.array(self._x)

    def GetMeasPosY(self):
        return np.array(self._y)

    def GetMeasPosZ(self):
        return np.array(self._z)

    def CopyMeasurementConfiguration(self, other):
        self._x, self._y, self._z = list(other._x), list(other._y), list(other._z)

    def ClearMeasurementPoints(self):
        self._x, self._y, self._z = [], [], []


    # ReadNetCDF / WriteNetCDF of the data classes (Gravity/ScalarGravityData.cpp:16-38
    # and the like): positions, data and errors through the format's functions
    _read = _save = None

    def ReadNetCDF(self, filename):
        from . import netcdf
        Data, PosX, PosY, PosZ, Error = getattr(netcdf, self._read)(filename)
        self.ClearMeasurementPoints()
        for x, y, z in zip(PosX, PosY, PosZ):
            self.AddMeasurementPoint(x, y, z)
        self.SetDataAndErrors(Data, Error if len(Error) == len(Data) else np.zeros(len(Data)))

    def WriteNetCDF(self, filename):
        from . import netcdf
        getattr(netcdf, self._save)(filename, self.GetData(), self.GetMeasPosX(),
                                    self.GetMeasPosY(), self.GetMeasPosZ(), self.GetErrors())


class ScalarGravityData(GeneralData):
    ModelType = ThreeDGravityModel
    _read, _save = "ReadScalarGravityMeasurements", "SaveScalarGravityMeasurements"


class TensorGravityData(GeneralData):
    ModelType = ThreeDGravityModel
    _read, _save = "ReadTensorGravityMeasurements", "SaveTensorGravityMeasurements"


class TotalFieldMagneticData(GeneralData):
    ModelType = ThreeDSusceptibilityModel
    _read, _save = "ReadTotalFieldMagneticMeasurements", "SaveTotalFieldMagneticMeasurements"


class ThreeComponentMagneticData(GeneralData):
    ModelType = ThreeDMagnetizationModel
    _read, _save = "ReadMagneticComponentMeasurements", "SaveMagneticComponentMeasurements"


# ---------------------------------------------------------------------------
# Transforms (host-side Transform / Derivative used by the cached calculator
# path, exactly as VectorTransform is used there)
class VectorTransform:
    code = capi.T_NONE
    inclination = 0.0
    declination = 0.0


class FTGInvariant(VectorTransform):
    """I2 invariant, Gravity/GravityTransforms.h:25-100."""
    code = capi.T_FTG_INVARIANT

    def GetInputSize(self):
        return 9

    def GetOutputSize(self):
        return 1

    def Transform(self, d):
        return np.array([d[0] * d[4] + d[4] * d[8] + d[0] * d[8] - d[3] * d[1] - d[7] * d[5]
                         - d[2] * d[6]])

    def Derivative(self, d):
        return np.array([[d[4] + d[8], -d[3], -d[6], -d[1], d[0] + d[8], -d[7], -d[2], -d[5],
                          d[0] + d[4]]])


class TotalField(VectorTransform):
    """|B|, Magnetics/MagneticTransforms.h:19-82."""
    code = capi.T_TOTAL_FIELD

    def GetInputSize(self):
        return 3

    def GetOutputSize(self):
        return 1

    def Transform(self, d):
        return np.array([np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])])

    def Derivative(self, d):
        t = np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
        return np.array([[d[0] / t, d[1] / t, d[2] / t]])


class TotalFieldAnomaly(VectorTransform):
    """Projection on the inducing field, Magnetics/MagneticTransforms.h:84-156."""
    code = capi.T_TFA

    def __init__(self, inc=0.0, dec=0.0):
        self.inclination = float(inc)
        self.declination = float(dec)
        self._b = np.array([np.cos(inc) * np.cos(dec), np.cos(inc) * np.sin(dec), np.sin(inc)])

    def GetInputSize(self):
        return 3

    def GetOutputSize(self):
        return 1

    def Transform(self, d):
        return np.array([self._b[0] * d[0] + self._b[1] * d[1] + self._b[2] * d[2]])

    def Derivative(self, d):
        return self._b.reshape(1, 3).copy()


def ApplyTransform(data, transform):
    """Global/VectorTransform.h:158-181."""
    step, nout = transform.GetInputSize(), transform.GetOutputSize()
    if data.size % step:
        raise FatalException("Transformation size needs to be integer multiple of input "
                             "data size")
    out = np.empty(data.size // step * nout)
    for i in range(0, data.size, step):
        out[i // step * nout:(i // step + 1) * nout] = transform.Transform(data[i:i + step])
    return out


# ---------------------------------------------------------------------------
# Implementations
class GB300GravMagImplementation:
    """GB300 counterpart of jif3D::ThreeDGravMagImplementation.

    Calculate and LQDerivative are overridden as whole-survey calls into the
    C ABI; the per-station obligations of the base class (fill the calculator's
    current sensitivities when they are large enough, call
    HandleSensitivities(i) in station order, store raw sensitivities) are kept.
    """

    KIND = None

    def __init__(self, device=0):
        self._device = device
        self._ctx = None
        self._key = None
        self.Transform = None

    def _context(self):
        if self._ctx is None:
            self._ctx = capi.Context(self._device)
        return self._ctx

    def RawDataPerMeasurement(self):
        return {capi.SCALAR: 1, capi.TENSOR: 9, capi.MAGNETIC: 3, capi.JOINT: 10,
                capi.MAG_GRADIENT: 1, capi.MAGNETIZATION: 3}[self.KIND]

    def SetDataTransform(self, transform):
        self.Transform = transform

    def GetDataPerMeasurement(self):
        return self.Transform.GetOutputSize() if self.Transform else self.RawDataPerMeasurement()

    def _kind_args(self):
        return (self.KIND, 0.0, 0.0, 0.0)

    def _prepare(self, Model, Data):
        ctx = self._context()
        key = (self.GetDataPerMeasurement(), self._kind_args(),
               self.Transform.code if self.Transform else 0,
               getattr(self.Transform, "inclination", 0.0),
               getattr(self.Transform, "declination", 0.0),
               Model.GetXOrigin(), Model.GetYOrigin(), Model.GetZOrigin(),
               Model.GetXCellSizes().tobytes(), Model.GetYCellSizes().tobytes(),
               Model.GetZCellSizes().tobytes(), Model.GetXCoordinates().tobytes(),
               Model.GetYCoordinates().tobytes(), Model.GetZCoordinates().tobytes(),
               Model.GetBackgroundThicknesses().tobytes(),
               Data.GetMeasPosX().tobytes(), Data.GetMeasPosY().tobytes(),
               Data.GetMeasPosZ().tobytes())
        if key != self._key:
            ctx.set_mesh(Model.GetXCoordinates(), Model.GetYCoordinates(),
                         Model.GetZCoordinates(), Model.GetXCellSizes(), Model.GetYCellSizes(),
                         Model.GetZCellSizes())
            ctx.set_background(Model.GetBackgroundThicknesses())
            ctx.set_stations(Data.GetMeasPosX(), Data.GetMeasPosY(), Data.GetMeasPosZ())
            ctx.set_kind(*self._kind_args())
            t = self.Transform
            ctx.set_transform(t.code if t else capi.T_NONE, getattr(t, "inclination", 0.0),
                              getattr(t, "declination", 0.0))
            self._key = key
        return ctx

    def Calculate(self, Model, Data, Calculator):
        """ThreeDGravMagImplementation::Calculate (ThreeDGravMagImplementation.h:116-168)."""
        ctx = self._prepare(Model, Data)
        model = Model.GetModelParameters()
        nmeas = Data.GetMeasPosX().size
        raw = self.RawDataPerMeasurement()
        cur = Calculator.SetCurrentSensitivities()
        wants_rows = cur.shape[0] >= raw and cur.shape[1] >= Model.GetNModelParm() \
            and Model.GetNModelElements() > 0
        if not wants_rows:
            return ctx.forward(model)
        data, J = ctx.forward_sens(model)
        ncol = Model.GetNModelParm()
        for i in range(nmeas):
            cur[:raw, :ncol] = J[i * raw:(i + 1) * raw]
            Calculator.HandleSensitivities(i)
        return data

    def LQDerivative(self, Model, Data, Misfit):
        """Matrix-free 2 J^T (T' misfit) (ThreeDGravMagImplementation.h:177-231)."""
        ctx = self._prepare(Model, Data)
        misfit = np.asarray(Misfit, dtype=float)
        if misfit.size != Data.GetMeasPosX().size * self.GetDataPerMeasurement():
            raise FatalException("Misfit size does not match the number of data")
        return ctx.lqderivative(Model.GetModelParameters(), misfit)


class ScalarGB300GravityImp(GB300GravMagImplementation):
    """Replaces ScalarOMPGravityImp / ScalarCudaGravityImp."""
    KIND = capi.SCALAR


class TensorGB300GravityImp(GB300GravMagImplementation):
    """Replaces TensorOMPGravityImp / TensorCudaGravityImp."""
    KIND = capi.TENSOR


class JointGB300GravityImp(GB300GravMagImplementation):
    """g_z and the 9 FTG values of each station in one pass (10 raw values)."""
    KIND = capi.JOINT


class GB300MagneticSusceptibilityImp(GB300GravMagImplementation):
    """Replaces OMPMagneticSusceptibilityImp / CudaMagneticSusceptibilityImp.
    Inclination and declination in radians, field strength in nT."""
    KIND = capi.MAGNETIC

    def __init__(self, Inc=0.0, Dec=0.0, Fs=1.0, device=0):
        super().__init__(device)
        self.Inclination, self.Declination, self.FieldStrength = float(Inc), float(Dec), float(Fs)

    def _kind_args(self):
        return (self.KIND, self.Inclination, self.Declination, self.FieldStrength)


class GB300MagneticGradImp(GB300MagneticSusceptibilityImp):
    """Replaces OMPMagneticGradImp (Magnetics/OMPMagneticGradImp.h:20-64): one
    datum per station, the vertical gradient Bz(z) - Bz(z + 1 m); background
    layers do not respond."""
    KIND = capi.MAG_GRADIENT

    def __init__(self, Inc=0.0, Dec=0.0, Fs=1.0, device=0):
        super().__init__(Inc, Dec, Fs, device)


class GB300MagnetizationImp(GB300GravMagImplementation):
    """Replaces OMPMagnetizationImp (Magnetics/OMPMagnetizationImp.h:20-50):
    Bx, By, Bz of a ThreeDMagnetizationModel (no inducing-field parameters)."""
    KIND = capi.MAGNETIZATION


# ---------------------------------------------------------------------------
# Calculators
class ThreeDGravMagCalculator:
    """GravMag/ThreeDGravMagCalculator.h:47-173."""

    def __init__(self, imp):
        self.Imp = imp
        self.Transform = None
        self._current = np.zeros((0, 0))

    def SetDataTransform(self, transform):
        self.Transform = transform
        self.Imp.SetDataTransform(transform)

    def GetDataPerMeasurement(self):
        return self.Imp.GetDataPerMeasurement()

    def SetCurrentSensitivities(self):
        return self._current

    def _resize_current(self, r, c):
        self._current = np.zeros((r, c))

    def CheckModelConsistency(self, Model):
        shp = Model.GetData().shape
        if shp[0] != Model.GetXCellSizes().size:
            raise FatalException("Model x-dimension does not match size for specification of "
                                 "cell sizes. ")
        if shp[1] != Model.GetYCellSizes().size:
            raise FatalException("Model y-dimension does not match size for specification of "
                                 "cell sizes. ")
        if shp[2] != Model.GetZCellSizes().size:
            raise FatalException("Model x-dimension does not match size for specification of "
                                 "cell sizes. ")

    def Calculate(self, Model, Data):
        self.CheckModelConsistency(Model)
        return self.Imp.Calculate(Model, Data, self)

    def LQDerivative(self, Model, Data, Misfit):
        self.CheckModelConsistency(Model)
        return self.Imp.LQDerivative(Model, Data, Misfit)

    def HandleSensitivities(self, measindex):
        raise NotImplementedError


class MinMemGravMagCalculator(ThreeDGravMagCalculator):
    """GravMag/MinMemGravMagCalculator.h: no sensitivities kept."""

    def Calculate(self, Model, Data):
        self._resize_current(0, 0)
        return super().Calculate(Model, Data)

    def HandleSensitivities(self, measindex):
        pass


class _GridBackgroundModelCache:
    """ModelBase/GridBackgroundModelCache.h: cell sizes + background values and
    thicknesses (station positions are not part of the key, as in the reference)."""

    def __init__(self):
        self._old = None

    def HasChanged(self, Model):
        new = (Model.GetXCellSizes().tobytes(), Model.GetYCellSizes().tobytes(),
               Model.GetZCellSizes().tobytes(), Model.GetBackgroundValues().tobytes(),
               Model.GetBackgroundThicknesses().tobytes())
        changed = new != self._old
        self._old = new
        return changed


class CachedGravMagCalculator(ThreeDGravMagCalculator):
    """GravMag/CachedGravMagCalculator.h:28-143."""

    def __init__(self, imp):
        super().__init__(imp)
        self._have_cache = False
        self._cache = _GridBackgroundModelCache()

    def InvalidateCache(self):
        self._have_cache = False

    def Calculate(self, Model, Data):
        self.CheckModelConsistency(Model)
        changed = self._cache.HasChanged(Model)
        if self._have_cache and not changed:
            return self.CalculateCachedResult(Model, Data)
        self._resize_current(self.Imp.RawDataPerMeasurement(), Model.GetNModelParm())
        result = self.CalculateNewModel(Model, Data)
        self._have_cache = True
        return result

    def LQDerivative(self, Model, Data, Misfit):
        self.CheckModelConsistency(Model)
        changed = self._cache.HasChanged(Model)
        if self._have_cache and not changed:
            return self.CachedLQDerivative(Model, Data, Misfit)
        self._resize_current(self.Imp.GetDataPerMeasurement(), Model.GetNModelParm())
        return ThreeDGravMagCalculator.LQDerivative(self, Model, Data, Misfit)


class FullSensitivityGravMagCalculator(CachedGravMagCalculator):
    """GravMag/FullSensitivityGravMagCalculator.h:33-221 (J kept in host memory)."""

    def __init__(self, imp):
        super().__init__(imp)
        self.Sensitivities = np.zeros((0, 0))

    def GetSensitivities(self):
        return self.Sensitivities

    def SetSensitivities(self):
        self.InvalidateCache()
        return self.Sensitivities

    def HandleSensitivities(self, measindex):
        raw = self.Imp.RawDataPerMeasurement()
        self.Sensitivities[measindex * raw:(measindex + 1) * raw, :] = \
            self._current[:, :self.Sensitivities.shape[1]]

    def CalculateNewModel(self, Model, Data):
        nmeas = Data.GetMeasPosX().size
        self.Sensitivities = np.zeros((nmeas * self.Imp.RawDataPerMeasurement(),
                                       Model.GetNModelParm()))
        return self.Imp.Calculate(Model, Data, self)

    def CalculateRawData(self, Model, Data):
        nrow = Data.GetMeasPosX().size * self.Imp.RawDataPerMeasurement()
        if self.Sensitivities.shape != (nrow, Model.GetNModelParm()):
            raise FatalException("Size of sensitivity matrix does not match model "
                                 "configuration ! ")
        return self.Sensitivities @ Model.GetModelParameters()

    def CalculateCachedResult(self, Model, Data):
        if self.Transform:
            return ApplyTransform(self.CalculateRawData(Model, Data), self.Transform)
        return self.CalculateRawData(Model, Data)

    def CachedLQDerivative(self, Model, Data, Misfit):
        result = self.CalculateRawData(Model, Data)
        misfit = np.asarray(Misfit, dtype=float)
        if not self.Transform:
            processed = misfit
        else:
            nin, nout = self.Transform.GetInputSize(), self.Transform.GetOutputSize()
            processed = np.empty(misfit.size // nout * nin)
            for i in range(0, misfit.size, nout):
                o = i // nout * nin
                processed[o:o + nin] = self.Transform.Derivative(result[o:o + nin]).T @ \
                    misfit[i:i + nout]
        return 2.0 * (self.Sensitivities.T @ processed)


class DeviceSensitivityGravMagCalculator(ThreeDGravMagCalculator):
    """GPU twin of FullSensitivity / CachedGravMagCalculator
    (GravMag/FullSensitivityGravMagCalculator.h:33-221,
    GravMag/CachedGravMagCalculator.h:28-143): the first call on a geometry
    computes the data in FP64 and builds the sensitivity matrix in HBM
    (j3g_build_sensitivity); later calls on the same geometry run the stored
    products on the device (FP32 streaming or fp16 hi/lo tensor-core,
    relative error <= 1e-6) instead of recomputing box terms.

    The cache key is the full geometry -- cell sizes, origin, background
    thicknesses, the station positions (which the reference's
    GridBackgroundModelCache omits) and the kind / transform -- and not the
    model values, which J does not depend on.
    """

    def __init__(self, imp, storage=capi.STORE_FP32):
        super().__init__(imp)
        self.storage = storage
        self._key = None

    def InvalidateCache(self):
        self._key = None

    def _geometry_key(self, Model, Data):
        t = self.Imp.Transform
        return (self.Imp._kind_args(), t.code if t else 0, getattr(t, "inclination", 0.0),
                getattr(t, "declination", 0.0),
                Model.GetXOrigin(), Model.GetYOrigin(), Model.GetZOrigin(),
                Model.GetXCellSizes().tobytes(), Model.GetYCellSizes().tobytes(),
                Model.GetZCellSizes().tobytes(), Model.GetBackgroundThicknesses().tobytes(),
                Data.GetMeasPosX().tobytes(), Data.GetMeasPosY().tobytes(),
                Data.GetMeasPosZ().tobytes())

    def _cached(self, Model, Data):
        """(context, True) on a cache hit, else (context, the new key)."""
        key = self._geometry_key(Model, Data)
        ctx = self.Imp._prepare(Model, Data)
        if key == self._key and ctx.sensitivity_info()["storage"] == self.storage:
            return ctx, True
        return ctx, key

    def Calculate(self, Model, Data):
        self.CheckModelConsistency(Model)
        ctx, hit = self._cached(Model, Data)
        model = Model.GetModelParameters()
        if hit is True:
            return ctx.batched_forward(model[None, :])[0]
        data = ctx.forward(model)  # FP64, as the first call of the reference
        ctx.build_sensitivity(self.storage)
        self._key = hit
        return data

    def LQDerivative(self, Model, Data, Misfit):
        self.CheckModelConsistency(Model)
        ctx, hit = self._cached(Model, Data)
        model = Model.GetModelParameters()
        misfit = np.asarray(Misfit, dtype=float)
        if hit is True:
            return ctx.batched_lqderivative(model[None, :], misfit[None, :])[0]
        return ctx.lqderivative(model, misfit)

    def HandleSensitivities(self, measindex):
        pass
