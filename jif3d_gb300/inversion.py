"""The inversion-side callers of the prism path: model refinement and the
least-squares objective, mirroring jif3D's classes of the same names.

* ``ModelRefiner`` -- ModelBase/ModelRefiner.h:33-128: refined axes on the
  host (RefineOneAxis), projection of cell values and combination of
  gradients on the GPU (bit-identical to the reference's walk and sums).
* ``ThreeDModelObjective`` -- Inversion/ThreeDModelObjective.h with the
  CalcMisfit / CalcGradient of Inversion/ObjectiveFunction.h:160-229: the
  inversion model lives on a coarse grid; with a fine model geometry the
  forward and the gradient run on the refined grid and the gradient is
  combined back onto the coarse cells.

Magnetisation models: the three blocks are refined alike.  The reference's
objective cannot refine them (its MagnetizationExtraParameterSetter checks the
extra parameters against the fine grid, Magnetics/ThreeDMagnetizationModel.h:
135-152, and throws); here the y and z blocks are projected and combined like
the x block.
"""
from __future__ import annotations

import copy

import numpy as np

from . import capi
from .gravmag import FatalException, ThreeDMagnetizationModel


class ModelRefiner:
    """jif3D::ModelRefiner with the cell passes on the GPU (one context per
    refiner, its mesh the refined grid and its refinement the coarse grid)."""

    def __init__(self, device=0):
        self._device = device
        self._refs = [np.zeros(0), np.zeros(0), np.zeros(0)]
        self._ctx = None
        self._fine_key = self._coarse_key = None

    def __deepcopy__(self, memo):
        other = ModelRefiner(self._device)
        other._refs = [r.copy() for r in self._refs]
        return other

    def SetXCoordinates(self, X):
        self._refs[0] = np.array(X, dtype=float)

    def SetYCoordinates(self, Y):
        self._refs[1] = np.array(Y, dtype=float)

    def SetZCoordinates(self, Z):
        self._refs[2] = np.array(Z, dtype=float)

    def RefineAxes(self, InputModel, RefinedModel):
        """ModelRefiner.cpp:74-90: refined cell sizes of all three axes (the
        refined model keeps its origin); the cell values are reallocated when
        the refined grid changes shape."""
        sizes = []
        for coords, cell, ref in ((InputModel.GetXCoordinates(), InputModel.GetXCellSizes(),
                                   self._refs[0]),
                                  (InputModel.GetYCoordinates(), InputModel.GetYCellSizes(),
                                   self._refs[1]),
                                  (InputModel.GetZCoordinates(), InputModel.GetZCellSizes(),
                                   self._refs[2])):
            try:
                sizes.append(capi.refine_axis(coords, cell, ref))
            except capi.J3GError as e:
                raise FatalException(str(e)) from e
        shape = tuple(v.size for v in sizes)
        if RefinedModel.GetData().shape != shape:
            RefinedModel.SetMeshSize(*shape)
        RefinedModel.SetXCellSizes(sizes[0])
        RefinedModel.SetYCellSizes(sizes[1])
        RefinedModel.SetZCellSizes(sizes[2])

    def _prepare(self, Coarse, Refined):
        if self._ctx is None:
            self._ctx = capi.Context(self._device)
        fk = tuple(np.asarray(v).tobytes() for v in (Refined.GetXCellSizes(),
                                                    Refined.GetYCellSizes(),
                                                    Refined.GetZCellSizes()))
        if fk != self._fine_key:
            self._ctx.set_mesh(Refined.GetXCoordinates(), Refined.GetYCoordinates(),
                               Refined.GetZCoordinates(), Refined.GetXCellSizes(),
                               Refined.GetYCellSizes(), Refined.GetZCellSizes())
            self._fine_key, self._coarse_key = fk, None
        ck = tuple(np.asarray(v).tobytes() for v in (Coarse.GetXCellSizes(),
                                                    Coarse.GetYCellSizes(),
                                                    Coarse.GetZCellSizes()))
        if ck != self._coarse_key:
            self._ctx.set_refinement(Coarse.GetXCellSizes(), Coarse.GetYCellSizes(),
                                     Coarse.GetZCellSizes())
            self._coarse_key = ck
        return self._ctx

    @staticmethod
    def _blocks(model, write=False):
        if isinstance(model, ThreeDMagnetizationModel):
            if write:
                return [model.SetMagnetization_X(), model.SetMagnetization_Y(),
                        model.SetMagnetization_Z()]
            return [model.GetMagnetization_X(), model.GetMagnetization_Y(),
                    model.GetMagnetization_Z()]
        return [model.SetData() if write else model.GetData()]

    def ProjectValues(self, InputModel, RefinedModel):
        """ModelRefiner.cpp:124-168 on the GPU (refined cells outside every
        coarse run keep their values)."""
        ctx = self._prepare(InputModel, RefinedModel)
        for src, dst in zip(self._blocks(InputModel), self._blocks(RefinedModel, write=True)):
            dst[...] = ctx.refine_project(src.reshape(-1), dst.reshape(-1)).reshape(dst.shape)

    def RefineModel(self, InputModel, RefinedModel):
        self.RefineAxes(InputModel, RefinedModel)
        self.ProjectValues(InputModel, RefinedModel)

    def CombineGradient(self, FineGradient, CoarseModel, RefinedModel):
        """ModelRefiner.cpp:170-218 on the GPU: the gradient of the coarse
        cells (one cell block per block of FineGradient)."""
        ctx = self._prepare(CoarseModel, RefinedModel)
        g = np.asarray(FineGradient, dtype=float)
        nfine = RefinedModel.GetData().size
        if g.size % nfine:
            raise FatalException("Fine gradient does not match the refined model")
        return np.concatenate([ctx.refine_combine(b) for b in g.reshape(-1, nfine)])


class ThreeDModelObjective:
    """Least-squares data objective of one calculator
    (Inversion/ThreeDModelObjective.h:36-329 with ObjectiveFunction.h:123-229):
    CalcMisfit returns chi^2 = sum (w (synthetic - observed))^2 with
    w = 1 / error, and keeps the weighted difference for CalcGradient."""

    def __init__(self, Calc, ethresh=0.0, device=0):
        self.Calculator = Calc
        self.CoarseModel = None
        self.FineModel = None
        self.wantrefinement = False
        self.Refiner = ModelRefiner(device)
        self.ObservedData = None
        self.ignorelargeerror = float(ethresh)
        self._invcov = None
        self.DataDifference = np.zeros(0)
        self.IndividualMisfits = np.zeros(0)
        self.SynthData = np.zeros(0)
        self.nEval = 0

    def clone(self):
        return copy.deepcopy(self)

    # -- setup (ThreeDModelObjective.h:143-201, ObjectiveFunction.h:123-131) -
    def SetDataTransform(self, DT):
        self.Calculator.SetDataTransform(DT)

    def SetObservedData(self, Data):
        if Data.GetData().size == 0:
            raise FatalException("Cannot have empty observations in objective function. ")
        self.ObservedData = Data
        self.SetDataError(Data.GetErrors())

    def SetDataError(self, Cov):
        self._invcov = 1.0 / np.asarray(Cov, dtype=float) ** 2

    def GetDataError(self):
        return 1.0 / np.sqrt(self._invcov)

    def SetCoarseModelGeometry(self, Model):
        if Model.GetData().size == 0:
            raise FatalException("Cannot have empty model in objective function. ")
        self.CoarseModel = copy.deepcopy(Model)

    def SetFineModelGeometry(self, Model):
        if Model.GetData().size == 0:
            raise FatalException("Cannot have empty model in objective function. ")
        self.FineModel = copy.deepcopy(Model)
        self.Refiner.SetXCoordinates(self.FineModel.GetXCoordinates())
        self.Refiner.SetYCoordinates(self.FineModel.GetYCoordinates())
        self.Refiner.SetZCoordinates(self.FineModel.GetZCoordinates())
        self.wantrefinement = True

    def GetObservedData(self):
        return self.ObservedData

    def GetSyntheticData(self):
        return self.SynthData

    def GetDataDifference(self):
        return self.DataDifference

    def GetIndividualMisfit(self):
        return self.IndividualMisfits

    def GetNEval(self):
        return self.nEval

    # -- the model vector into the model objects ------------------------------
    def _set_model(self, Model):
        m = np.asarray(Model, dtype=float)
        ngrid = self.CoarseModel.GetNModelElements()
        if m.size < ngrid:
            raise FatalException("Not enough inversion parameters to fill the grid !")
        self.CoarseModel.SetData()[...] = m[:ngrid].reshape(self.CoarseModel.GetData().shape)
        extra = m[ngrid:]
        if isinstance(self.CoarseModel, ThreeDMagnetizationModel):
            if extra.size != 2 * ngrid:
                raise FatalException(f"Extra magnetization values {extra.size} do not match "
                                     f"number of required values {2 * ngrid}")
            shape = self.CoarseModel.GetData().shape
            self.CoarseModel.SetMagnetization_Y()[...] = extra[:ngrid].reshape(shape)
            self.CoarseModel.SetMagnetization_Z()[...] = extra[ngrid:].reshape(shape)
        elif extra.size:
            # BackgroundDensitySetter / susceptibility setter: the extra
            # parameters are the background values, coarse and fine alike
            self.CoarseModel.SetBackgroundValues(extra)
            if self.wantrefinement:
                self.FineModel.SetBackgroundValues(extra)
        return m

    # -- ImplDataDifference (ThreeDModelObjective.h:228-275) ------------------
    def _data_difference(self, Model):
        self._set_model(Model)
        if self.wantrefinement:
            self.Refiner.RefineModel(self.CoarseModel, self.FineModel)
            self.SynthData = np.asarray(self.Calculator.Calculate(self.FineModel,
                                                                  self.ObservedData))
        else:
            self.SynthData = np.asarray(self.Calculator.Calculate(self.CoarseModel,
                                                                  self.ObservedData))
        obs = self.ObservedData.GetData()
        if self.SynthData.size != obs.size:
            raise FatalException(" ThreeDModelObjective: Forward calculation does not give "
                                 "same amount of data !")
        err = (self.GetDataError() if self._invcov is not None and self._invcov.size == obs.size
               else np.ones(obs.size))
        keep = np.abs(obs) > self.ignorelargeerror * err
        return np.where(keep, self.SynthData - obs, 0.0)

    # -- ObjectiveFunction::CalcMisfit / CalcGradient (:160-229) --------------
    def CalcMisfit(self, Model):
        diff = self._data_difference(Model)
        if self._invcov is None or self._invcov.size != diff.size:
            self._invcov = np.ones(diff.size)
        weighted = self._invcov * diff
        self.nEval += 1
        ind = diff * weighted
        chi = float(np.sum(ind))
        self.IndividualMisfits = np.sqrt(ind) * np.where(diff >= 0, 1.0, -1.0)
        self.DataDifference = weighted
        return chi

    def CalcGradient(self, Model):
        self.nEval += 1
        return self._gradient(Model, self.DataDifference)

    # -- ImplGradient (ThreeDModelObjective.h:279-327) -------------------------
    def _gradient(self, Model, Diff):
        m = np.asarray(Model, dtype=float)
        ngrid = self.CoarseModel.GetNModelElements()
        if m.size < ngrid:
            raise FatalException("Not enough inversion parameters to fill the grid !")
        if not np.array_equal(m[:ngrid], self.CoarseModel.GetData().reshape(-1)):
            raise FatalException("Gradient calculation needs identical model to forward !")
        if not self.wantrefinement:
            return np.asarray(self.Calculator.LQDerivative(self.CoarseModel, self.ObservedData,
                                                           Diff))
        self.Refiner.RefineModel(self.CoarseModel, self.FineModel)
        fine = np.asarray(self.Calculator.LQDerivative(self.FineModel, self.ObservedData, Diff))
        nfine = self.FineModel.GetNModelElements()
        nblock = 3 if isinstance(self.FineModel, ThreeDMagnetizationModel) else 1
        coarse = self.Refiner.CombineGradient(fine[:nblock * nfine], self.CoarseModel,
                                              self.FineModel)
        return np.concatenate([coarse, fine[nblock * nfine:]])
