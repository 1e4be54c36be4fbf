"""Host-side mirror of the Teton routines that drive the sweep path.

Teton's host side is Fortran; no Fortran compiler exists on the machines this
project builds on, so the routines above the C-ABI are mirrored here with the
reference's names and argument meaning, calling the CUDA library through
umt_gb300.capi.  A Fortran caller binds the same C entry points directly
through an ISO_C_BINDING interface block.

    radtr            aux/radtr.F90:12-71           one radiation cycle
    initializeSets   control/initializeSets.F90:12 tau, Sigt, PsiB, PhiTotal, EnergyRadBOC
    rtmainsn         rt/rtmainsn.F90:10-287        TemperatureIteration + savePsi sweep
    LinearSolver     rt/LinearSolver.F90:10-124    one sweep (GTA compiled out of the mini-app)
    ControlSweep     rt/ControlSweep.F90:15-81     SetSweep + getPhiTotal, on the GPU
    ConvergenceTest  rt/ConvergenceTest.F90:10-219 zone energy-density and temperature errors
    rtedit           aux/rtedit.F90:8-327          EnergyRadiation, EnergyCheck (+ BoundaryEdit)

Errors from the library raise capi.UmtError (the reference aborts instead).
"""
from __future__ import annotations

import numpy as np

from . import capi
from .problems import Problem, SPEED_LIGHT


class Teton:
    def __init__(self, prob: Problem, precision: int = capi.UMT_FP64, lib: capi.Library | None = None):
        self.prob = prob
        self.precision = precision
        self.lib = lib or capi.Library()
        m = prob.mesh
        flags = 1 if precision == capi.UMT_FP64 else 2
        self.lib.init(m, prob.omega, prob.weight, prob.ngr, flags=flags)
        self.A, self.G = len(prob.weight), prob.ngr
        self.PsiB = np.zeros((self.A, m.nbelem, self.G))
        self.STotal = np.zeros((m.ncornr, self.G))     # mini-app: never assembled
        self.lib.set_psi(prob.psi0, self.PsiB)
        self.volume = None
        self.edits = []
        self.EnergyRadBOC = None
        self.PhiTotal = None
        self.maxTempIters = 50                         # default_iter_controls_mod.F90:10-22
        self.epsEnergyDensity = 1.0e-5
        self.epsTemperature = 1.0e-5

    # -- initializeSets ------------------------------------------------------
    def initializeSets(self):
        p = self.prob
        self.lib.set_materials(p.sigt, p.sigs, p.tau)
        if self.volume is None:
            self.volume = self.lib.geometry()[2]
        if self.PhiTotal is None:      # initPhiTotal: PhiTotal = sum_a w_a Psi_a
            self.PhiTotal = np.einsum("a,acg->cg", p.weight, p.psi0)
        m = p.mesh
        # initializeZones: radEnergy per zone and EnergyRadBOC
        vphi = self.volume * self.PhiTotal.sum(1)
        self.radEnergy = np.bincount(m.cToZone, weights=vphi, minlength=m.nzones)
        self.volumeZone = np.bincount(m.cToZone, weights=self.volume, minlength=m.nzones)
        self.EnergyRadBOC = self.radEnergy.sum() / SPEED_LIGHT
        self.EnergyDensityOld = self.radEnergy / self.volumeZone

    # -- ControlSweep ----------------------------------------------------------
    def ControlSweep(self, savePsi: bool):
        self.PhiTotal = self.lib.sweep(self.STotal, savePsi=savePsi, PsiB=self.PsiB, precision=self.precision)
        return self.PhiTotal

    def LinearSolver(self, savePsi: bool = False):
        return self.ControlSweep(savePsi)

    # -- ConvergenceTest ---------------------------------------------------------
    def ConvergenceTest(self):
        """Relative change of the zone energy density above 1e-6 of its max
        (ConvergenceTest.F90:128-160).  The mini-app updates radEnergy only
        at the start of a cycle, and the material temperature never changes,
        so both errors are zero from the second iteration on."""
        ed = self.radEnergy / self.volumeZone
        thr = 1.0e-6 * ed.max()
        sel = ed > thr
        err = float(np.max(np.abs((ed[sel] - self.EnergyDensityOld[sel]) / ed[sel]))) if sel.any() else 0.0
        self.EnergyDensityOld = ed
        return err, 0.0

    # -- rtmainsn ----------------------------------------------------------------
    def rtmainsn(self):
        tempIter = 0
        while True:
            tempIter += 1
            self.LinearSolver(False)
            edErr, tErr = self.ConvergenceTest()
            if tempIter >= self.maxTempIters:
                break
            if tempIter > 1 and tErr < self.epsTemperature and edErr < self.epsEnergyDensity:
                break
        self.ControlSweep(True)
        return tempIter

    # -- rtedit --------------------------------------------------------------------
    def rtedit(self):
        p = self.prob
        t = self.lib.tally(p.siga, SPEED_LIGHT, precision=self.precision)
        dErad = t["EnergyRadiation"] - self.EnergyRadBOC
        check = p.dt * (t["PowerIncident"] - t["PowerEscape"]) - dErad
        closed = p.dt * (t["PowerIncident"] - t["PowerEscape"] - t["PowerAbsorbed"]) - dErad
        e = dict(EnergyRadiation=t["EnergyRadiation"], PowerEscape=t["PowerEscape"],
                 PowerIncident=t["PowerIncident"], PowerAbsorbed=t["PowerAbsorbed"],
                 EnergyCheck=check, EnergyCheckClosed=closed, EnergyRadBOC=self.EnergyRadBOC)
        self.edits.append(e)
        return e

    # -- radtr -----------------------------------------------------------------------
    def radtr(self):
        """One radiation cycle: initializeSets, rtmainsn, rtedit."""
        self.initializeSets()
        iters = self.rtmainsn()
        e = self.rtedit()
        e["tempIters"] = iters
        return e
