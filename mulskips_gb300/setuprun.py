"""pymulskips-compatible front end: setup_mulskips_src, compile_mulskips and
run_mulskips with the signatures and behaviour of pymulskips/setuprun.py
(:15-553), driving the GB300 mulskips.e built in mulskips_gb300/_lib.

Differences, all on the build side: the box size is written to
mulskips_box.dat beside the executable instead of being compiled in
(pymulskips/setuprun.py:499-521), so setup_mulskips_src and
compile_mulskips do not recompile; they write make.log with the
"Compilation terminated" line the reference checks (:479-485).
"""
import math
import os
import shutil
import subprocess
import sys
import time

import numpy as np

DEFAULT_EXEC = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib")


class PlainSi:
    """Process object of the plain Si(001) model (what pymulskips' process
    classes provide to run_mulskips: listcry/listcryZ/listcov/listcovZ,
    indices(), KMC_sf, get_PtransE(), get_PtransD(), calibration_params)."""

    def __init__(self, T=1100.0, e_bond=0.6, nu=1e13, flux=0.5, sf=5.43 / 12):
        self.listcry, self.listcryZ = ["Si"], [14]
        self.listcov, self.listcovZ = [], []
        self.KMC_sf = sf
        self.T, self.e_bond, self.nu, self.flux = T, e_bond, nu, flux
        self.calibration_params = {"T": T, "E_bond": e_bond, "nu": nu, "F": flux}

    def indices(self):
        return [[1], [2], [3]]

    def get_PtransE(self):
        kb = 0.00008617330350
        e = np.zeros((1, 4))
        for n in (1, 2, 3):
            e[0, n] = self.nu * math.exp(-n * self.e_bond / (kb * self.T))
        return e

    def get_PtransD(self):
        return np.full((1, 3), self.flux)


def compile_mulskips(execpath=DEFAULT_EXEC):
    """The engine is prebuilt; record the build like the reference make does."""
    if not os.path.exists(os.path.join(execpath, "mulskips.e")):
        from .build import build_all
        build_all()
    with open(os.path.join(execpath, "make.log"), "w") as f:
        f.write("Compilation terminated\n")
    return True


def setup_mulskips_src(execpath=DEFAULT_EXEC, lenx=480, leny=480, lenz=480, socketport=None):
    """Set the box of mulskips.e (LenX=..., LenY=..., LenZ=... of the reference)."""
    for v in (lenx, leny):
        if v % 12:
            raise ValueError("LenX and LenY must be multiples of 12 (whole conventional cells)")
    with open(os.path.join(execpath, "mulskips_box.dat"), "w") as f:
        f.write(f"{lenx} {leny} {lenz}\n")
    return compile_mulskips(execpath)


def _write_startdat(path, Simulation, mp, PtransZig, ExitStrategy, OutMolMol, IterMax, TotTime, OutTime,
                    Seed_box, RunType, IDUM, SaveFinalState, restartfilename, SaveCoo, coofilename,
                    cadfilename=None, tempfilename=None, LenVac=None, LenNuc=None, initialState="homogeneous",
                    ProbTable=None):
    """start.dat in the layout of pymulskips/setuprun.py:292-389.  File names
    are taken relative to the caller's $PWD, as the reference writes them
    (:53, :301-306, :347-352).  For LA the rate lines carry the energetics
    (mp.get_energetics_evap / _depo, :224-235) and the LA block follows the
    file names (:303-317); SiGe crystals add the substrate Ge fraction
    mp.calibration_params['X0'][1] (:324-325); coverage species add the
    absorption and desorption lines (mp.get_PtransAbs / _PtransDes, :376-386);
    ST with a probability table names the table in place of the rates."""
    here = os.environ.get("PWD", os.getcwd())
    ncry, ncov = len(mp.listcry), len(mp.listcov)
    if Simulation == "LA":
        PtransE, PtransD = mp.get_energetics_evap(), mp.get_energetics_depo()
    else:
        PtransE, PtransD = mp.get_PtransE(), mp.get_PtransD()
    L = [f"{ncry} {ncov} ! NCrystal, NCov ",
         "{} ! Atomic numbers of crystal species ".format(" ".join(str(x) for x in mp.listcryZ))]
    if ncov:
        L.append("{} ! Atomic numbers of coverage species ".format(" ".join(str(x) for x in mp.listcovZ)))
    L.append(Simulation + " ! Initstat")
    if Simulation in ("IN", "SH"):
        L.append(os.path.join(here, cadfilename))
    elif Simulation == "LA":
        homoflag = {"homogeneous": "T", "inhomogeneous": "F"}.get(initialState)
        if homoflag is None:
            raise ValueError("initialState must be 'homogeneous' or 'inhomogeneous' for this main program")
        L += [os.path.join(here, cadfilename), os.path.join(here, tempfilename),
              "{} ! Melting temperature in Kelvin ".format(" ".join(str(x) for x in mp.Tm)),
              "{} ! prefactor P0 ".format(" ".join(str(x) for x in mp.calibration_params["P0"])),
              "{} ! errf param A ".format(" ".join(str(x) for x in mp.calibration_params["A"])),
              "{} ! errf param Tflex ".format(" ".join(str(x) for x in mp.calibration_params["Tflex"])),
              "{:.15f}".format(LenVac) + " ! LenVac -> Top air thickness in Ang",
              "{:.15f}".format(LenNuc) + " ! LenNuc -> Nucleus radius in Ang",
              homoflag + " ! Initial Nucleation State"]
    else:
        L.append(" ".join(str(s) for s in Seed_box) + " ! Len1 [Len2 Len3 Len4 Len5]")
    if 14 in mp.listcryZ and 32 in mp.listcryZ:
        L.append(str(mp.calibration_params["X0"][1]) + " ! Ge fraction in substrate ")
    L.append(f"{PtransZig} ! PtransZig")
    L.append("{:.15f}".format(mp.KMC_sf) + " ! KMC_sf -> KMC Super-Lattice parameter in Ang")
    L.append(ExitStrategy + " ! ExitStrategy")
    if ExitStrategy == "Iter":
        L += [f"{IterMax} ! IterMax -> Max number of iterations", f"{OutMolMol} ! OutMolMol -> output frequency"]
    else:
        L += ["{:.15f}".format(TotTime) + " ! TotTime", "{:.15f}".format(OutTime) + " ! OutTime"]
    L.append(RunType + " ! RunType. R = truly random . T = not so random (use this for regression tests). "
                       "C = continuation run")
    L.append(f"{IDUM} ! Random seed")
    L.append(("T" if SaveFinalState else "F") + " ! Save final state")
    if SaveFinalState:
        L.append(os.path.join(here, restartfilename))
    L.append(("T" if SaveCoo else "F") + " ! Save final Coor")
    if SaveCoo:
        L.append(os.path.join(here, coofilename))
    if Simulation == "ST" and ProbTable is not None:
        L.append(ProbTable)
    else:
        thr = 5e-12   # the minimum rate written by pymulskips (:360-386)
        for s in range(ncry):
            for ind in mp.indices():
                key = "".join(str(v) for v in ind)
                v = max(thr, float(PtransE[(s, *ind)]))
                L.append(f"{s + 1} {key} {v} ! PtransE[{s + 1},{ind}] ")
        for s in range(ncry):
            for ii in range(3):
                v = max(thr, float(PtransD[s, ii]))
                L.append(f"{s + 1} {ii + 1} {v} ! PtransD[{s + 1},{ii + 1}] ")
        if ncov:
            for name, P in (("PtransAbs", mp.get_PtransAbs()), ("PtransDes", mp.get_PtransDes())):
                for s in range(ncry, ncry + ncov):
                    for ii in range(3):
                        v = max(thr, float(P[s - ncry, ii]))
                        L.append(f"{s + 1} {ii + 1} {v} ! {name}[{s + 1},{ii + 1}] ")
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


def run_mulskips(execpath=DEFAULT_EXEC, runpath=None, Simulation=None, mp=None, PtransZig=1.0, ExitStrategy="Iter",
                 OutMolMol=None, IterMax=None, TotTime=None, OutTime=None, Seed_box=None, RunType="R",
                 IDUM=9117116, setup_only=False, cadfilename=None, tempfilename=None, LenVac=None, LenNuc=None,
                 initialState="homogeneous", LenSiGe=None, SaveCoo=False, coofilename=None, SaveFinalState=False,
                 restartfilename=None, useProbTable=False, ProbTable=None, **unused):
    """Write start.dat in runpath and run `execpath/mulskips.e | tee log.txt`
    there (pymulskips/setuprun.py:15-456).  Returns True unless the run
    stopped on "few MC particles" (None with setup_only)."""
    t0 = time.time()
    if runpath is None or (mp is None and Simulation is None):
        print("ERROR. Please define all the necessary input: [execpath, runpath, Simulation, mp]")
        sys.exit()
    Seed_box = Seed_box or [120, 120, 120]
    if os.path.abspath(runpath) != os.getcwd():
        shutil.rmtree(runpath, ignore_errors=True)
        os.makedirs(runpath)
    if mp != "custom":
        if ExitStrategy == "Iter":
            OutMolMol, IterMax = int(round(OutMolMol)), int(round(IterMax))
        _write_startdat(os.path.join(runpath, "start.dat"), Simulation, mp, PtransZig, ExitStrategy, OutMolMol,
                        IterMax, TotTime, OutTime, Seed_box, RunType, IDUM, SaveFinalState, restartfilename,
                        SaveCoo, coofilename, cadfilename, tempfilename, LenVac, LenNuc, initialState,
                        ProbTable if useProbTable else None)
    print("DONE MulSKIPs setup. ETA: {} sec".format(time.time() - t0))
    if setup_only:
        return None
    exe = os.path.join(execpath, "mulskips.e")
    p = subprocess.Popen(exe + " | tee log.txt", shell=True, stdout=subprocess.PIPE, cwd=runpath)
    for line in p.stdout:
        print("KMC:\t" + line.decode(errors="replace").rstrip())
    p.wait()
    with open(os.path.join(runpath, "log.txt")) as f:
        endok = "few MC particles: stop MC" not in f.read()
    print("DONE MulSKIPs run. ETA: {} sec".format(time.time() - t0))
    return endok
