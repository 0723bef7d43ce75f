"""Synthetic G4HepEmState tables in the reference JSON schema.

The reference builds its tables with G4HepEmInit from Geant4 models and the
G4LEDATA data files (G4HepEm/G4HepEmInit/src/*.cc).  Neither is available
here, so this module builds tables of the same layout and of realistic
magnitude from textbook formulas, and writes them in the exact schema read by
G4HepEmStateFromJson (G4HepEm/G4HepEmDataJsonIO/src/G4HepEmDataJsonIOImpl.hh:
125-981).  Any real G4HepEmInit JSON loads through the same path.

Layouts follow the reference data headers:
  * energy-loss tables  [R,R''] [dEdx,dEdx''] [S''] per couple
    (G4HepEm/G4HepEmData/include/G4HepEmElectronData.hh:104-155)
  * restricted macroscopic cross sections [M, E(max), max, logE0, 1/dlogE,
    (E, sigma, sigma'')*M], ionisation then brem (same file :183-234; grid
    size rule G4HepEmElectronTableBuilder.cc:258-261)
  * element selectors [K, Q, logE0, 1/dlogE, (E, P_0..P_{Q-2})*K]
    (same file :297-352; grid rule G4HepEmElectronTableBuilder.cc:671-684)
  * Seltzer-Berger sampling tables per Z (G4HepEmSBTableData.hh:8-42, packing
    G4HepEmElectronTableBuilder.cc:783-833), cumulative and rational
    interpolation parameters from the RITA method (Penelope 2008 manual, sec.
    1.2.4), cut cumulative by inverting that interpolation
    (G4HepEmSBBremTableBuilder.cc:143-171)
  * gamma macroscopic cross sections in three energy windows
    (G4HepEmGammaData.hh:20-44, G4HepEmGammaTableBuilder.cc:36-136) and the
    conversion element selector (G4HepEmGammaTableBuilder.cc:150-199)
  * material and element derived data (G4HepEmMaterialInit.cc:121-227).

Physics used for the values (all in Geant4 units: MeV, mm):
  restricted collision stopping power: Berger-Seltzer formula (ICRU 37);
  restricted Moller/Bhabha cross sections (Messel-Crawford); bremsstrahlung:
  complete-screening Bethe-Heitler with Tsai radiation logarithms; transport
  cross section: screened Rutherford with Moliere screening; Compton:
  Klein-Nishina; pair production: 7/9 X0^-1 with a threshold factor;
  photoabsorption: hydrogenic Z^4.5/E^3 with K and L edges in Sandia form.
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass, field

import numpy as np

# --- constants (CLHEP values, Geant4 units) ---------------------------------
MEC2 = 0.51099890999999997            # MeV
ALPHA = 7.2973525653052150e-03
R0 = 2.8179403262e-12                  # classic electron radius [mm]
HBARC = 197.32698045930e-12            # MeV mm
BOHR = 5.29177210903e-08               # mm
NAV = 6.02214076e23
GCM3 = 6.241509074460763e18            # g/cm3 in Geant4 internal units
LAMBDA_E = HBARC / MEC2                # reduced Compton wavelength [mm]
MIGDAL = 4.0 * math.pi * R0 * LAMBDA_E * LAMBDA_E

# Tsai radiation logarithms for Z < 5 (Tsai, Rev. Mod. Phys. 46 (1974) 815)
_FEL_LOW = [0.0, 5.31, 4.79, 4.74, 4.71]
_FINEL_LOW = [0.0, 6.144, 5.621, 5.805, 5.924]


def atomic_mass(z: int) -> float:
    """Approximate standard atomic weight [g/mol] for Z (exact for the named ones)."""
    known = {1: 1.008, 2: 4.0026, 6: 12.011, 7: 14.007, 8: 15.999, 13: 26.982,
             14: 28.085, 18: 39.948, 26: 55.845, 29: 63.546, 74: 183.84, 79: 196.97, 82: 207.2}
    if z in known:
        return known[z]
    return z * (2.0 + 0.0072 * z) + (0.0 if z < 3 else 0.5)


def coulomb_correction(z: float) -> float:
    """Davies-Bethe-Maximon Coulomb correction f_C(Z)."""
    a2 = (ALPHA * z) ** 2
    return a2 * (1.0 / (1.0 + a2) + 0.20206 - 0.0369 * a2 + 0.0083 * a2 * a2 - 0.002 * a2 ** 3)


def rad_logs(z: int):
    if z < 5:
        return _FEL_LOW[z], _FINEL_LOW[z]
    lz = math.log(z)
    return math.log(184.15) - lz / 3.0, math.log(1194.0) - 2.0 * lz / 3.0


def k_shell_energy(z: int) -> float:
    return 13.6e-6 * max(z - 1, 1) ** 2


def l_shell_energy(z: int) -> float:
    return 13.6e-6 * max(z - 7.4, 1.0) ** 2 / 4.0


def element_sandia(z: int):
    """Sandia-form photoabsorption per atom: intervals and 4 coefficients each.

    sigma(E) = a1/E + a2/E^2 + a3/E^3 + a4/E^4 [mm^2], hydrogenic Z^4.5/E^3
    shape with a K-edge jump of 5.5 and an L-edge jump of 4."""
    c = 4.2e-31 * z ** 4.5
    e_k, e_l = k_shell_energy(z), l_shell_energy(z)
    energies = [1.0e-5]
    coefs = [[0.0, 0.0, c / 22.0, 0.0]]
    if e_l > 1.0e-5:
        energies.append(e_l)
        coefs.append([0.0, 0.0, c / 5.5, 0.0])
    if e_k > max(e_l, 1.0e-5):
        energies.append(e_k)
        coefs.append([0.0, 0.0, c, 0.0])
    return energies, coefs


def sandia_eval(energies, coefs, e):
    iv = 0
    if e >= energies[0]:
        for i in range(len(energies) - 1, -1, -1):
            if e >= energies[i]:
                iv = i
                break
    a = coefs[iv]
    inv = 1.0 / e
    return inv * (a[0] + inv * (a[1] + inv * (a[2] + inv * a[3])))


@dataclass
class Material:
    name: str
    zs: list
    natoms_rel: list          # relative atom counts
    density: float            # g/cm3
    mean_exc: float | None = None   # eV; None -> Bragg additivity estimate
    # derived
    natoms: list = field(default_factory=list)   # per mm3

    def finish(self):
        molar = sum(n * atomic_mass(z) for z, n in zip(self.zs, self.natoms_rel))
        per_mm3 = self.density * NAV / molar / 1000.0
        self.natoms = [per_mm3 * n for n in self.natoms_rel]
        if self.mean_exc is None:
            num = sum(n * z * math.log(16.0 * z ** 0.9 if z > 1 else 19.2)
                      for z, n in zip(self.zs, self.natoms))
            den = sum(n * z for z, n in zip(self.zs, self.natoms))
            self.mean_exc = math.exp(num / den)
        return self

    @property
    def n_el(self):
        return sum(n * z for z, n in zip(self.zs, self.natoms))

    @property
    def zeff(self):
        return sum(n * z * z for z, n in zip(self.zs, self.natoms)) / self.n_el

    @property
    def radlen(self):
        s = 0.0
        for z, n in zip(self.zs, self.natoms):
            fel, finel = rad_logs(z)
            s += n * 4.0 * ALPHA * R0 * R0 * (z * z * (fel - coulomb_correction(z)) + z * finel)
        return 1.0 / s


NAMED = {
    "G4_PbWO4": lambda: Material("G4_PbWO4", [82, 74, 8], [1, 1, 4], 8.28, 600.7).finish(),
    "G4_lAr": lambda: Material("G4_lAr", [18], [1], 1.396, 188.0).finish(),
    "G4_Pb": lambda: Material("G4_Pb", [82], [1], 11.35, 823.0).finish(),
}


# --- cross sections and stopping powers ------------------------------------
def dedx_collision(mat: Material, t: float, cut: float, positron: bool) -> float:
    """Restricted collision stopping power [MeV/mm], Berger-Seltzer form."""
    tlow = 1.0e-2
    if t < tlow:
        return dedx_collision(mat, tlow, cut, positron) * (t / tlow) ** -0.35
    tau = t / MEC2
    gam = tau + 1.0
    g2 = gam * gam
    bg2 = tau * (tau + 2.0)
    b2 = bg2 / g2
    eexc = mat.mean_exc * 1e-6 / MEC2
    tmax = t if positron else 0.5 * t
    d = min(cut, tmax) / MEC2
    if positron:
        d2 = d * d * 0.5
        d3 = d2 * d / 1.5
        d4 = d3 * d * 0.75
        y = 1.0 / (1.0 + gam)
        core = (math.log(2.0 * (tau + 2.0) / (eexc * eexc)) + math.log(tau * d)
                - b2 * (tau + 2.0 * d - y * (3.0 * d2 + y * (d - d3 + y * (d2 - tau * d3 + d4)))) / tau)
    else:
        core = (math.log(2.0 * (tau + 2.0) / (eexc * eexc)) - 1.0 - b2 + math.log((tau - d) * d)
                + tau / (tau - d) + (0.5 * d * d + (2.0 * tau + 1.0) * math.log(1.0 - d / tau)) / g2)
    # density effect (Sternheimer-like, single parameter)
    hw = 28.816e-6 * math.sqrt(mat.n_el * 1000.0 / NAV)        # plasma energy [MeV]
    cbar = 1.0 + 2.0 * math.log(mat.mean_exc * 1e-6 / hw)
    x = math.log10(math.sqrt(bg2))
    delta = max(0.0, 2.0 * math.log(10.0) * x - cbar)
    val = 2.0 * math.pi * R0 * R0 * MEC2 * mat.n_el / b2 * (core - delta)
    return max(val, 1e-12)


def brem_sum_factor(mat: Material) -> float:
    s = 0.0
    for z, n in zip(mat.zs, mat.natoms):
        fel, _ = rad_logs(z)
        s += n * 4.0 * ALPHA * R0 * R0 * z * (z + 1.0) * (fel - coulomb_correction(z) / 3.0)
    return s


def dedx_brem(mat: Material, t: float, kc: float) -> float:
    et = t + MEC2
    km = min(kc, t)
    return brem_sum_factor(mat) * (4.0 / 3.0 * km - 2.0 / 3.0 * km * km / et + km ** 3 / (3.0 * et * et))


def xs_brem(mat: Material, t: float, kc: float) -> float:
    if t <= kc:
        return 0.0
    et = t + MEC2
    return brem_sum_factor(mat) * (4.0 / 3.0 * math.log(t / kc) - 4.0 / 3.0 * (t - kc) / et
                                   + (t * t - kc * kc) / (2.0 * et * et))


def xs_ioni(mat: Material, t: float, cut: float, positron: bool) -> float:
    """Restricted Moller (e-) or Bhabha (e+) macroscopic cross section [1/mm]."""
    tmax = t if positron else 0.5 * t
    if cut >= tmax:
        return 0.0
    xmin, xmax = cut / t, tmax / t
    gam = t / MEC2 + 1.0
    g2 = gam * gam
    b2 = 1.0 - 1.0 / g2
    if not positron:
        gg = (2.0 * gam - 1.0) / g2
        cross = ((xmax - xmin) * (1.0 - gg + 1.0 / (xmin * xmax) + 1.0 / ((1.0 - xmin) * (1.0 - xmax)))
                 - gg * math.log(xmax * (1.0 - xmin) / (xmin * (1.0 - xmax)))) / b2
    else:
        y = 1.0 / (1.0 + gam)
        y2 = y * y
        y12 = 1.0 - 2.0 * y
        b1 = 2.0 - y2
        bb2 = y12 * (3.0 + y2)
        y122 = y12 * y12
        b4 = y122 * y12
        b3 = b4 + y122
        cross = ((xmax - xmin) * (1.0 / (b2 * xmin * xmax) + bb2 - 0.5 * b3 * (xmin + xmax)
                                  + b4 * (xmin * xmin + xmin * xmax + xmax * xmax) / 3.0)
                 - b1 * math.log(xmax / xmin))
    return max(0.0, cross * 2.0 * math.pi * R0 * R0 * MEC2 / t * mat.n_el)


def xs_tr1(mat: Material, t: float) -> float:
    """First transport macroscopic cross section, screened Rutherford [1/mm]."""
    pc2 = t * (t + 2.0 * MEC2)
    b2 = pc2 / (t + MEC2) ** 2
    s = 0.0
    for z, n in zip(mat.zs, mat.natoms):
        a_tf = 0.885 * BOHR * z ** (-1.0 / 3.0)
        scr = (HBARC / (2.0 * math.sqrt(pc2) * a_tf)) ** 2 * (1.13 + 3.76 * (ALPHA * z) ** 2 / b2)
        s += n * 2.0 * math.pi * z * (z + 1.0) * R0 * R0 * (MEC2 * MEC2 / (pc2 * b2)) * (
            math.log1p(1.0 / scr) - 1.0 / (1.0 + scr))
    return s


def xs_enuc(mat: Material, t: float) -> float:
    return sum(n * atomic_mass(z) ** 0.9 * 1e-31 for z, n in zip(mat.zs, mat.natoms)) * (
        1.0 + 0.05 * math.log(t / 100.0))


def xs_compton(mat: Material, e: float) -> float:
    k = e / MEC2
    sig_t = 8.0 * math.pi * R0 * R0 / 3.0
    if k < 1e-2:
        s = sig_t * (1.0 - 2.0 * k + 5.2 * k * k - 13.3 * k ** 3)
    else:
        l2 = math.log1p(2.0 * k)
        s = 2.0 * math.pi * R0 * R0 * ((1.0 + k) / (k * k) * (2.0 * (1.0 + k) / (1.0 + 2.0 * k) - l2 / k)
                                       + l2 / (2.0 * k) - (1.0 + 3.0 * k) / (1.0 + 2.0 * k) ** 2)
    return mat.n_el * s


def xs_pair_atom(z: int, e: float) -> float:
    if e <= 2.0 * MEC2:
        return 0.0
    fel, finel = rad_logs(z)
    asym = 7.0 / 9.0 * 4.0 * ALPHA * R0 * R0 * (z * z * (fel - coulomb_correction(z)) + z * finel)
    g = (1.0 - 2.0 * MEC2 / e) ** 2 * (1.0 - math.exp(-e / 8.0)) ** 0.7
    return asym * g


def xs_pair(mat: Material, e: float) -> float:
    return sum(n * xs_pair_atom(z, e) for z, n in zip(mat.zs, mat.natoms))


def xs_gnuc(mat: Material, e: float) -> float:
    if e < 8.0:
        return 0.0
    asym = xs_pair(mat, 1e6)
    return asym * (2e-3 * math.exp(-((e - 15.0) / 5.0) ** 2) + 2e-4 * (1.0 - math.exp(-(e - 8.0) / 20.0)))


# --- numerics --------------------------------------------------------------
def log_grid(emin, emax, n):
    delta = math.log(emax / emin) / (n - 1)
    g = [emin] + [math.exp(math.log(emin) + i * delta) for i in range(1, n - 1)] + [emax]
    return g, math.log(emin), 1.0 / delta


def spline_sd(x, y):
    """Second derivatives of the natural cubic spline through (x, y)."""
    n = len(x)
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    a = np.zeros((n, n))
    r = np.zeros(n)
    a[0, 0] = a[-1, -1] = 1.0
    for i in range(1, n - 1):
        h0, h1 = x[i] - x[i - 1], x[i + 1] - x[i]
        a[i, i - 1] = h0 / 6.0
        a[i, i] = (h0 + h1) / 3.0
        a[i, i + 1] = h1 / 6.0
        r[i] = (y[i + 1] - y[i]) / h1 - (y[i] - y[i - 1]) / h0
    return [float(v) for v in np.linalg.solve(a, r)]


def spline_eval(x, y, sd, xv, i):
    dl = x[i + 1] - x[i]
    b = max(0.0, min(1.0, (xv - x[i]) / dl))
    return y[i] + b * (y[i + 1] - y[i]) + b * (b - 1.0) * ((2.0 - b) * sd[i] + (1.0 + b) * sd[i + 1]) * dl * dl / 6.0


# --- production cuts --------------------------------------------------------
def energy_cuts(mat: Material, range_cut: float):
    """(gamma, e-, e+) production energy cuts for a range cut [mm]."""
    def csda(e):
        n = 200
        es = np.geomspace(1e-4, e, n)
        inv = [1.0 / (dedx_collision(mat, x, 1e30, False) + dedx_brem(mat, x, 1e30)) for x in es]
        return float(np.sum(0.5 * (np.array(inv[1:]) + np.array(inv[:-1])) * np.diff(es))) + 2e-4 / (dedx_collision(mat, 1e-4, 1e30, False))

    def solve(f, target, lo, hi):
        for _ in range(80):
            mid = math.sqrt(lo * hi)
            if f(mid) < target:
                lo = mid
            else:
                hi = mid
        return math.sqrt(lo * hi)

    ecut = max(solve(csda, range_cut, 1e-4, 1e4), 1e-3)

    def att_len(e):
        es, cs = element_tables(mat)
        pe = sandia_eval(es, cs, e)
        return 1.0 / (pe + xs_compton(mat, e) + xs_pair(mat, e))
    gcut = max(solve(att_len, range_cut / 5.0, 1e-5, 1e4), 990e-6)
    return gcut, ecut, ecut


def element_tables(mat: Material):
    """Material Sandia table: union of the element edges, atom-weighted sums."""
    edges = sorted({e for z in mat.zs for e in element_sandia(z)[0]})
    coefs = []
    for e in edges:
        c = [0.0] * 4
        for z, n in zip(mat.zs, mat.natoms):
            ez, cz = element_sandia(z)
            iv = 0
            for i in range(len(ez) - 1, -1, -1):
                if e >= ez[i]:
                    iv = i
                    break
            for j in range(4):
                c[j] += n * cz[iv][j]
        coefs.append(c)
    return edges, coefs


# --- builders -------------------------------------------------------------------
@dataclass
class Couple:
    mat: int
    range_cut: float
    region: int = 0


class StateBuilder:
    NLOSS_BINS = 84
    EMIN_LOSS, EMAX_LOSS = 1e-4, 1e8
    BREM_LIM = 1000.0
    BINS_PER_DECADE = 7

    def __init__(self, materials, couples, regions=None):
        self.mats = materials
        self.couples = couples
        self.regions = regions or [dict()]
        self.cuts = [energy_cuts(materials[c.mat], c.range_cut) for c in couples]

    # -- parameters ---------------------------------------------------------
    def parameters(self):
        regs = []
        for r in self.regions:
            d = dict(fFinalRange=1.0, fDRoverRange=0.2, fLinELossLimit=0.01, fMSCRangeFactor=0.04,
                     fMSCSafetyFactor=0.6, fIsMSCMinimalStepLimit=False, fIsELossFluctuation=True,
                     fIsMultipleStepsInMSCTrans=True, fIsApplyCuts=True)
            d.update(r)
            regs.append(d)
        return dict(fElectronTrackingCut=0.001, fGammaTrackingCut=0.0, fMinLossTableEnergy=self.EMIN_LOSS,
                    fMaxLossTableEnergy=self.EMAX_LOSS, fNumLossTableBins=self.NLOSS_BINS,
                    fElectronBremModelLim=self.BREM_LIM, fIsMSCPositronCor=True, fIsMSCDisplacement=True,
                    fNumRegions=len(regs), fParametersPerRegion=regs)

    # -- elements / materials / couples ---------------------------------------
    def elements(self):
        zs = sorted({z for m in self.mats for z in m.zs})
        out = []
        for z in zs:
            dz = float(z)
            fc = coulomb_correction(dz)
            lz = math.log(dz)
            fel, finel = rad_logs(z)
            z23 = dz ** (2.0 / 3.0)
            vs1 = z23 / (184.15 * 184.15)
            es, cs = element_sandia(z)
            out.append(dict(
                fZet=dz, fZet13=dz ** (1.0 / 3.0), fZet23=z23, fCoulomb=fc, fLogZ=lz,
                fZFactor1=(fel - fc) + finel / dz,
                fDeltaMaxLow=math.exp((42.038 - 8.0 * lz / 3.0) / 8.29) - 0.958,
                fDeltaMaxHigh=math.exp((42.038 - 8.0 * (lz / 3.0 + fc)) / 8.29) - 0.958,
                fILVarS1=1.0 / math.log(vs1), fILVarS1Cond=1.0 / math.log(math.sqrt(2.0) * vs1),
                fSandiaEnergies=es, fSandiaCoefficients=[v for c in cs for v in c],
                fKShellBindingEnergy=k_shell_energy(z)))
        return out

    def material_data(self):
        md = []
        for i, m in enumerate(self.mats):
            zeff = m.zeff
            z16 = zeff ** (1.0 / 6.0)
            z13 = z16 * z16
            es, cs = element_tables(m)
            dum0 = 9.90395e-1 + z16 * (-1.68386e-1 + z16 * 9.3286e-2)
            md.append(dict(
                fG4MatIndex=i, fElementVect=list(m.zs), fNumOfAtomsPerVolumeVect=list(m.natoms),
                fDensity=m.density * GCM3, fDensityCorfactor=MIGDAL * m.n_el, fElectronDensity=m.n_el,
                fRadiationLength=m.radlen, fMeanExEnergy=m.mean_exc * 1e-6,
                fSandiaEnergies=es, fSandiaCoefficients=[v for c in cs for v in c],
                fZeff=zeff, fZeff23=z13 * z13, fZeffSqrt=math.sqrt(zeff),
                fUMSCPar=9.62800e-1 - 8.4848e-2 * math.sqrt(zeff) + 4.3769e-3 * zeff,
                fUMSCStepMinPars=[2.7725e1 / (1.0 + 2.03e-1 * zeff), 6.152 / (1.0 + 1.11e-1 * zeff)],
                fUMSCTailCoeff=[2.3785 - z13 * (4.1981e-1 - z13 * 6.3100e-2),
                                4.7526e-1 + z13 * (1.7694 - z13 * 3.3885e-1),
                                2.3683e-1 - z13 * (1.8111 - z13 * 3.2774e-1),
                                1.7888e-2 + z13 * (1.9659e-2 - z13 * 2.6664e-3)],
                fUMSCThetaCoeff=[dum0 * (1.0 - 8.7780e-2 / zeff), dum0 * (4.0780e-2 + 1.7315e-4 * zeff)]))
        n = len(self.mats)
        return dict(fNumG4Material=n, fNumMaterialData=n, fG4MatIndexToHepEmMatIndex=list(range(n)),
                    fMaterialData=md)

    def matcut_data(self):
        mc = []
        for i, (c, (g, e, p)) in enumerate(zip(self.couples, self.cuts)):
            mc.append(dict(fSecElProdCutE=e, fSecPosProdCutE=p, fSecGamProdCutE=g, fLogSecGamCutE=math.log(g),
                           fHepEmMatIndex=c.mat, fG4MatCutIndex=i, fG4RegionIndex=c.region))
        n = len(mc)
        return dict(fNumG4MatCuts=n, fNumMatCutData=n, fG4MCIndexToHepEmMCIndex=list(range(n)), fMatCutData=mc)

    # -- electron / positron -----------------------------------------------------
    def _selector(self, mat, emin, emax, weight):
        ratio = math.log(emax / emin)
        nb = int(self.BINS_PER_DECADE * ratio / (6.0 * math.log(10.0)))
        nb = max(nb, 3) + 1
        grid, lmin, ild = log_grid(emin, emax, nb)
        data = [float(nb), float(len(mat.zs)), lmin, ild]
        for e in grid:
            data.append(e)
            w = [n * weight(z, e) for z, n in zip(mat.zs, mat.natoms)]
            tot = sum(w)
            acc = 0.0
            for j in range(len(w) - 1):
                acc += w[j]
                data.append(acc / tot if tot > 0 else acc)
        return data

    def electron_data(self, positron: bool):
        nl = self.NLOSS_BINS + 1
        grid, lmin, ild = log_grid(self.EMIN_LOSS, self.EMAX_LOSS, nl)
        eloss = []
        xs_start, xs_data = [], []
        sel = {"Ioni": ([], []), "BremSB": ([], []), "BremRB": ([], [])}
        for c, (gcut, ecut, pcut) in zip(self.couples, self.cuts):
            m = self.mats[c.mat]
            elcut = pcut if positron else ecut
            dedx = [dedx_collision(m, e, elcut, positron) + dedx_brem(m, e, gcut) for e in grid]
            dsd = spline_sd(grid, dedx)
            rng = [2.0 * grid[0] / dedx[0]]
            gl_x, gl_w = np.polynomial.legendre.leggauss(16)
            for i in range(nl - 1):
                a, b = grid[i], grid[i + 1]
                xs = 0.5 * (b - a) * gl_x + 0.5 * (b + a)
                s = sum(w / spline_eval(grid, dedx, dsd, x, i) for x, w in zip(xs, gl_w))
                rng.append(rng[-1] + 0.5 * (b - a) * s)
            rsd = spline_sd(grid, rng)
            isd = spline_sd(rng, grid)
            blk = [0.0] * (5 * nl)
            for i in range(nl):
                blk[2 * i], blk[2 * i + 1] = rng[i], rsd[i]
                blk[2 * (nl + i)], blk[2 * (nl + i) + 1] = dedx[i], dsd[i]
                blk[4 * nl + i] = isd[i]
            eloss.extend(blk)
            # restricted macroscopic cross sections: ioni then brem
            xs_start.append(len(xs_data))
            scale = math.log(self.EMAX_LOSS / self.EMIN_LOSS)
            for emin, fxs in ((elcut if positron else 2.0 * elcut,
                               lambda e: xs_ioni(m, e, elcut, positron)),
                              (gcut, lambda e: xs_brem(m, e, gcut))):
                ne = max(4, int(round(nl * math.log(self.EMAX_LOSS / emin) / scale)) + 1)
                g, lm, il = log_grid(emin, self.EMAX_LOSS, ne)
                vals = [max(0.0, fxs(e)) for e in g]
                imax = int(np.argmax(vals))
                sd = spline_sd(g, vals)
                xs_data.extend([float(ne), g[imax], vals[imax], lm, il])
                for e, v, s in zip(g, vals, sd):
                    xs_data.extend([e, v, s])
            # element selectors
            if len(m.zs) < 2:
                for k in sel:
                    sel[k][0].append(-1)
                continue
            emin_i = elcut if positron else 2.0 * elcut
            specs = {"Ioni": (emin_i, self.EMAX_LOSS, lambda z, e: float(z)),
                     "BremSB": (gcut, self.BREM_LIM,
                                lambda z, e: z * (z + 1.0) * rad_logs(z)[0] * (1.0 + 0.02 * math.log(e / gcut))),
                     "BremRB": (max(gcut, self.BREM_LIM), self.EMAX_LOSS,
                                lambda z, e: z * (z + 1.0) * (rad_logs(z)[0] - coulomb_correction(z) / 3.0))}
            for k, (lo, hi, wf) in specs.items():
                if lo >= hi:
                    sel[k][0].append(-1)
                else:
                    sel[k][0].append(len(sel[k][1]))
                    sel[k][1].extend(self._selector(m, lo, hi, wf))
        # e-/e+ nuclear and transport tables per material
        ngrid, nlmin, nild = log_grid(100.0, 1e8, 128)
        enuc, tr1 = [], []
        for m in self.mats:
            v = [xs_enuc(m, e if i else e + 1e-6) for i, e in enumerate(ngrid)]
            sd = spline_sd(ngrid, v)
            for a, b in zip(v, sd):
                enuc.extend([a, b])
            v = [xs_tr1(m, e) for e in grid]
            sd = spline_sd(grid, v)
            for a, b in zip(v, sd):
                tr1.extend([a, b])
        d = dict(fNumMatCuts=len(self.couples), fNumMaterials=len(self.mats), fELossLogMinEkin=lmin,
                 fELossEILDelta=ild, fELossEnergyGrid=grid, fELossData=eloss,
                 fResMacXSecStartIndexPerMatCut=xs_start, fResMacXSecData=xs_data,
                 fENucLogMinEkin=nlmin, fENucEILDelta=nild, fENucEnergyGrid=ngrid, fENucMacXsecData=enuc,
                 fTr1MacXSecData=tr1)
        for k, (st, dat) in sel.items():
            d[f"fElemSelector{k}StartIndexPerMatCut"] = st
            d[f"fElemSelector{k}Data"] = dat
        return d

    # -- Seltzer-Berger sampling tables ----------------------------------------------
    NUM_EL_E, NUM_KAPPA = 65, 54

    @staticmethod
    def kappa_grid():
        lo = list(np.geomspace(1e-12, 1e-2, 11))
        hi = list(np.geomspace(1e-2, 1.0, 44))[1:]
        k = lo + hi
        k[-1] = 1.0
        return [float(v) for v in k]

    @staticmethod
    def sb_shape(kappa, e, z):
        """Scaled DCS chi(kappa) at e- energy e [MeV] for element z (smooth, positive)."""
        a = 0.9 + 0.08 * math.tanh(math.log10(e))
        b = 0.6 + 0.002 * z
        return 1.0 - a * kappa + b * kappa * kappa + 0.05 * math.exp(-kappa * 50.0)

    def sb_tables(self):
        el_grid, _, _ = log_grid(1e-4, 1e4, self.NUM_EL_E)
        l_el = [math.log(e) for e in el_grid]
        kap = self.kappa_grid()
        lk = [math.log(v) for v in kap]
        used_low = max(1e-3, 1e-4)
        used_high = min(self.BREM_LIM, 1e4)
        zs = sorted({z for m in self.mats for z in m.zs})
        start_per_z = [0] * 121
        data = []
        cutlists = {}
        for z in zs:
            cl = sorted({self.cuts[i][0] for i, c in enumerate(self.couples)
                         if z in self.mats[c.mat].zs and self.cuts[i][0] < used_high})
            if cl:
                cutlists[z] = cl
        for z in zs:
            if z not in cutlists:
                continue
            cl = cutlists[z]
            elemin = max(used_low, min(cl))
            if elemin >= el_grid[-1]:
                imin = self.NUM_EL_E - 1
            else:
                imin = int(np.searchsorted(el_grid, elemin, side="left")) - 1
            imax = self.NUM_EL_E - 1 if used_high >= el_grid[-1] else int(np.searchsorted(el_grid, used_high, side="left"))
            start_per_z[z] = len(data)
            ncut = len(cl)
            data.extend([float((imax - imin + 1) * (ncut + 3 * self.NUM_KAPPA) + 4), float(imin), float(imax), float(ncut)])
            for ie in range(imin, imax + 1):
                e = el_grid[ie]
                pdf = [self.sb_shape(k, e, z) for k in kap]
                # cumulative over ln(kappa) (trapezoid), normalised
                cum = [0.0]
                for j in range(1, len(kap)):
                    cum.append(cum[-1] + 0.5 * (pdf[j] + pdf[j - 1]) * (lk[j] - lk[j - 1]))
                tot = cum[-1]
                cum = [c / tot for c in cum]
                p = [v / tot for v in pdf]
                pa, pb = [], []
                for j in range(len(kap) - 1):
                    dx = lk[j + 1] - lk[j]
                    dxi = cum[j + 1] - cum[j]
                    bb = 1.0 - dxi * dxi / (dx * dx * p[j + 1] * p[j])
                    aa = dxi / (dx * p[j]) - bb - 1.0
                    pa.append(aa)
                    pb.append(bb)
                pa.append(0.0)
                pb.append(0.0)
                # cumulative at each gamma cut (1 if no emission possible)
                for gc in cl:
                    val = 1.0
                    if e > gc:
                        ck = max(1e-12, gc / e)
                        ikl = int(np.searchsorted(kap, ck, side="left")) - 1 if ck > 1e-12 else 0
                        alph = math.log(ck / kap[ikl]) / math.log(kap[ikl + 1] / kap[ikl])
                        aa, bb = pa[ikl], pb[ikl]
                        dum = aa * (alph - 1.0) - 1.0 - bb
                        val = cum[ikl]
                        if alph != 0.0:
                            if abs(bb) > 1e-300:
                                v = -(dum + math.sqrt(dum * dum - 4.0 * bb * alph * alph)) / (2.0 * bb * alph)
                            else:
                                v = -alph / dum
                            val = v * (cum[ikl + 1] - cum[ikl]) + cum[ikl]
                    data.append(val)
                for j in range(len(kap)):
                    data.extend([cum[j], pa[j], pb[j]])
        gc_start, gc_idx = [], []
        for i, c in enumerate(self.couples):
            m = self.mats[c.mat]
            first = True
            st = -1
            for z in m.zs:
                if z not in cutlists:
                    continue
                g = self.cuts[i][0]
                if g >= used_high:
                    continue
                if first:
                    st = len(gc_idx)
                    first = False
                gc_idx.append(cutlists[z].index(g))
            gc_start.append(st)
        return dict(fLogMinElEnergy=math.log(1e-4), fILDeltaElEnergy=1.0 / (math.log(1e8) / 64.0),
                    fElEnergyVect=el_grid, fLElEnergyVect=l_el, fKappaVect=kap, fLKappaVect=lk,
                    fGammaCutIndxStartIndexPerMC=gc_start, fGammaCutIndices=gc_idx,
                    fSBStartTablesStartPerZ=start_per_z, fSBTableData=data)

    # -- gamma -------------------------------------------------------------------------------
    def gamma_data(self):
        g0, l0, d0 = log_grid(1e-4, 0.15, 32)
        g1, l1, d1 = log_grid(0.15, 2.0 * MEC2, 32)
        g2, l2, d2 = log_grid(2.0 * MEC2, 1e8, 256)
        per = 2 * 32 + 3 * 32 + 9 * 256
        mx = []
        for m in self.mats:
            es, cs = element_tables(m)
            for e in g0:
                mx.extend([e, xs_compton(m, e)])
            for e in g1:
                pe = sandia_eval(es, cs, e)
                mx.extend([e, xs_compton(m, e) + pe, pe])
            conv = [xs_pair(m, e) for e in g2]
            comp = [xs_compton(m, e) for e in g2]
            pe = [sandia_eval(es, cs, e) for e in g2]
            tot = [a + b + c + xs_gnuc(m, e) for a, b, c, e in zip(conv, comp, pe, g2)]
            sds = [spline_sd(g2, v) for v in (tot, conv, comp, pe)]
            for i, e in enumerate(g2):
                mx.append(e)
                for v, sd in zip((tot, conv, comp, pe), sds):
                    mx.extend([v[i], sd[i]])
        nconv = int(self.BINS_PER_DECADE * math.log(1e8 / (2.0 * MEC2)) / (6.0 * math.log(10.0)))
        cg, cl, cd = log_grid(2.0 * MEC2, 1e8, nconv)
        cstart, cdata = [], []
        for m in self.mats:
            if len(m.zs) < 2:
                cstart.append(-1)
                continue
            cstart.append(len(cdata))
            cdata.append(float(len(m.zs)))
            for e in cg:
                w = [n * xs_pair_atom(z, e) for z, n in zip(m.zs, m.natoms)]
                tot = sum(w)
                acc = 0.0
                for j in range(len(w) - 1):
                    acc += w[j]
                    cdata.append(acc / tot if tot > 0 else acc)
        return dict(fNumMaterials=len(self.mats), fDataPerMat=per, fNumData0=64, fNumData1=96,
                    fEMin0=1e-4, fEMax0=0.15, fLogEMin0=l0, fEILDelta0=d0,
                    fEMax1=2.0 * MEC2, fLogEMin1=l1, fEILDelta1=d1,
                    fEMax2=1e8, fLogEMin2=l2, fEILDelta2=d2, fMacXsecData=mx,
                    fElemSelectorConvLogMinEkin=cl, fElemSelectorConvEILDelta=cd,
                    fElemSelectorConvStartIndexPerMat=cstart, fElemSelectorConvEgrid=cg,
                    fElemSelectorConvData=cdata)

    def state(self):
        data = dict(fTheMatCutData=self.matcut_data(), fTheMaterialData=self.material_data(),
                    fTheElementData=self.elements(), fTheElectronData=self.electron_data(False),
                    fThePositronData=self.electron_data(True), fTheSBTableData=self.sb_tables(),
                    fTheGammaData=self.gamma_data())
        return dict(fParameters=self.parameters(), fData=data)


def three_couple_state(range_cut=0.7):
    """G4_PbWO4, G4_lAr and G4_Pb at one range cut (the lookup, step and precision workloads)."""
    mats = [NAMED["G4_PbWO4"](), NAMED["G4_lAr"](), NAMED["G4_Pb"]()]
    return StateBuilder(mats, [Couple(i, range_cut) for i in range(3)]).state()


def random_couple_state(n_couples=16, seed=1234, regions=None):
    """n random materials of 1-4 elements, Z in 1..82, density U[1,12] g/cm3,
    cut in {0.1, 0.7, 1.0} mm (the uneven-batching workload)."""
    rng = np.random.default_rng(seed)
    mats, couples = [], []
    for i in range(n_couples):
        ne = int(rng.integers(1, 5))
        zs = sorted({int(z) for z in rng.integers(1, 83, size=ne)})
        rel = [int(v) for v in rng.integers(1, 5, size=len(zs))]
        dens = float(rng.uniform(1.0, 12.0))
        mats.append(Material(f"RND_{i}", zs, rel, dens).finish())
        cut = float(rng.choice([0.1, 0.7, 1.0]))
        reg = int(rng.integers(0, len(regions))) if regions else 0
        couples.append(Couple(i, cut, reg))
    return StateBuilder(mats, couples, regions).state()


def dumps(state) -> str:
    """JSON text; floats written with 17 significant digits (exact round trip)."""
    return json.dumps(state, separators=(",", ":"), allow_nan=False)


def write(state, path):
    with open(path, "w") as f:
        f.write(dumps(state))
