/*
 * hepem_port.h -- TEST INFRASTRUCTURE (oracle).  Data model of the CPU port:
 * a plain restatement of the reference table structs (G4HepEm/G4HepEmData/
 * include/*.hh) filled from the G4HepEmState JSON schema by hepem_port_json.cpp.
 */
#ifndef HEPEM_PORT_H
#define HEPEM_PORT_H

#include <vector>

namespace port {

struct Region {                 // G4HepEmRegionParmeters (G4HepEmParameters.hh:25-45)
  double finalRange, dRoverRange, linELossLimit, mscRangeFactor, mscSafetyFactor;
  bool mscMinimal, eLossFluct, multiSteps, applyCuts;
};

struct Params {                 // G4HepEmParameters (G4HepEmParameters.hh:48-93)
  double electronTrackingCut, gammaTrackingCut, minLossE, maxLossE;
  int numLossBins;
  double bremModelLim;
  bool mscPosCor, mscDisplacement;
  std::vector<Region> regions;
};

struct Elem {                   // G4HepEmElemData (G4HepEmElementData.hh:36-70)
  double Z = -1, Z13 = 0, Z23 = 0, coulomb = 0, logZ = 0, zFactor1 = 0, deltaMaxLow = 0,
         deltaMaxHigh = 0, ilVarS1 = 0, ilVarS1Cond = 0, kShell = 0;
  std::vector<double> sandiaE, sandiaC;
};

struct Mat {                    // G4HepEmMatData (G4HepEmMaterialData.hh:41-77)
  std::vector<int> elems;
  std::vector<double> natoms;
  double density, densityCor, elDensity, radLength, meanExc;
  std::vector<double> sandiaE, sandiaC;
  double zeff, zeff23, zeffSqrt, umscPar, stepMin[2], tail[4], theta[2];
};

struct Couple {                 // G4HepEmMCCData (G4HepEmMatCutData.hh:41-56)
  double elCut, posCut, gamCut, logGamCut;
  int mat, g4Index, region;
};

struct ElData {                 // G4HepEmElectronData (G4HepEmElectronData.hh:81-354)
  int nLoss = 0;
  double lossLogMin = 0, lossILD = 0;
  std::vector<double> lossGrid, loss;
  std::vector<int> xsStart;
  std::vector<double> xs;
  int nNuc = 128;
  double nucLogMin = 0, nucILD = 0;
  std::vector<double> nucGrid, nuc, tr1;
  std::vector<int> selIoniStart, selSBStart, selRBStart;
  std::vector<double> selIoni, selSB, selRB;
};

struct SB {                     // G4HepEmSBTableData (G4HepEmSBTableData.hh:8-42)
  int numKappa = 54;
  double logMinE = 0, ildE = 0;
  double elE[65], lelE[65], kappa[54], lkappa[54];
  std::vector<int> gcStart, gcIdx;
  int startPerZ[121];
  std::vector<double> data;
};

struct Gamma {                  // G4HepEmGammaData (G4HepEmGammaData.hh:15-79)
  int nE0 = 32, nE1 = 32, nE2 = 256;
  int dataPerMat = 0, nData0 = 0, nData1 = 0;
  double eMin0, eMax0, logEMin0, ild0, eMax1, logEMin1, ild1, eMax2, logEMin2, ild2;
  std::vector<double> mx;
  int convN = 0;
  double convLogMin = 0, convILD = 0;
  std::vector<int> convStart;
  std::vector<double> convGrid, conv;
};

struct State {
  Params pars;
  std::vector<Elem> elem;       // indexed by Z, 121 entries
  std::vector<Mat> mats;
  std::vector<Couple> couples;
  ElData el[2];                 // [0] e-, [1] e+
  SB sb;
  Gamma gm;
};

// hepem_port_json.cpp: returns nullptr (and a message) on a schema error
State* load_state(const char* path, const char** err);

}  // namespace port

#endif
