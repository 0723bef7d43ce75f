// tables.h -- device image of the G4HepEmData tables.
//
// The reference keeps every table as a separately allocated array reached
// through nested structs (G4HepEm/G4HepEmData/include/G4HepEmData.hh:44-74)
// and deep-copies it to the GPU with one cudaMalloc per array
// (G4HepEm/G4HepEmData/src/G4HepEmData.cc:78-101).  Here all arrays live in
// ONE device allocation (the arena); DevTables holds pointers into it and is
// passed to kernels by value (__grid_constant__).  Scalar per-couple,
// per-material and per-element data are packed into small records so that a
// step reads each record with a few wide loads.  Array layouts inside the
// arena are the reference layouts unchanged, so the lookups are the same
// index arithmetic as the reference functions.
#pragma once

#include <cstdint>

namespace hepem {

constexpr int kMaxZ = 120;          // G4HepEmElementData::fMaxZet (G4HepEmElementData.cc:11-13)
constexpr int kNumElEnergySB = 65;  // G4HepEmSBTableData.hh:11-12
constexpr int kNumKappaSB = 54;

struct alignas(16) DevRegion {      // G4HepEmRegionParmeters (G4HepEmParameters.hh:25-45)
  double finalRange, dRoverRange, linELossLimit, mscRangeFactor, mscSafetyFactor;
  int32_t mscMinimal, eLossFluct;
};

struct alignas(16) DevCouple {      // G4HepEmMCCData (G4HepEmMatCutData.hh:41-56) + its region
  double elCut, posCut, gamCut, logGamCut;
  int32_t mat, region, pad0, pad1;
};

struct alignas(16) DevMat {         // G4HepEmMatData (G4HepEmMaterialData.hh:41-77)
  double densityCor, elDensity, radLength, meanExc;
  double zeff, zeff23, zeffSqrt, umscPar;
  double stepMin[2], tail[4], theta[2];
  int32_t nElem, elemOff;           // into matElemZ / matElemN
  int32_t nSandia, sandiaOff;       // into sandiaE / sandiaC (4 per interval)
};

struct alignas(16) DevElem {        // G4HepEmElemData (G4HepEmElementData.hh:36-70), index Z
  double Z13, Z23, coulomb, logZ, zFactor1, deltaMaxLow, deltaMaxHigh, ilVarS1, ilVarS1Cond, kShell;
  int32_t nSandia, sandiaOff, present, pad;
};

struct DevElData {                  // G4HepEmElectronData (G4HepEmElectronData.hh:81-354)
  int32_t nLoss, nNuc;
  double lossLogMin, lossILD, nucLogMin, nucILD;
  const double* lossGrid;           // [nLoss]
  const double* loss;               // [5*nLoss*nCouples]
  const int32_t* xsStart;           // [nCouples]
  const double* xs;
  const double* nucGrid;            // [nNuc]
  const double* nuc;                // [2*nNuc*nMats]
  const double* tr1;                // [2*nLoss*nMats]
  const int32_t* selStart[3];       // Ioni, BremSB, BremRB  [nCouples]
  const double* sel[3];
};

struct DevSB {                      // G4HepEmSBTableData (G4HepEmSBTableData.hh:8-42)
  double logMinE, ildE;
  const double* elE;                // [65]
  const double* lelE;               // [65]
  const double* lkappa;             // [54]
  const int32_t* gcStart;           // [nCouples]
  const int32_t* gcIdx;
  const int32_t* startPerZ;         // [121]
  const double* data;
};

struct DevGamma {                   // G4HepEmGammaData (G4HepEmGammaData.hh:15-79)
  int32_t nE0, nE1, nE2, dataPerMat, nData0, nData1, convN, pad;
  double eMax0, eMax1, logEMin0, ild0, logEMin1, ild1, logEMin2, ild2, convLogMin, convILD;
  const double* mx;                 // [nMats*dataPerMat]
  const int32_t* convStart;         // [nMats]
  const double* convGrid;           // [convN]
  const double* conv;
};

// FP32 copies of the e+- spline tables for the precision form: same layouts
// and index arithmetic as the FP64 arrays they are rounded from.
struct DevElData32 {
  float lossLogMin, lossILD, nucLogMin, nucILD;
  const float* lossGrid;            // [nLoss]
  const float* loss;                // [5*nLoss*nCouples]
  const float* xs;                  // same layout as DevElData::xs
  const float* nucGrid;             // [nNuc]
  const float* nuc;                 // [2*nNuc*nMats]
  const float* tr1;                 // [2*nLoss*nMats]
};

// FP32 copy of the gamma macroscopic cross-section table (same layout as
// DevGamma::mx) with its binning constants
struct DevGamma32 {
  float logEMin0, ild0, logEMin1, ild1, logEMin2, ild2;
  const float* mx;
};

// FP32 copies of the per-region, per-couple and per-material parameters that
// the precision form reads (rounded to nearest from the FP64 records)
struct alignas(16) DevRegion32 {
  float finalRange, dRoverRange, linELossLimit, mscRangeFactor, mscSafetyFactor;
  int32_t mscMinimal, eLossFluct, pad;
};

struct alignas(16) DevCouple32 {
  float elCut, posCut, gamCut, logGamCut;
};

struct alignas(16) DevMat32 {
  float elDensity, radLength, meanExc, zeff, zeff23, zeffSqrt, umscPar, pad;
  float stepMin[2], theta[2], tail[4];
};

struct DevTables {
  // G4HepEmParameters (G4HepEmParameters.hh:48-93)
  double elTrackingCut, gammaTrackingCut, minLossE, bremModelLim;
  float elTrackingCut32, gammaTrackingCut32, minLossE32, bremModelLim32;
  int32_t mscPosCor, mscDisplacement;
  int32_t nCouples, nMats, nRegions, pad;
  const DevRegion* regions;
  const DevCouple* couples;
  const DevMat* mats;
  const DevElem* elems;             // [kMaxZ+1]
  const int32_t* matElemZ;
  const double* matElemN;
  const double* sandiaE;
  const double* sandiaC;
  DevElData el[2];                  // [0] e-, [1] e+
  DevSB sb;
  DevGamma gm;
  DevElData32 el32[2];              // FP32 copies (precision form)
  const DevRegion32* regions32;
  const DevCouple32* couples32;
  const DevMat32* mats32;
  DevGamma32 gm32;
};

}  // namespace hepem
