/*
 * hepem_port_json.cpp -- TEST INFRASTRUCTURE (oracle).  Minimal JSON reader
 * for the G4HepEmState schema (G4HepEm/G4HepEmDataJsonIO/src/
 * G4HepEmDataJsonIOImpl.hh:125-981) filling the port's data model.
 * Numbers go through strtod (correctly rounded), so the 17-digit values of the
 * schema round-trip exactly.
 */
#include "hepem_port.h"

#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>

namespace port {
namespace {

struct JV {
  enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
  bool b = false;
  double num = 0;
  std::string str;
  std::vector<JV> arr;
  std::map<std::string, JV> obj;
  const JV& at(const char* k) const {
    auto it = obj.find(k);
    if (kind != Obj || it == obj.end()) throw std::runtime_error(std::string("missing key ") + k);
    return it->second;
  }
  double d() const {
    if (kind == Num) return num;
    if (kind == Bool) return b ? 1.0 : 0.0;
    throw std::runtime_error("number expected");
  }
  int i() const { return (int)d(); }
  bool bl() const { return kind == Bool ? b : d() != 0.0; }
  std::vector<double> vd() const {
    std::vector<double> v;
    if (kind == Null) return v;
    if (kind != Arr) throw std::runtime_error("array expected");
    for (auto& x : arr) v.push_back(x.d());
    return v;
  }
  std::vector<int> vi() const {
    std::vector<int> v;
    if (kind == Null) return v;
    if (kind != Arr) throw std::runtime_error("array expected");
    for (auto& x : arr) v.push_back(x.i());
    return v;
  }
};

struct Parser {
  const char* p;
  const char* e;
  void ws() { while (p < e && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p; }
  JV value() {
    ws();
    if (p >= e) throw std::runtime_error("unexpected end");
    JV v;
    if (*p == '{') {
      v.kind = JV::Obj; ++p; ws();
      if (*p == '}') { ++p; return v; }
      for (;;) {
        ws();
        JV k = value();
        if (k.kind != JV::Str) throw std::runtime_error("key expected");
        ws();
        if (*p != ':') throw std::runtime_error("':' expected");
        ++p;
        v.obj[k.str] = value();
        ws();
        if (*p == ',') { ++p; continue; }
        if (*p == '}') { ++p; break; }
        throw std::runtime_error("',' or '}' expected");
      }
    } else if (*p == '[') {
      v.kind = JV::Arr; ++p; ws();
      if (*p == ']') { ++p; return v; }
      for (;;) {
        v.arr.push_back(value());
        ws();
        if (*p == ',') { ++p; continue; }
        if (*p == ']') { ++p; break; }
        throw std::runtime_error("',' or ']' expected");
      }
    } else if (*p == '"') {
      v.kind = JV::Str; ++p;
      while (p < e && *p != '"') { if (*p == '\\') ++p; v.str.push_back(*p++); }
      ++p;
    } else if (!strncmp(p, "true", 4)) { v.kind = JV::Bool; v.b = true; p += 4; }
    else if (!strncmp(p, "false", 5)) { v.kind = JV::Bool; v.b = false; p += 5; }
    else if (!strncmp(p, "null", 4)) { v.kind = JV::Null; p += 4; }
    else {
      char* end = nullptr;
      v.kind = JV::Num;
      v.num = strtod(p, &end);
      if (end == p) throw std::runtime_error("bad number");
      p = end;
    }
    return v;
  }
};

void fill_el(ElData& d, const JV& j) {
  d.lossLogMin = j.at("fELossLogMinEkin").d();
  d.lossILD = j.at("fELossEILDelta").d();
  d.lossGrid = j.at("fELossEnergyGrid").vd();
  d.nLoss = (int)d.lossGrid.size();
  d.loss = j.at("fELossData").vd();
  d.xsStart = j.at("fResMacXSecStartIndexPerMatCut").vi();
  d.xs = j.at("fResMacXSecData").vd();
  d.nucLogMin = j.at("fENucLogMinEkin").d();
  d.nucILD = j.at("fENucEILDelta").d();
  d.nucGrid = j.at("fENucEnergyGrid").vd();
  d.nuc = j.at("fENucMacXsecData").vd();
  d.tr1 = j.at("fTr1MacXSecData").vd();
  d.selIoniStart = j.at("fElemSelectorIoniStartIndexPerMatCut").vi();
  d.selIoni = j.at("fElemSelectorIoniData").vd();
  d.selSBStart = j.at("fElemSelectorBremSBStartIndexPerMatCut").vi();
  d.selSB = j.at("fElemSelectorBremSBData").vd();
  d.selRBStart = j.at("fElemSelectorBremRBStartIndexPerMatCut").vi();
  d.selRB = j.at("fElemSelectorBremRBData").vd();
}

}  // namespace

State* load_state(const char* path, const char** err) {
  static thread_local std::string msg;
  try {
    std::ifstream in(path, std::ios::binary);
    if (!in.good()) throw std::runtime_error("cannot open file");
    std::stringstream ss;
    ss << in.rdbuf();
    const std::string text = ss.str();
    Parser ps{text.data(), text.data() + text.size()};
    JV root = ps.value();
    std::unique_ptr<State> s(new State());
    const JV& jp = root.at("fParameters");
    Params& P = s->pars;
    P.electronTrackingCut = jp.at("fElectronTrackingCut").d();
    P.gammaTrackingCut = jp.at("fGammaTrackingCut").d();
    P.minLossE = jp.at("fMinLossTableEnergy").d();
    P.maxLossE = jp.at("fMaxLossTableEnergy").d();
    P.numLossBins = jp.at("fNumLossTableBins").i();
    P.bremModelLim = jp.at("fElectronBremModelLim").d();
    P.mscPosCor = jp.at("fIsMSCPositronCor").bl();
    P.mscDisplacement = jp.at("fIsMSCDisplacement").bl();
    for (auto& r : jp.at("fParametersPerRegion").arr) {
      Region g;
      g.finalRange = r.at("fFinalRange").d();
      g.dRoverRange = r.at("fDRoverRange").d();
      g.linELossLimit = r.at("fLinELossLimit").d();
      g.mscRangeFactor = r.at("fMSCRangeFactor").d();
      g.mscSafetyFactor = r.at("fMSCSafetyFactor").d();
      g.mscMinimal = r.at("fIsMSCMinimalStepLimit").bl();
      g.eLossFluct = r.at("fIsELossFluctuation").bl();
      g.multiSteps = r.at("fIsMultipleStepsInMSCTrans").bl();
      g.applyCuts = r.at("fIsApplyCuts").bl();
      P.regions.push_back(g);
    }
    const JV& jd = root.at("fData");
    // couples
    for (auto& c : jd.at("fTheMatCutData").at("fMatCutData").arr) {
      Couple k;
      k.elCut = c.at("fSecElProdCutE").d();
      k.posCut = c.at("fSecPosProdCutE").d();
      k.gamCut = c.at("fSecGamProdCutE").d();
      k.logGamCut = c.at("fLogSecGamCutE").d();
      k.mat = c.at("fHepEmMatIndex").i();
      k.g4Index = c.at("fG4MatCutIndex").i();
      k.region = c.at("fG4RegionIndex").i();
      s->couples.push_back(k);
    }
    // materials
    for (auto& m : jd.at("fTheMaterialData").at("fMaterialData").arr) {
      Mat t;
      t.elems = m.at("fElementVect").vi();
      t.natoms = m.at("fNumOfAtomsPerVolumeVect").vd();
      t.density = m.at("fDensity").d();
      t.densityCor = m.at("fDensityCorfactor").d();
      t.elDensity = m.at("fElectronDensity").d();
      t.radLength = m.at("fRadiationLength").d();
      t.meanExc = m.at("fMeanExEnergy").d();
      t.sandiaE = m.at("fSandiaEnergies").vd();
      t.sandiaC = m.at("fSandiaCoefficients").vd();
      t.zeff = m.at("fZeff").d();
      t.zeff23 = m.at("fZeff23").d();
      t.zeffSqrt = m.at("fZeffSqrt").d();
      t.umscPar = m.at("fUMSCPar").d();
      auto sm = m.at("fUMSCStepMinPars").vd();
      auto tc = m.at("fUMSCTailCoeff").vd();
      auto th = m.at("fUMSCThetaCoeff").vd();
      if (sm.size() != 2 || tc.size() != 4 || th.size() != 2) throw std::runtime_error("UMSC sizes");
      for (int i = 0; i < 2; ++i) { t.stepMin[i] = sm[i]; t.theta[i] = th[i]; }
      for (int i = 0; i < 4; ++i) t.tail[i] = tc[i];
      s->mats.push_back(t);
    }
    // elements, stored at index Z
    s->elem.resize(121);
    for (auto& e : jd.at("fTheElementData").arr) {
      Elem t;
      t.Z = e.at("fZet").d();
      t.Z13 = e.at("fZet13").d();
      t.Z23 = e.at("fZet23").d();
      t.coulomb = e.at("fCoulomb").d();
      t.logZ = e.at("fLogZ").d();
      t.zFactor1 = e.at("fZFactor1").d();
      t.deltaMaxLow = e.at("fDeltaMaxLow").d();
      t.deltaMaxHigh = e.at("fDeltaMaxHigh").d();
      t.ilVarS1 = e.at("fILVarS1").d();
      t.ilVarS1Cond = e.at("fILVarS1Cond").d();
      t.sandiaE = e.at("fSandiaEnergies").vd();
      t.sandiaC = e.at("fSandiaCoefficients").vd();
      t.kShell = e.at("fKShellBindingEnergy").d();
      const int z = (int)t.Z;
      if (z < 0 || z > 120) throw std::runtime_error("element Z out of range");
      s->elem[z] = t;
    }
    fill_el(s->el[0], jd.at("fTheElectronData"));
    fill_el(s->el[1], jd.at("fThePositronData"));
    // SB tables
    const JV& js = jd.at("fTheSBTableData");
    SB& sb = s->sb;
    sb.logMinE = js.at("fLogMinElEnergy").d();
    sb.ildE = js.at("fILDeltaElEnergy").d();
    auto a = js.at("fElEnergyVect").vd(); if (a.size() != 65) throw std::runtime_error("SB grid");
    auto b = js.at("fLElEnergyVect").vd(); if (b.size() != 65) throw std::runtime_error("SB grid");
    auto c = js.at("fKappaVect").vd(); if (c.size() != 54) throw std::runtime_error("SB kappa");
    auto d = js.at("fLKappaVect").vd(); if (d.size() != 54) throw std::runtime_error("SB kappa");
    for (int i = 0; i < 65; ++i) { sb.elE[i] = a[i]; sb.lelE[i] = b[i]; }
    for (int i = 0; i < 54; ++i) { sb.kappa[i] = c[i]; sb.lkappa[i] = d[i]; }
    sb.gcStart = js.at("fGammaCutIndxStartIndexPerMC").vi();
    sb.gcIdx = js.at("fGammaCutIndices").vi();
    auto spz = js.at("fSBStartTablesStartPerZ").vi();
    if (spz.size() != 121) throw std::runtime_error("SB start per Z");
    for (int i = 0; i < 121; ++i) sb.startPerZ[i] = spz[i];
    sb.data = js.at("fSBTableData").vd();
    // gamma
    const JV& jg = jd.at("fTheGammaData");
    Gamma& g = s->gm;
    g.dataPerMat = jg.at("fDataPerMat").i();
    g.nData0 = jg.at("fNumData0").i();
    g.nData1 = jg.at("fNumData1").i();
    g.eMin0 = jg.at("fEMin0").d(); g.eMax0 = jg.at("fEMax0").d();
    g.logEMin0 = jg.at("fLogEMin0").d(); g.ild0 = jg.at("fEILDelta0").d();
    g.eMax1 = jg.at("fEMax1").d(); g.logEMin1 = jg.at("fLogEMin1").d(); g.ild1 = jg.at("fEILDelta1").d();
    g.eMax2 = jg.at("fEMax2").d(); g.logEMin2 = jg.at("fLogEMin2").d(); g.ild2 = jg.at("fEILDelta2").d();
    g.mx = jg.at("fMacXsecData").vd();
    g.convLogMin = jg.at("fElemSelectorConvLogMinEkin").d();
    g.convILD = jg.at("fElemSelectorConvEILDelta").d();
    g.convStart = jg.at("fElemSelectorConvStartIndexPerMat").vi();
    g.convGrid = jg.at("fElemSelectorConvEgrid").vd();
    g.convN = (int)g.convGrid.size();
    g.conv = jg.at("fElemSelectorConvData").vd();
    return s.release();
  } catch (const std::exception& ex) {
    msg = ex.what();
    if (err) *err = msg.c_str();
    return nullptr;
  }
}

}  // namespace port
