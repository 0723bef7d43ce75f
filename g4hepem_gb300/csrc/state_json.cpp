// state_json.cpp -- G4HepEmState JSON -> validated table arena.
//
// Reads the document written by G4HepEmStateToJson / read by
// G4HepEmStateFromJson (reference G4HepEm/G4HepEmDataJsonIO/src/
// G4HepEmDataJsonIOImpl.hh:125-981; key names, including the reference's
// spellings "fDensityCorfactor" (:360) and "fSBStartTablesStartPerZ" (:727),
// are the schema and are kept).  Every array length and every stored index is
// checked against the sizes it will be used with, so a malformed document is a
// HEPEM_PARSE_ERROR on the host and never an out-of-bounds read on the GPU.
#include "state_image.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace hepem {
namespace {

// ---- a small DOM JSON reader (numbers via strtod: correctly rounded) -------
struct Node {
  enum Kind : uint8_t { Null, False, True, Number, String, Array, Object } kind = Null;
  double num = 0.0;
  std::string str;
  std::vector<Node> items;                       // array elements or object values
  std::vector<std::string> keys;                 // object keys (parallel to items)

  const Node* find(const char* k) const {
    for (size_t i = 0; i < keys.size(); ++i)
      if (keys[i] == k) return &items[i];
    return nullptr;
  }
  const Node& at(const char* k) const {
    if (kind != Object) throw std::runtime_error(std::string("object expected around key ") + k);
    const Node* n = find(k);
    if (!n) throw std::runtime_error(std::string("missing key ") + k);
    return *n;
  }
  double d(const char* what) const {
    if (kind == Number) return num;
    if (kind == True) return 1.0;
    if (kind == False) return 0.0;
    throw std::runtime_error(std::string("number expected: ") + what);
  }
};

class Reader {
 public:
  Reader(const char* b, size_t n) : p_(b), e_(b + n) {}
  Node parse() {
    Node n = value(0);
    ws();
    if (p_ != e_) fail("trailing characters");
    return n;
  }

 private:
  const char* p_;
  const char* e_;
  [[noreturn]] void fail(const char* m) { throw std::runtime_error(std::string("JSON: ") + m); }
  void ws() { while (p_ < e_ && (*p_ == ' ' || *p_ == '\n' || *p_ == '\r' || *p_ == '\t')) ++p_; }
  bool lit(const char* s) {
    size_t l = strlen(s);
    if ((size_t)(e_ - p_) >= l && !memcmp(p_, s, l)) { p_ += l; return true; }
    return false;
  }
  std::string string() {
    std::string s;
    ++p_;
    while (p_ < e_ && *p_ != '"') {
      if (*p_ == '\\') { ++p_; if (p_ >= e_) fail("bad escape"); }
      s.push_back(*p_++);
    }
    if (p_ >= e_) fail("unterminated string");
    ++p_;
    return s;
  }
  Node value(int depth) {
    if (depth > 64) fail("nesting too deep");
    ws();
    if (p_ >= e_) fail("unexpected end");
    Node n;
    const char c = *p_;
    if (c == '{') {
      n.kind = Node::Object;
      ++p_;
      ws();
      if (p_ < e_ && *p_ == '}') { ++p_; return n; }
      for (;;) {
        ws();
        if (p_ >= e_ || *p_ != '"') fail("object key expected");
        n.keys.push_back(string());
        ws();
        if (p_ >= e_ || *p_ != ':') fail("':' expected");
        ++p_;
        n.items.push_back(value(depth + 1));
        ws();
        if (p_ < e_ && *p_ == ',') { ++p_; continue; }
        if (p_ < e_ && *p_ == '}') { ++p_; break; }
        fail("',' or '}' expected");
      }
    } else if (c == '[') {
      n.kind = Node::Array;
      ++p_;
      ws();
      if (p_ < e_ && *p_ == ']') { ++p_; return n; }
      for (;;) {
        n.items.push_back(value(depth + 1));
        ws();
        if (p_ < e_ && *p_ == ',') { ++p_; continue; }
        if (p_ < e_ && *p_ == ']') { ++p_; break; }
        fail("',' or ']' expected");
      }
    } else if (c == '"') {
      n.kind = Node::String;
      n.str = string();
    } else if (lit("true")) {
      n.kind = Node::True;
    } else if (lit("false")) {
      n.kind = Node::False;
    } else if (lit("null")) {
      n.kind = Node::Null;
    } else {
      char buf[64];
      size_t k = 0;
      while (p_ < e_ && k < sizeof(buf) - 1 &&
             (isdigit((unsigned char)*p_) || *p_ == '-' || *p_ == '+' || *p_ == '.' || *p_ == 'e' || *p_ == 'E'))
        buf[k++] = *p_++;
      buf[k] = 0;
      char* end = nullptr;
      n.num = strtod(buf, &end);
      if (k == 0 || end != buf + k) fail("bad number");
      n.kind = Node::Number;
    }
    return n;
  }
};

std::vector<double> vd(const Node& n, const char* what) {
  std::vector<double> v;
  if (n.kind == Node::Null) return v;
  if (n.kind != Node::Array) throw std::runtime_error(std::string("array expected: ") + what);
  v.reserve(n.items.size());
  for (auto& x : n.items) v.push_back(x.d(what));
  return v;
}
std::vector<int32_t> vi(const Node& n, const char* what) {
  std::vector<int32_t> v;
  for (double x : vd(n, what)) {
    if (x != std::floor(x) || std::fabs(x) > 2e9) throw std::runtime_error(std::string("integer expected: ") + what);
    v.push_back((int32_t)x);
  }
  return v;
}
int ival(const Node& n, const char* what) {
  const double x = n.d(what);
  if (x != std::floor(x) || std::fabs(x) > 2e9) throw std::runtime_error(std::string("integer expected: ") + what);
  return (int)x;
}

void check(bool ok, const std::string& msg) {
  if (!ok) throw std::runtime_error("schema: " + msg);
}

// ---- arena builder -----------------------------------------------------------
struct Builder {
  std::vector<uint8_t> bytes;
  std::vector<std::pair<const void**, size_t>> relocs;
  size_t append(const void* src, size_t nb) {
    size_t off = (bytes.size() + 255) & ~size_t(255);
    bytes.resize(off + (nb ? nb : 8), 0);
    if (nb) memcpy(bytes.data() + off, src, nb);
    return off;
  }
  template <class T>
  void put(const T*& field, const std::vector<T>& v) {
    size_t off = append(v.data(), v.size() * sizeof(T));
    relocs.push_back({reinterpret_cast<const void**>(&field), off});
  }
  // FP32 copy (round to nearest) of an FP64 table
  void put32(const float*& field, const std::vector<double>& v) {
    std::vector<float> f(v.size());
    for (size_t i = 0; i < v.size(); ++i) f[i] = (float)v[i];
    put(field, f);
  }
};

struct ElSrc {
  std::vector<double> lossGrid, loss, xs, nucGrid, nuc, tr1, sel[3];
  std::vector<int32_t> xsStart, selStart[3];
};

void read_el(const Node& j, DevElData& d, ElSrc& s, int nCouples, int nMats, int nLossExpected) {
  d.lossLogMin = j.at("fELossLogMinEkin").d("fELossLogMinEkin");
  d.lossILD = j.at("fELossEILDelta").d("fELossEILDelta");
  s.lossGrid = vd(j.at("fELossEnergyGrid"), "fELossEnergyGrid");
  d.nLoss = (int)s.lossGrid.size();
  check(d.nLoss >= 4, "fELossEnergyGrid too short");
  check(d.nLoss == nLossExpected, "fELossEnergyGrid size != fNumLossTableBins+1");
  s.loss = vd(j.at("fELossData"), "fELossData");
  check((long)s.loss.size() == 5L * d.nLoss * nCouples, "fELossData size");
  s.xsStart = vi(j.at("fResMacXSecStartIndexPerMatCut"), "fResMacXSecStartIndexPerMatCut");
  check((int)s.xsStart.size() == nCouples, "fResMacXSecStartIndexPerMatCut size");
  s.xs = vd(j.at("fResMacXSecData"), "fResMacXSecData");
  const long nxs = (long)s.xs.size();
  for (int c = 0; c < nCouples; ++c) {
    const long st = s.xsStart[c];
    check(st >= 0 && st + 5 <= nxs, "xs start index");
    const long ni = (long)s.xs[st];
    check(ni >= 2 && st + 5 + 3 * ni + 5 <= nxs, "ionisation xs block");
    const long sb = st + 3 * ni + 5;
    const long nb = (long)s.xs[sb];
    check(nb >= 2 && sb + 5 + 3 * nb <= nxs, "brem xs block");
  }
  d.nucLogMin = j.at("fENucLogMinEkin").d("fENucLogMinEkin");
  d.nucILD = j.at("fENucEILDelta").d("fENucEILDelta");
  s.nucGrid = vd(j.at("fENucEnergyGrid"), "fENucEnergyGrid");
  d.nNuc = (int)s.nucGrid.size();
  check(d.nNuc >= 2, "fENucEnergyGrid size");
  s.nuc = vd(j.at("fENucMacXsecData"), "fENucMacXsecData");
  check((long)s.nuc.size() == 2L * d.nNuc * nMats, "fENucMacXsecData size");
  s.tr1 = vd(j.at("fTr1MacXSecData"), "fTr1MacXSecData");
  check((long)s.tr1.size() == 2L * d.nLoss * nMats, "fTr1MacXSecData size");
  const char* names[3][2] = {{"fElemSelectorIoniStartIndexPerMatCut", "fElemSelectorIoniData"},
                             {"fElemSelectorBremSBStartIndexPerMatCut", "fElemSelectorBremSBData"},
                             {"fElemSelectorBremRBStartIndexPerMatCut", "fElemSelectorBremRBData"}};
  for (int k = 0; k < 3; ++k) {
    s.selStart[k] = vi(j.at(names[k][0]), names[k][0]);
    check((int)s.selStart[k].size() == nCouples, names[k][0]);
    s.sel[k] = vd(j.at(names[k][1]), names[k][1]);
    for (int c = 0; c < nCouples; ++c) {
      const long st = s.selStart[k][c];
      if (st < 0) continue;
      check(st + 4 <= (long)s.sel[k].size(), "selector start");
      const long K = (long)s.sel[k][st], Q = (long)s.sel[k][st + 1];
      check(K >= 2 && Q >= 1 && st + 4 + K * Q <= (long)s.sel[k].size(), "selector block");
    }
  }
}

}  // namespace

StateImage build_state_image(const char* text, size_t len) {
  Reader rd(text, len);
  Node root = rd.parse();
  StateImage img;
  DevTables& T = img.host;
  memset(&T, 0, sizeof(T));
  Builder B;

  // -- parameters
  const Node& jp = root.at("fParameters");
  T.elTrackingCut = jp.at("fElectronTrackingCut").d("fElectronTrackingCut");
  T.gammaTrackingCut = jp.at("fGammaTrackingCut").d("fGammaTrackingCut");
  T.minLossE = jp.at("fMinLossTableEnergy").d("fMinLossTableEnergy");
  const int nBins = ival(jp.at("fNumLossTableBins"), "fNumLossTableBins");
  T.bremModelLim = jp.at("fElectronBremModelLim").d("fElectronBremModelLim");
  T.mscPosCor = jp.at("fIsMSCPositronCor").d("fIsMSCPositronCor") != 0.0;
  T.mscDisplacement = jp.at("fIsMSCDisplacement").d("fIsMSCDisplacement") != 0.0;
  std::vector<DevRegion> regions;
  for (auto& r : jp.at("fParametersPerRegion").items) {
    DevRegion g{};
    g.finalRange = r.at("fFinalRange").d("fFinalRange");
    g.dRoverRange = r.at("fDRoverRange").d("fDRoverRange");
    g.linELossLimit = r.at("fLinELossLimit").d("fLinELossLimit");
    g.mscRangeFactor = r.at("fMSCRangeFactor").d("fMSCRangeFactor");
    g.mscSafetyFactor = r.at("fMSCSafetyFactor").d("fMSCSafetyFactor");
    g.mscMinimal = r.at("fIsMSCMinimalStepLimit").d("fIsMSCMinimalStepLimit") != 0.0;
    g.eLossFluct = r.at("fIsELossFluctuation").d("fIsELossFluctuation") != 0.0;
    regions.push_back(g);
  }
  T.nRegions = (int)regions.size();
  check(T.nRegions >= 1, "no regions");

  const Node& jd = root.at("fData");
  // -- materials and elements
  const Node& jm = jd.at("fTheMaterialData").at("fMaterialData");
  std::vector<DevMat> mats;
  std::vector<int32_t> matZ;
  std::vector<double> matN, sandiaE, sandiaC;
  for (auto& m : jm.items) {
    DevMat t{};
    auto z = vi(m.at("fElementVect"), "fElementVect");
    auto na = vd(m.at("fNumOfAtomsPerVolumeVect"), "fNumOfAtomsPerVolumeVect");
    check(!z.empty() && z.size() == na.size(), "material element vectors");
    for (int v : z) check(v >= 1 && v <= kMaxZ, "element Z out of range");
    t.nElem = (int)z.size();
    t.elemOff = (int)matZ.size();
    matZ.insert(matZ.end(), z.begin(), z.end());
    matN.insert(matN.end(), na.begin(), na.end());
    t.densityCor = m.at("fDensityCorfactor").d("fDensityCorfactor");
    t.elDensity = m.at("fElectronDensity").d("fElectronDensity");
    t.radLength = m.at("fRadiationLength").d("fRadiationLength");
    t.meanExc = m.at("fMeanExEnergy").d("fMeanExEnergy");
    auto se = vd(m.at("fSandiaEnergies"), "fSandiaEnergies");
    auto sc = vd(m.at("fSandiaCoefficients"), "fSandiaCoefficients");
    check(!se.empty() && sc.size() == 4 * se.size(), "material Sandia table");
    t.nSandia = (int)se.size();
    t.sandiaOff = (int)sandiaE.size();
    sandiaE.insert(sandiaE.end(), se.begin(), se.end());
    sandiaC.insert(sandiaC.end(), sc.begin(), sc.end());
    t.zeff = m.at("fZeff").d("fZeff");
    t.zeff23 = m.at("fZeff23").d("fZeff23");
    t.zeffSqrt = m.at("fZeffSqrt").d("fZeffSqrt");
    t.umscPar = m.at("fUMSCPar").d("fUMSCPar");
    auto sm = vd(m.at("fUMSCStepMinPars"), "fUMSCStepMinPars");
    auto tc = vd(m.at("fUMSCTailCoeff"), "fUMSCTailCoeff");
    auto th = vd(m.at("fUMSCThetaCoeff"), "fUMSCThetaCoeff");
    check(sm.size() == 2 && tc.size() == 4 && th.size() == 2, "UMSC parameter sizes");
    for (int i = 0; i < 2; ++i) { t.stepMin[i] = sm[i]; t.theta[i] = th[i]; }
    for (int i = 0; i < 4; ++i) t.tail[i] = tc[i];
    mats.push_back(t);
  }
  T.nMats = (int)mats.size();
  check(T.nMats >= 1, "no materials");
  std::vector<DevElem> elems(kMaxZ + 1);
  memset(elems.data(), 0, elems.size() * sizeof(DevElem));
  for (auto& e : jd.at("fTheElementData").items) {
    const double zd = e.at("fZet").d("fZet");
    const int z = (int)zd;
    check(z >= 1 && z <= kMaxZ && zd == z, "element fZet");
    DevElem t{};
    t.Z13 = e.at("fZet13").d("fZet13");
    t.Z23 = e.at("fZet23").d("fZet23");
    t.coulomb = e.at("fCoulomb").d("fCoulomb");
    t.logZ = e.at("fLogZ").d("fLogZ");
    t.zFactor1 = e.at("fZFactor1").d("fZFactor1");
    t.deltaMaxLow = e.at("fDeltaMaxLow").d("fDeltaMaxLow");
    t.deltaMaxHigh = e.at("fDeltaMaxHigh").d("fDeltaMaxHigh");
    t.ilVarS1 = e.at("fILVarS1").d("fILVarS1");
    t.ilVarS1Cond = e.at("fILVarS1Cond").d("fILVarS1Cond");
    t.kShell = e.at("fKShellBindingEnergy").d("fKShellBindingEnergy");
    auto se = vd(e.at("fSandiaEnergies"), "fSandiaEnergies");
    auto sc = vd(e.at("fSandiaCoefficients"), "fSandiaCoefficients");
    check(!se.empty() && sc.size() == 4 * se.size(), "element Sandia table");
    t.nSandia = (int)se.size();
    t.sandiaOff = (int)sandiaE.size();
    sandiaE.insert(sandiaE.end(), se.begin(), se.end());
    sandiaC.insert(sandiaC.end(), sc.begin(), sc.end());
    t.present = 1;
    elems[z] = t;
  }
  for (int z : matZ) check(elems[z].present, "material uses an element without element data");

  // -- couples
  const Node& jc = jd.at("fTheMatCutData").at("fMatCutData");
  std::vector<DevCouple> couples;
  for (auto& c : jc.items) {
    DevCouple k{};
    k.elCut = c.at("fSecElProdCutE").d("fSecElProdCutE");
    k.posCut = c.at("fSecPosProdCutE").d("fSecPosProdCutE");
    k.gamCut = c.at("fSecGamProdCutE").d("fSecGamProdCutE");
    k.logGamCut = c.at("fLogSecGamCutE").d("fLogSecGamCutE");
    k.mat = ival(c.at("fHepEmMatIndex"), "fHepEmMatIndex");
    k.region = ival(c.at("fG4RegionIndex"), "fG4RegionIndex");
    check(k.mat >= 0 && k.mat < T.nMats, "couple material index");
    check(k.region >= 0 && k.region < T.nRegions, "couple region index");
    couples.push_back(k);
  }
  T.nCouples = (int)couples.size();
  check(T.nCouples >= 1, "no couples");

  // -- electron / positron data
  ElSrc es[2];
  read_el(jd.at("fTheElectronData"), T.el[0], es[0], T.nCouples, T.nMats, nBins + 1);
  read_el(jd.at("fThePositronData"), T.el[1], es[1], T.nCouples, T.nMats, nBins + 1);

  // -- SB tables
  const Node& js = jd.at("fTheSBTableData");
  T.sb.logMinE = js.at("fLogMinElEnergy").d("fLogMinElEnergy");
  T.sb.ildE = js.at("fILDeltaElEnergy").d("fILDeltaElEnergy");
  auto elE = vd(js.at("fElEnergyVect"), "fElEnergyVect");
  auto lelE = vd(js.at("fLElEnergyVect"), "fLElEnergyVect");
  auto lk = vd(js.at("fLKappaVect"), "fLKappaVect");
  check(elE.size() == kNumElEnergySB && lelE.size() == kNumElEnergySB, "SB energy grid size");
  check(lk.size() == kNumKappaSB && vd(js.at("fKappaVect"), "fKappaVect").size() == kNumKappaSB, "SB kappa grid");
  auto gcStart = vi(js.at("fGammaCutIndxStartIndexPerMC"), "fGammaCutIndxStartIndexPerMC");
  auto gcIdx = vi(js.at("fGammaCutIndices"), "fGammaCutIndices");
  auto spz = vi(js.at("fSBStartTablesStartPerZ"), "fSBStartTablesStartPerZ");
  auto sbd = vd(js.at("fSBTableData"), "fSBTableData");
  check((int)gcStart.size() == T.nCouples, "fGammaCutIndxStartIndexPerMC size");
  check(spz.size() == 121, "fSBStartTablesStartPerZ size");
  // every (couple, element) that can reach SB sampling must have valid tables
  for (int c = 0; c < T.nCouples; ++c) {
    const DevMat& m = mats[couples[c].mat];
    if (couples[c].gamCut >= T.bremModelLim) continue;
    check(gcStart[c] >= 0 && gcStart[c] + m.nElem <= (int)gcIdx.size(), "SB gamma-cut start index");
    for (int e = 0; e < m.nElem; ++e) {
      const int z = matZ[m.elemOff + e];
      const long st = spz[z];
      check(st >= 0 && st + 4 <= (long)sbd.size(), "SB start per Z");
      const long nd = (long)sbd[st], imin = (long)sbd[st + 1], imax = (long)sbd[st + 2], ncut = (long)sbd[st + 3];
      check(imin >= 0 && imax < kNumElEnergySB && imin <= imax && ncut >= 1, "SB table header");
      check(nd == (imax - imin + 1) * (ncut + 3 * kNumKappaSB) + 4 && st + nd <= (long)sbd.size(), "SB table size");
      const int gci = gcIdx[gcStart[c] + e];
      check(gci >= 0 && gci < ncut, "SB gamma-cut index");
    }
  }

  // -- gamma data
  const Node& jg = jd.at("fTheGammaData");
  DevGamma& G = T.gm;
  G.nE0 = 32; G.nE1 = 32; G.nE2 = 256;           // const sizes of G4HepEmGammaData.hh:40-42
  G.dataPerMat = ival(jg.at("fDataPerMat"), "fDataPerMat");
  G.nData0 = ival(jg.at("fNumData0"), "fNumData0");
  G.nData1 = ival(jg.at("fNumData1"), "fNumData1");
  check(G.nData0 == 2 * G.nE0 && G.nData1 == 3 * G.nE1 && G.dataPerMat == G.nData0 + G.nData1 + 9 * G.nE2,
        "gamma table sizes");
  G.eMax0 = jg.at("fEMax0").d("fEMax0");
  G.logEMin0 = jg.at("fLogEMin0").d("fLogEMin0");
  G.ild0 = jg.at("fEILDelta0").d("fEILDelta0");
  G.eMax1 = jg.at("fEMax1").d("fEMax1");
  G.logEMin1 = jg.at("fLogEMin1").d("fLogEMin1");
  G.ild1 = jg.at("fEILDelta1").d("fEILDelta1");
  G.logEMin2 = jg.at("fLogEMin2").d("fLogEMin2");
  G.ild2 = jg.at("fEILDelta2").d("fEILDelta2");
  auto mx = vd(jg.at("fMacXsecData"), "fMacXsecData");
  check((long)mx.size() == (long)T.nMats * G.dataPerMat, "fMacXsecData size");
  G.convLogMin = jg.at("fElemSelectorConvLogMinEkin").d("fElemSelectorConvLogMinEkin");
  G.convILD = jg.at("fElemSelectorConvEILDelta").d("fElemSelectorConvEILDelta");
  auto convStart = vi(jg.at("fElemSelectorConvStartIndexPerMat"), "fElemSelectorConvStartIndexPerMat");
  auto convGrid = vd(jg.at("fElemSelectorConvEgrid"), "fElemSelectorConvEgrid");
  auto conv = vd(jg.at("fElemSelectorConvData"), "fElemSelectorConvData");
  check((int)convStart.size() == T.nMats, "conversion selector start size");
  G.convN = (int)convGrid.size();
  for (int m = 0; m < T.nMats; ++m) {
    if (mats[m].nElem < 2) continue;
    check(G.convN >= 2, "conversion selector grid");
    const long st = convStart[m];
    check(st >= 0 && st + 1 + (long)G.convN * (mats[m].nElem - 1) <= (long)conv.size(), "conversion selector block");
    check((int)conv[st] == mats[m].nElem, "conversion selector element count");
  }
  for (int m = 0; m < T.nMats; ++m) {
    if (mats[m].nElem < 2) continue;
    for (int c = 0; c < T.nCouples; ++c) {
      if (couples[c].mat != m) continue;
      for (int k = 0; k < 3; ++k) {
        const long st = es[0].selStart[k][c];
        if (st >= 0) check((int)es[0].sel[k][st + 1] == mats[m].nElem, "electron selector element count");
        const long sp = es[1].selStart[k][c];
        if (sp >= 0) check((int)es[1].sel[k][sp + 1] == mats[m].nElem, "positron selector element count");
      }
    }
  }

  // -- FP32 parameter copies (precision form)
  T.elTrackingCut32 = (float)T.elTrackingCut;
  T.gammaTrackingCut32 = (float)T.gammaTrackingCut;
  T.minLossE32 = (float)T.minLossE;
  T.bremModelLim32 = (float)T.bremModelLim;
  std::vector<DevRegion32> regions32(regions.size());
  for (size_t i = 0; i < regions.size(); ++i) {
    const DevRegion& r = regions[i];
    regions32[i] = DevRegion32{(float)r.finalRange, (float)r.dRoverRange, (float)r.linELossLimit,
                               (float)r.mscRangeFactor, (float)r.mscSafetyFactor, r.mscMinimal, r.eLossFluct, 0};
  }
  std::vector<DevCouple32> couples32(couples.size());
  for (size_t i = 0; i < couples.size(); ++i) {
    const DevCouple& c = couples[i];
    couples32[i] = DevCouple32{(float)c.elCut, (float)c.posCut, (float)c.gamCut, (float)c.logGamCut};
  }
  std::vector<DevMat32> mats32(mats.size());
  for (size_t i = 0; i < mats.size(); ++i) {
    const DevMat& m = mats[i];
    DevMat32& f = mats32[i];
    f = DevMat32{};
    f.elDensity = (float)m.elDensity;
    f.radLength = (float)m.radLength;
    f.meanExc = (float)m.meanExc;
    f.zeff = (float)m.zeff;
    f.zeff23 = (float)m.zeff23;
    f.zeffSqrt = (float)m.zeffSqrt;
    f.umscPar = (float)m.umscPar;
    for (int k = 0; k < 2; ++k) f.stepMin[k] = (float)m.stepMin[k];
    for (int k = 0; k < 2; ++k) f.theta[k] = (float)m.theta[k];
    for (int k = 0; k < 4; ++k) f.tail[k] = (float)m.tail[k];
  }

  // -- pack the arena
  B.put(T.regions, regions);
  B.put(T.couples, couples);
  B.put(T.mats, mats);
  B.put(T.regions32, regions32);
  B.put(T.couples32, couples32);
  B.put(T.mats32, mats32);
  B.put(T.elems, elems);
  B.put(T.matElemZ, matZ);
  B.put(T.matElemN, matN);
  B.put(T.sandiaE, sandiaE);
  B.put(T.sandiaC, sandiaC);
  for (int p = 0; p < 2; ++p) {
    DevElData& d = T.el[p];
    B.put(d.lossGrid, es[p].lossGrid);
    B.put(d.loss, es[p].loss);
    B.put(d.xsStart, es[p].xsStart);
    B.put(d.xs, es[p].xs);
    B.put(d.nucGrid, es[p].nucGrid);
    B.put(d.nuc, es[p].nuc);
    B.put(d.tr1, es[p].tr1);
    for (int k = 0; k < 3; ++k) {
      B.put(d.selStart[k], es[p].selStart[k]);
      B.put(d.sel[k], es[p].sel[k]);
    }
    DevElData32& f = T.el32[p];
    f.lossLogMin = (float)d.lossLogMin;
    f.lossILD = (float)d.lossILD;
    f.nucLogMin = (float)d.nucLogMin;
    f.nucILD = (float)d.nucILD;
    B.put32(f.lossGrid, es[p].lossGrid);
    B.put32(f.loss, es[p].loss);
    B.put32(f.xs, es[p].xs);
    B.put32(f.nucGrid, es[p].nucGrid);
    B.put32(f.nuc, es[p].nuc);
    B.put32(f.tr1, es[p].tr1);
  }
  B.put(T.sb.elE, elE);
  B.put(T.sb.lelE, lelE);
  B.put(T.sb.lkappa, lk);
  B.put(T.sb.gcStart, gcStart);
  B.put(T.sb.gcIdx, gcIdx);
  B.put(T.sb.startPerZ, spz);
  B.put(T.sb.data, sbd);
  B.put(G.mx, mx);
  T.gm32.logEMin0 = (float)G.logEMin0;
  T.gm32.ild0 = (float)G.ild0;
  T.gm32.logEMin1 = (float)G.logEMin1;
  T.gm32.ild1 = (float)G.ild1;
  T.gm32.logEMin2 = (float)G.logEMin2;
  T.gm32.ild2 = (float)G.ild2;
  B.put32(T.gm32.mx, mx);
  B.put(G.convStart, convStart);
  B.put(G.convGrid, convGrid);
  B.put(G.conv, conv);
  img.bytes = std::move(B.bytes);
  img.relocs.clear();
  for (auto& r : B.relocs)
    img.relocs.push_back({reinterpret_cast<uint8_t*>(r.first) - reinterpret_cast<uint8_t*>(&img.host), r.second});
  return img;
}

void relocate(StateImage& img, DevTables& out, const void* base) {
  out = img.host;
  for (auto& r : img.relocs) {
    const void** field = reinterpret_cast<const void**>(reinterpret_cast<uint8_t*>(&out) + r.first);
    *field = static_cast<const uint8_t*>(base) + r.second;
  }
}

StateImage build_state_image_file(const char* path) {
  std::ifstream in(path, std::ios::binary);
  if (!in.good()) throw std::runtime_error(std::string("cannot open ") + path);
  std::stringstream ss;
  ss << in.rdbuf();
  const std::string s = ss.str();
  return build_state_image(s.data(), s.size());
}

// ---- binary image of the arena ---------------------------------------------------
// Layout (host byte order, 64-bit):
//   "HEPEMIMG" | u32 version | u32 sizeof(DevTables) | u64 arena bytes |
//   u64 number of relocations | DevTables (pointer fields meaningless) |
//   relocations (u64 field offset, u64 arena offset)... | arena bytes |
//   u64 FNV-1a checksum of everything before it.
// Loading it skips parsing and validation of the JSON document: the arena was
// validated when the image was made, and the image carries a checksum.
uint64_t fnv1a(const uint8_t* p, size_t n) {
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

namespace {
const char kImgMagic[8] = {'H', 'E', 'P', 'E', 'M', 'I', 'M', 'G'};
constexpr uint32_t kImgVersion = 1;

template <class T>
void put_pod(std::vector<uint8_t>& out, const T& v) {
  const uint8_t* b = reinterpret_cast<const uint8_t*>(&v);
  out.insert(out.end(), b, b + sizeof(T));
}

template <class T>
T get_pod(const uint8_t* p, size_t size, size_t& off) {
  if (off + sizeof(T) > size) throw std::runtime_error("image: truncated");
  T v;
  memcpy(&v, p + off, sizeof(T));
  off += sizeof(T);
  return v;
}
}  // namespace

std::vector<uint8_t> serialize_image(const StateImage& img) {
  std::vector<uint8_t> out;
  out.insert(out.end(), kImgMagic, kImgMagic + 8);
  put_pod(out, kImgVersion);
  put_pod(out, (uint32_t)sizeof(DevTables));
  put_pod(out, (uint64_t)img.bytes.size());
  put_pod(out, (uint64_t)img.relocs.size());
  DevTables t = img.host;
  for (auto& r : img.relocs) memset(reinterpret_cast<uint8_t*>(&t) + r.first, 0, sizeof(void*));
  put_pod(out, t);
  for (auto& r : img.relocs) {
    put_pod(out, (uint64_t)r.first);
    put_pod(out, (uint64_t)r.second);
  }
  out.insert(out.end(), img.bytes.begin(), img.bytes.end());
  put_pod(out, fnv1a(out.data(), out.size()));
  return out;
}

StateImage deserialize_image(const void* data, size_t size) {
  const uint8_t* p = static_cast<const uint8_t*>(data);
  if (!p || size < 8 + 8 || memcmp(p, kImgMagic, 8) != 0) throw std::runtime_error("image: bad magic");
  if (size < 8 + 8 + 8 + 8 + sizeof(uint64_t)) throw std::runtime_error("image: truncated");
  const uint64_t sum = fnv1a(p, size - sizeof(uint64_t));
  uint64_t stored;
  memcpy(&stored, p + size - sizeof(uint64_t), sizeof(uint64_t));
  if (sum != stored) throw std::runtime_error("image: checksum mismatch");
  size_t off = 8;
  const uint32_t ver = get_pod<uint32_t>(p, size, off);
  if (ver != kImgVersion) throw std::runtime_error("image: unsupported version " + std::to_string(ver));
  const uint32_t tsz = get_pod<uint32_t>(p, size, off);
  if (tsz != sizeof(DevTables)) throw std::runtime_error("image: made by an incompatible build (table record size)");
  const uint64_t nb = get_pod<uint64_t>(p, size, off);
  const uint64_t nr = get_pod<uint64_t>(p, size, off);
  StateImage img;
  img.host = get_pod<DevTables>(p, size, off);
  if (nr > sizeof(DevTables) / sizeof(void*)) throw std::runtime_error("image: bad relocation count");
  for (uint64_t k = 0; k < nr; ++k) {
    const uint64_t fo = get_pod<uint64_t>(p, size, off);
    const uint64_t ao = get_pod<uint64_t>(p, size, off);
    if (fo % alignof(void*) != 0 || fo + sizeof(void*) > sizeof(DevTables) || ao > nb)
      throw std::runtime_error("image: relocation out of range");
    img.relocs.push_back({(size_t)fo, (size_t)ao});
  }
  if (off + nb + sizeof(uint64_t) != size) throw std::runtime_error("image: size mismatch");
  img.bytes.assign(p + off, p + off + nb);
  return img;
}

}  // namespace hepem
