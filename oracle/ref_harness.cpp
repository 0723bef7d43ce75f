/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE.  Drives the UNMODIFIED reference
 * G4HepEmRun functions (compiled from the reference sources by
 * oracle/Makefile into oracle/_ref/libhepem_ref.so) so that tests can compare
 * the GPU path and the CPU port against the reference itself, and so that
 * tests/golden/make_golden.py can write golden vectors.  Nothing in the
 * product links this file.
 *
 * It supplies the consumer side of the reference RNG facade,
 * G4HepEmRandomEngine::flat()/flatArray() (left undefined by the reference,
 * G4HepEm/G4HepEmRun/src/G4HepEmRandomEngine.cc:5-11), reading the per-track
 * uniform stream defined in include/g4hepem_gb300.h, and calls the reference
 * in the order of its own client G4HepEmProcess
 * (apps/examples/TestEm3/src/G4HepEmProcess.cc:119-200).
 */
#include <cstdint>
#include <cstring>
#include <cmath>
#include <fstream>
#include <limits>
#include <vector>

// The Gauss cache of G4HepEmRandomEngine is private; the harness carries it
// across steps as per-track state, so it is opened up for this file only.
#define private public
#include "G4HepEmRandomEngine.hh"
#undef private

#include "G4HepEmData.hh"
#include "G4HepEmParameters.hh"
#include "G4HepEmState.hh"
#include "G4HepEmDataJsonIO.hh"
#include "G4HepEmMatCutData.hh"
#include "G4HepEmMaterialData.hh"
#include "G4HepEmElectronData.hh"
#include "G4HepEmGammaData.hh"
#include "G4HepEmTLData.hh"
#include "G4HepEmTrack.hh"
#include "G4HepEmElectronTrack.hh"
#include "G4HepEmGammaTrack.hh"
#include "G4HepEmElectronManager.hh"
#include "G4HepEmGammaManager.hh"
#include "G4HepEmElectronInteractionBrem.hh"
#include "G4HepEmGammaInteractionConversion.hh"
#include "G4HepEmMath.hh"

#include "g4hepem_gb300.h"
#include "philox.h"

namespace {
struct Stream {
  const double* u;
  int32_t n;
  int32_t cursor;
  uint64_t seed;
  int32_t id;
  int overflow;
  double next() {
    double v;
    if (cursor < n) {
      v = u[cursor];
    } else {
      v = oracle_philox_uniform(seed, id, cursor);
      overflow = 1;
    }
    ++cursor;
    return v;
  }
};
}  // namespace

double G4HepEmRandomEngine::flat() { return static_cast<Stream*>(fObject)->next(); }

void G4HepEmRandomEngine::flatArray(const int size, double* vect) {
  Stream* s = static_cast<Stream*>(fObject);
  for (int i = 0; i < size; ++i) vect[i] = s->next();
}

extern "C" {

void* ref_load_state(const char* path) {
  std::ifstream in(path);
  if (!in.good()) return nullptr;
  return G4HepEmStateFromJson(in);
}

void ref_free_state(void* st) {
  G4HepEmState* s = static_cast<G4HepEmState*>(st);
  if (!s) return;
  FreeG4HepEmData(s->fData);
  delete s->fData;
  FreeG4HepEmParameters(s->fParameters);
  delete s->fParameters;
  delete s;
}

int ref_num_couples(void* st) {
  return static_cast<G4HepEmState*>(st)->fData->fTheMatCutData->fNumMatCutData;
}

// VDT-method log / exp as used by the reference on the host (G4HepEmMath.hh).
void ref_vdt_log(int64_t n, const double* x, double* y) {
  for (int64_t i = 0; i < n; ++i) y[i] = G4HepEmLog(x[i]);
}
void ref_vdt_exp(int64_t n, const double* x, double* y) {
  for (int64_t i = 0; i < n; ++i) y[i] = G4HepEmExp(x[i]);
}
void ref_vdt_pow(int64_t n, const double* x, const double* a, double* y) {
  for (int64_t i = 0; i < n; ++i) y[i] = G4HepEmPow(x[i], a[i]);
}

// Table lookups of the electron tables (2^20-track lookup workload).
void ref_electron_lookup(void* st, int64_t n, int is_positron, const double* ekin,
                         const int32_t* imc, double* xs_ioni, double* xs_brem,
                         double* dedx, double* range, double* invrange_half) {
  G4HepEmData* d = static_cast<G4HepEmState*>(st)->fData;
  const G4HepEmElectronData* el = is_positron ? d->fThePositronData : d->fTheElectronData;
  for (int64_t i = 0; i < n; ++i) {
    const double e = ekin[i];
    const double le = G4HepEmLog(e);
    xs_ioni[i] = G4HepEmElectronManager::GetRestMacXSec(el, imc[i], e, le, true);
    xs_brem[i] = G4HepEmElectronManager::GetRestMacXSec(el, imc[i], e, le, false);
    dedx[i]    = G4HepEmElectronManager::GetRestDEDX(el, imc[i], e, le);
    range[i]   = G4HepEmElectronManager::GetRestRange(el, imc[i], e, le);
    invrange_half[i] = G4HepEmElectronManager::GetInvRange(el, imc[i], 0.5 * range[i]);
  }
}

// Step-limit cross sections (HowFarToDiscreteInteraction inputs) and the
// transport mean free path.
void ref_electron_xs_stepping(void* st, int64_t n, int is_positron, const double* ekin,
                              const int32_t* imc, double* xs_ioni, double* xs_brem,
                              double* xs_annih, double* xs_nuc, double* tr_mfp) {
  G4HepEmData* d = static_cast<G4HepEmState*>(st)->fData;
  const G4HepEmElectronData* el = is_positron ? d->fThePositronData : d->fTheElectronData;
  for (int64_t i = 0; i < n; ++i) {
    const double e = ekin[i];
    const double le = G4HepEmLog(e);
    const int imat = d->fTheMatCutData->fMatCutData[imc[i]].fHepEmMatIndex;
    xs_ioni[i] = G4HepEmElectronManager::GetRestMacXSecForStepping(el, imc[i], e, le, true);
    xs_brem[i] = G4HepEmElectronManager::GetRestMacXSecForStepping(el, imc[i], e, le, false);
    xs_annih[i] = is_positron ? G4HepEmElectronManager::ComputeMacXsecAnnihilationForStepping(
                                    e, d->fTheMaterialData->fMaterialData[imat].fElectronDensity)
                              : 0.0;
    xs_nuc[i] = G4HepEmElectronManager::GetMacXSecNuclearForStepping(el, imat, e, le);
    tr_mfp[i] = G4HepEmElectronManager::GetTransportMFP(el, imat, e, le);
  }
}

// Target element selection for brem (SB or RB), multi-element couples only.
void ref_brem_select_target(void* st, int64_t n, int is_positron, int is_sb,
                            const double* ekin, const int32_t* imc, const double* urnd,
                            int32_t* elem) {
  G4HepEmData* d = static_cast<G4HepEmState*>(st)->fData;
  const G4HepEmElectronData* el = is_positron ? d->fThePositronData : d->fTheElectronData;
  for (int64_t i = 0; i < n; ++i) {
    const int imat = d->fTheMatCutData->fMatCutData[imc[i]].fHepEmMatIndex;
    if (d->fTheMaterialData->fMaterialData[imat].fNumOfElement < 2) { elem[i] = 0; continue; }
    elem[i] = G4HepEmElectronInteractionBrem::SelectTargetAtom(el, imc[i], ekin[i],
                                                               G4HepEmLog(ekin[i]), urnd[i], is_sb != 0);
  }
}

// Gamma total macroscopic cross section, PE cross section and the sampled
// interaction for a given uniform (reference test T/GammaXSections).
void ref_gamma_xs(void* st, int64_t n, const double* ekin, const int32_t* imc,
                  const double* urnd, double* xs_tot, double* xs_pe, int32_t* winner) {
  G4HepEmData* d = static_cast<G4HepEmState*>(st)->fData;
  G4HepEmGammaTrack gt;
  for (int64_t i = 0; i < n; ++i) {
    gt.ReSet();
    G4HepEmTrack* t = gt.GetTrack();
    t->SetEKin(ekin[i]);
    t->SetMCIndex(imc[i]);
    const double tot = G4HepEmGammaManager::GetTotalMacXSec(d, &gt);
    xs_tot[i] = tot;
    t->SetMFP(tot > 0. ? 1. / tot : kALargeValue, 0);
    G4HepEmGammaManager::SampleInteraction(d, &gt, urnd[i]);
    winner[i] = t->GetWinnerProcessIndex();
    xs_pe[i] = winner[i] == 2 ? gt.GetPEmxSec() : 0.0;
  }
}

void ref_conv_select_target(void* st, int64_t n, const double* ekin, const int32_t* imc,
                            const double* urnd, int32_t* elem) {
  G4HepEmData* d = static_cast<G4HepEmState*>(st)->fData;
  for (int64_t i = 0; i < n; ++i) {
    const int imat = d->fTheMatCutData->fMatCutData[imc[i]].fHepEmMatIndex;
    if (d->fTheMaterialData->fMaterialData[imat].fNumOfElement < 2) { elem[i] = 0; continue; }
    elem[i] = G4HepEmGammaInteractionConversion::SelectTargetAtom(d->fTheGammaData, imat, ekin[i],
                                                                  G4HepEmLog(ekin[i]), urnd[i]);
  }
}

// One HowFar + Perform step per track, SoA in/out as in include/g4hepem_gb300.h.
int ref_step(void* st, int64_t n, const hepem_track_state* in, hepem_track_state* out,
             const double* uniforms, int32_t n_uniform, uint64_t seed, hepem_step_out* res) {
  G4HepEmState* s = static_cast<G4HepEmState*>(st);
  G4HepEmData* d = s->fData;
  G4HepEmParameters* p = s->fParameters;
  G4HepEmTLData tl;
  for (int64_t i = 0; i < n; ++i) {
    Stream strm{uniforms + i * (int64_t)n_uniform, n_uniform, in->rng_cursor[i], seed, in->id[i], 0};
    G4HepEmRandomEngine rng(&strm);
    rng.fIsGauss = in->gauss_valid[i] != 0;
    rng.fGauss = in->gauss_value[i];
    tl.SetRandomEngine(&rng);
    tl.ResetNumSecondaryElectronTrack();
    tl.ResetNumSecondaryGammaTrack();
    const int type = in->type[i];
    const double dir[3] = {in->dir_x[i], in->dir_y[i], in->dir_z[i]};
    G4HepEmTrack* t = nullptr;
    double pstep = 0.0;
    const double* disp = nullptr;
    double zero3[3] = {0.0, 0.0, 0.0};
    G4HepEmMSCTrackData* msc = nullptr;
    if (type == 2) {
      G4HepEmGammaTrack* gt = tl.GetPrimaryGammaTrack();
      gt->ReSet();
      t = gt->GetTrack();
      t->SetCharge(0.0);
      t->SetEKin(in->ekin[i]);
      t->SetDirection(dir[0], dir[1], dir[2]);
      t->SetMCIndex(in->imc[i]);
      t->SetID(in->id[i]);
      t->SetNumIALeft(in->nia0[i], 0);
      t->SetOnBoundary(in->on_boundary[i] != 0);
      G4HepEmGammaManager::HowFar(d, p, &tl);
      if (in->on_boundary[i]) {
        G4HepEmGammaManager::UpdateNumIALeft(t);
      } else {
        G4HepEmGammaManager::SelectInteraction(d, &tl);
        G4HepEmGammaManager::Perform(d, p, &tl);
      }
      pstep = t->GetGStepLength();
      disp = zero3;
    } else {
      G4HepEmElectronTrack* et = tl.GetPrimaryElectronTrack();
      et->ReSet();
      t = et->GetTrack();
      t->SetCharge(type == 0 ? -1.0 : 1.0);
      t->SetEKin(in->ekin[i]);
      t->SetDirection(dir[0], dir[1], dir[2]);
      t->SetMCIndex(in->imc[i]);
      t->SetID(in->id[i]);
      t->SetNumIALeft(in->nia0[i], 0);
      t->SetNumIALeft(in->nia1[i], 1);
      t->SetNumIALeft(in->nia2[i], 2);
      t->SetNumIALeft(in->nia3[i], 3);
      t->SetSafety(in->safety[i]);
      t->SetOnBoundary(in->on_boundary[i] != 0);
      msc = et->GetMSCTrackData();
      msc->fInitialRange = in->msc_init_range[i];
      msc->fDynamicRangeFactor = in->msc_dyn_factor[i];
      msc->fTlimitMin = in->msc_tlimit_min[i];
      msc->fIsFirstStep = in->msc_first_step[i] != 0;
      G4HepEmElectronManager::HowFar(d, p, &tl);
      // no geometry: the geometrical step is the proposed one, the direction
      // and the boundary status are unchanged
      G4HepEmElectronManager::Perform(d, p, &tl);
      pstep = et->GetPStepLength();
      disp = msc->GetDisplacement();
    }
    // persistent state out
    out->ekin[i] = t->GetEKin();
    const double* nd = t->GetDirection();
    out->dir_x[i] = nd[0]; out->dir_y[i] = nd[1]; out->dir_z[i] = nd[2];
    out->nia0[i] = t->GetNumIALeft(0);
    if (type != 2) {
      out->nia1[i] = t->GetNumIALeft(1);
      out->nia2[i] = t->GetNumIALeft(2);
      out->nia3[i] = t->GetNumIALeft(3);
      out->msc_init_range[i] = msc->fInitialRange;
      out->msc_dyn_factor[i] = msc->fDynamicRangeFactor;
      out->msc_tlimit_min[i] = msc->fTlimitMin;
      out->msc_first_step[i] = msc->fIsFirstStep ? 1 : 0;
    } else {
      out->nia1[i] = in->nia1[i];
      out->nia2[i] = in->nia2[i];
      out->nia3[i] = in->nia3[i];
      out->msc_init_range[i] = in->msc_init_range[i];
      out->msc_dyn_factor[i] = in->msc_dyn_factor[i];
      out->msc_tlimit_min[i] = in->msc_tlimit_min[i];
      out->msc_first_step[i] = in->msc_first_step[i];
    }
    out->gauss_valid[i] = rng.fIsGauss ? 1 : 0;
    out->gauss_value[i] = rng.fGauss;
    out->rng_cursor[i] = strm.cursor;
    if (out != in) {
      out->type[i] = in->type[i];
      out->imc[i] = in->imc[i];
      out->id[i] = in->id[i];
      out->safety[i] = in->safety[i];
      out->on_boundary[i] = in->on_boundary[i];
    }
    // step results
    res->edep[i] = t->GetEnergyDeposit();
    res->gstep[i] = t->GetGStepLength();
    res->pstep[i] = pstep;
    res->winner[i] = (int8_t)t->GetWinnerProcessIndex();
    res->disp_x[i] = disp[0]; res->disp_y[i] = disp[1]; res->disp_z[i] = disp[2];
    res->flags[i] = strm.overflow ? 1 : 0;
    int ns = 0;
    const int nel = (int)tl.GetNumSecondaryElectronTrack();
    const int ngm = (int)tl.GetNumSecondaryGammaTrack();
    for (int k = 0; k < nel && ns < 2; ++k, ++ns) {
      G4HepEmTrack* sec = tl.GetSecondaryElectronTrack(k)->GetTrack();
      // the reference marks the positron of a pair by charge +1
      // (G4HepEmGammaInteractionConversion.icc:51); all other e- secondaries
      // are electrons
      const bool isPos = (type == 2 && res->winner[i] == 0 && k == 1);
      res->sec_type[2 * i + ns] = isPos ? 1 : 0;
      res->sec_ekin[2 * i + ns] = sec->GetEKin();
      const double* sd = sec->GetDirection();
      res->sec_dir_x[2 * i + ns] = sd[0];
      res->sec_dir_y[2 * i + ns] = sd[1];
      res->sec_dir_z[2 * i + ns] = sd[2];
    }
    for (int k = 0; k < ngm && ns < 2; ++k, ++ns) {
      G4HepEmTrack* sec = tl.GetSecondaryGammaTrack(k)->GetTrack();
      res->sec_type[2 * i + ns] = 2;
      res->sec_ekin[2 * i + ns] = sec->GetEKin();
      const double* sd = sec->GetDirection();
      res->sec_dir_x[2 * i + ns] = sd[0];
      res->sec_dir_y[2 * i + ns] = sd[1];
      res->sec_dir_z[2 * i + ns] = sd[2];
    }
    res->n_sec[i] = (int8_t)ns;
    if (nel + ngm > 2) return -1;  // never expected: at most two per step
  }
  return 0;
}

// HowFar, then the transport of a caller, then Perform, per track, in the
// order of G4HepEmProcess::PostStepGetPhysicalInteractionLength and
// ::PostStepDoIt (apps/examples/TestEm3/src/G4HepEmProcess.cc:119-197).
// `in` holds the pre-step state (on_boundary: the pre-step point's status).
// proposed[i] receives the geometrical step HowFar proposes; transport then
// makes the geometrical step gfrac[i] * proposed[i] (gfrac 1: the proposed
// step itself), leaves the track with direction (ndx, ndy, ndz)[i] and
// post-step boundary status post_bnd[i].  A gamma on a boundary only updates
// its number of interaction lengths left (G4HepEmProcess.cc:167-171); every
// other track gets the new direction, step and status before Perform
// (:175-197), gammas after SelectInteraction.  The direction is set for a
// boundary gamma too (the reference leaves it to Geant4, which moved it).
int ref_step_geom(void* st, int64_t n, const hepem_track_state* in, hepem_track_state* out,
                  const double* uniforms, int32_t n_uniform, uint64_t seed, const double* gfrac,
                  const double* ndx, const double* ndy, const double* ndz, const uint8_t* post_bnd,
                  double* proposed, hepem_step_out* res) {
  G4HepEmState* s = static_cast<G4HepEmState*>(st);
  G4HepEmData* d = s->fData;
  G4HepEmParameters* p = s->fParameters;
  G4HepEmTLData tl;
  for (int64_t i = 0; i < n; ++i) {
    Stream strm{uniforms + i * (int64_t)n_uniform, n_uniform, in->rng_cursor[i], seed, in->id[i], 0};
    G4HepEmRandomEngine rng(&strm);
    rng.fIsGauss = in->gauss_valid[i] != 0;
    rng.fGauss = in->gauss_value[i];
    tl.SetRandomEngine(&rng);
    tl.ResetNumSecondaryElectronTrack();
    tl.ResetNumSecondaryGammaTrack();
    const int type = in->type[i];
    const bool post = post_bnd[i] != 0;
    G4HepEmTrack* t = nullptr;
    double pstep = 0.0;
    const double* disp = nullptr;
    double zero3[3] = {0.0, 0.0, 0.0};
    G4HepEmMSCTrackData* msc = nullptr;
    if (type == 2) {
      G4HepEmGammaTrack* gt = tl.GetPrimaryGammaTrack();
      gt->ReSet();
      t = gt->GetTrack();
      t->SetCharge(0.0);
      t->SetEKin(in->ekin[i]);
      t->SetDirection(in->dir_x[i], in->dir_y[i], in->dir_z[i]);
      t->SetMCIndex(in->imc[i]);
      t->SetID(in->id[i]);
      t->SetNumIALeft(in->nia0[i], 0);
      t->SetOnBoundary(in->on_boundary[i] != 0);
      G4HepEmGammaManager::HowFar(d, p, &tl);
      proposed[i] = t->GetGStepLength();
      const double g = gfrac[i] * proposed[i];
      t->SetDirection(ndx[i], ndy[i], ndz[i]);
      if (post) {
        t->SetGStepLength(g);
        G4HepEmGammaManager::UpdateNumIALeft(t);
      } else {
        t->SetGStepLength(g);
        t->SetOnBoundary(false);
        G4HepEmGammaManager::SelectInteraction(d, &tl);
        G4HepEmGammaManager::Perform(d, p, &tl);
      }
      pstep = t->GetGStepLength();
      disp = zero3;
    } else {
      G4HepEmElectronTrack* et = tl.GetPrimaryElectronTrack();
      et->ReSet();
      t = et->GetTrack();
      t->SetCharge(type == 0 ? -1.0 : 1.0);
      t->SetEKin(in->ekin[i]);
      t->SetDirection(in->dir_x[i], in->dir_y[i], in->dir_z[i]);
      t->SetMCIndex(in->imc[i]);
      t->SetID(in->id[i]);
      t->SetNumIALeft(in->nia0[i], 0);
      t->SetNumIALeft(in->nia1[i], 1);
      t->SetNumIALeft(in->nia2[i], 2);
      t->SetNumIALeft(in->nia3[i], 3);
      t->SetSafety(in->safety[i]);
      t->SetOnBoundary(in->on_boundary[i] != 0);
      msc = et->GetMSCTrackData();
      msc->fInitialRange = in->msc_init_range[i];
      msc->fDynamicRangeFactor = in->msc_dyn_factor[i];
      msc->fTlimitMin = in->msc_tlimit_min[i];
      msc->fIsFirstStep = in->msc_first_step[i] != 0;
      G4HepEmElectronManager::HowFar(d, p, &tl);
      proposed[i] = t->GetGStepLength();
      const double g = gfrac[i] * proposed[i];
      t->SetDirection(ndx[i], ndy[i], ndz[i]);
      t->SetGStepLength(g);
      t->SetOnBoundary(post);
      G4HepEmElectronManager::Perform(d, p, &tl);
      pstep = et->GetPStepLength();
      disp = msc->GetDisplacement();
    }
    out->ekin[i] = t->GetEKin();
    const double* nd = t->GetDirection();
    out->dir_x[i] = nd[0]; out->dir_y[i] = nd[1]; out->dir_z[i] = nd[2];
    out->nia0[i] = t->GetNumIALeft(0);
    if (type != 2) {
      out->nia1[i] = t->GetNumIALeft(1);
      out->nia2[i] = t->GetNumIALeft(2);
      out->nia3[i] = t->GetNumIALeft(3);
      out->msc_init_range[i] = msc->fInitialRange;
      out->msc_dyn_factor[i] = msc->fDynamicRangeFactor;
      out->msc_tlimit_min[i] = msc->fTlimitMin;
      out->msc_first_step[i] = msc->fIsFirstStep ? 1 : 0;
    } else {
      out->nia1[i] = in->nia1[i];
      out->nia2[i] = in->nia2[i];
      out->nia3[i] = in->nia3[i];
      out->msc_init_range[i] = in->msc_init_range[i];
      out->msc_dyn_factor[i] = in->msc_dyn_factor[i];
      out->msc_tlimit_min[i] = in->msc_tlimit_min[i];
      out->msc_first_step[i] = in->msc_first_step[i];
    }
    out->gauss_valid[i] = rng.fIsGauss ? 1 : 0;
    out->gauss_value[i] = rng.fGauss;
    out->rng_cursor[i] = strm.cursor;
    out->type[i] = in->type[i];
    out->imc[i] = in->imc[i];
    out->id[i] = in->id[i];
    out->safety[i] = in->safety[i];
    out->on_boundary[i] = post_bnd[i];
    res->edep[i] = t->GetEnergyDeposit();
    res->gstep[i] = t->GetGStepLength();
    res->pstep[i] = pstep;
    res->winner[i] = (int8_t)t->GetWinnerProcessIndex();
    res->disp_x[i] = disp[0]; res->disp_y[i] = disp[1]; res->disp_z[i] = disp[2];
    res->flags[i] = strm.overflow ? 1 : 0;
    int ns = 0;
    const int nel = (int)tl.GetNumSecondaryElectronTrack();
    const int ngm = (int)tl.GetNumSecondaryGammaTrack();
    for (int k = 0; k < nel && ns < 2; ++k, ++ns) {
      G4HepEmTrack* sec = tl.GetSecondaryElectronTrack(k)->GetTrack();
      const bool isPos = (type == 2 && res->winner[i] == 0 && k == 1);
      res->sec_type[2 * i + ns] = isPos ? 1 : 0;
      res->sec_ekin[2 * i + ns] = sec->GetEKin();
      const double* sd = sec->GetDirection();
      res->sec_dir_x[2 * i + ns] = sd[0];
      res->sec_dir_y[2 * i + ns] = sd[1];
      res->sec_dir_z[2 * i + ns] = sd[2];
    }
    for (int k = 0; k < ngm && ns < 2; ++k, ++ns) {
      G4HepEmTrack* sec = tl.GetSecondaryGammaTrack(k)->GetTrack();
      res->sec_type[2 * i + ns] = 2;
      res->sec_ekin[2 * i + ns] = sec->GetEKin();
      const double* sd = sec->GetDirection();
      res->sec_dir_x[2 * i + ns] = sd[0];
      res->sec_dir_y[2 * i + ns] = sd[1];
      res->sec_dir_z[2 * i + ns] = sd[2];
    }
    res->n_sec[i] = (int8_t)ns;
    if (nel + ngm > 2) return -1;
  }
  return 0;
}

}  // extern "C"
