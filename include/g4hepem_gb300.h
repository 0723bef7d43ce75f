/*
 * g4hepem_gb300.h -- C-ABI of the GB300-native G4HepEmRun stepping-physics path.
 *
 * The reference exposes this path as C++ static functions over one track at a
 * time (G4HepEmElectronManager / G4HepEmGammaManager, tables in G4HepEmData,
 * loaded by G4HepEmDataJsonIO, uniforms from a consumer-supplied
 * G4HepEmRandomEngine::flat()).  This header replaces that surface by batch
 * entry points over structure-of-arrays (SoA) track batches in GPU memory.
 * Plain C: pointers, sizes, integer status codes; no CUDA or torch types.
 *
 * Conventions
 *  - Every function returns an int status (HEPEM_OK == 0); none calls exit().
 *  - A context owns the tables (device arena) and is immutable after
 *    hepem_create(); it may be shared by host threads.  Launches go to the
 *    stream passed by the caller (a cudaStream_t passed as void*, NULL = the
 *    legacy default stream).  The caller owns every track buffer.
 *  - Device-pointer entry points return once the work is enqueued; the
 *    *_host variants copy host buffers in and out and return when done.
 *  - Particle type codes: 0 = e-, 1 = e+, 2 = gamma.
 *
 * Per-track uniform random streams (replaces G4HepEmRandomEngine::flat/flatArray,
 * reference G4HepEm/G4HepEmRun/include/G4HepEmRandomEngine.hh:40-51 and
 * G4HepEm/G4HepEmRun/src/G4HepEmRandomEngine.cc:5-11):
 *   uniform k of track i is  uniforms[i*n_uniform + k]          for k <  n_uniform
 *                            hepem_philox_uniform(seed, id[i], k) for k >= n_uniform
 *   starting at k = rng_cursor[i]; the cursor is advanced by the number of
 *   uniforms the step consumed.  Tracks that read past n_uniform get bit 0 of
 *   flags set and are counted in hepem_step_counters.rng_overflow; the stream
 *   continues deterministically instead of wrapping.  Filling the buffer with
 *   hepem_philox_uniform() makes the stream seamless.  With n_uniform = 0 and
 *   at least 2^20 tracks, the batched forms draw the first 32 values of each
 *   stepped track's stream ahead into their workspace; the values, the flag
 *   and the counters are those of the draws in place.
 */
#ifndef G4HEPEM_GB300_H
#define G4HEPEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  HEPEM_OK            = 0,
  HEPEM_BAD_ARG       = 1,  /* null pointer, negative size, bad index range  */
  HEPEM_PARSE_ERROR   = 2,  /* state JSON does not follow the schema          */
  HEPEM_CUDA_ERROR    = 3,  /* a CUDA runtime call failed                     */
  HEPEM_RNG_EXHAUSTED = 4,  /* informational: some track read past n_uniform  */
  HEPEM_TIMEOUT       = 5,  /* a bounded wait gave up                          */
  HEPEM_OOM_ADMISSION = 6,  /* serving: request does not fit the memory budget */
  HEPEM_NO_DEVICE     = 7,  /* no CUDA device visible                         */
  HEPEM_CANCELLED     = 8   /* serving: the request was cancelled             */
};

typedef struct hepem_ctx hepem_ctx;

/* Forms of the step, for the entry points that take one: the plain FP64 form
 * (hepem_step), the batched FP64 form (hepem_step_batched) and the precision
 * form (hepem_step_mixed). */
enum { HEPEM_FORM_PLAIN = 0, HEPEM_FORM_BATCHED = 1, HEPEM_FORM_MIXED = 2 };

/* ---- track batches ----------------------------------------------------- */
/* Persistent per-track state, SoA, arrays of length n.  Mirrors the fields of
 * G4HepEmTrack (G4HepEm/G4HepEmRun/include/G4HepEmTrack.hh:246-264),
 * G4HepEmElectronTrack (.../G4HepEmElectronTrack.hh:20-93), the persistent part
 * of G4HepEmMSCTrackData (.../G4HepEmMSCTrackData.hh:14-133) and the Gauss
 * cache of G4HepEmRandomEngine (.../G4HepEmRandomEngine.hh:50-70). */
typedef struct hepem_track_state {
  int8_t*  type;           /* 0 e-, 1 e+, 2 gamma                              */
  int32_t* imc;            /* material-cuts couple index (G4HepEmMCCData)     */
  int32_t* id;             /* track id: RNG stream id and parent id           */
  double*  ekin;           /* kinetic energy [MeV]                            */
  double*  dir_x;          /* unit direction                                  */
  double*  dir_y;
  double*  dir_z;
  double*  nia0;           /* number-of-interaction-left per process; <=0     */
  double*  nia1;           /*   means "sample a new one" (gamma uses nia0)    */
  double*  nia2;
  double*  nia3;
  double*  safety;         /* isotropic safety [mm] (e+- MSC step limit)      */
  uint8_t* on_boundary;    /* step starts and ends on a volume boundary       */
  double*  msc_init_range; /* MSC fInitialRange        (1e21 for a new track) */
  double*  msc_dyn_factor; /* MSC fDynamicRangeFactor  (0.04)                 */
  double*  msc_tlimit_min; /* MSC fTlimitMin           (1e-7 mm)              */
  uint8_t* msc_first_step; /* MSC fIsFirstStep         (1)                    */
  uint8_t* gauss_valid;    /* cached second Gaussian of the polar method      */
  double*  gauss_value;
  int32_t* rng_cursor;     /* next uniform index of this track's stream       */
} hepem_track_state;

/* Per-step results and secondaries (at most 2 per step, fixed slots 2i, 2i+1). */
typedef struct hepem_step_out {
  double*  edep;           /* energy deposit of the step [MeV]                */
  double*  gstep;          /* geometrical step length [mm]                    */
  double*  pstep;          /* true (physical) step length [mm]                */
  int8_t*  winner;         /* e+-: -2 MSC, -1 continuous, 0 ioni, 1 brem,
                              2 annihilation, 3 nuclear; gamma: 0 conversion,
                              1 Compton, 2 photoelectric, 3 nuclear           */
  double*  disp_x;         /* MSC lateral displacement (lab frame) [mm]       */
  double*  disp_y;
  double*  disp_z;
  uint8_t* flags;          /* bit0: read past n_uniform                       */
  int8_t*  n_sec;          /* number of secondaries of track i (0..2)         */
  int8_t*  sec_type;       /* [2n] particle type of the secondary             */
  double*  sec_ekin;       /* [2n]                                            */
  double*  sec_dir_x;      /* [2n]                                            */
  double*  sec_dir_y;
  double*  sec_dir_z;
} hepem_step_out;

typedef struct hepem_step_counters {
  uint64_t steps;          /* tracks stepped                                  */
  uint64_t uniforms;       /* uniforms consumed                               */
  uint64_t rng_overflow;   /* tracks that read past n_uniform                 */
  uint64_t secondaries;    /* secondaries produced                            */
  uint64_t interactions[8];/* e+- winner 0..3, gamma winner 0..3              */
  uint64_t fp64_fallback;  /* precision form: tracks re-stepped in FP64       */
} hepem_step_counters;

/* ---- context ------------------------------------------------------------ */
/* Parse a G4HepEmState JSON document (the schema of G4HepEmStateFromJson,
 * reference G4HepEm/G4HepEmDataJsonIO/include/G4HepEmDataJsonIO.hh:84 and
 * src/G4HepEmDataJsonIOImpl.hh:125-981) and build the device table arena on
 * the current CUDA device.  Replaces G4HepEmStateFromJson +
 * CopyG4HepEmDataToGPU (G4HepEm/G4HepEmData/src/G4HepEmData.cc:78-101). */
int  hepem_create(const char* state_json, size_t len, hepem_ctx** out);
int  hepem_create_from_file(const char* path, hepem_ctx** out);
/* Binary image of the table arena: parsing the JSON document once and keeping
 * the image makes later loads a checksum and one copy (JSON loading is slow
 * for large states: G4HepEm/G4HepEmDataJsonIO/src/G4HepEmDataJsonIOImpl.hh).
 * hepem_image_from_json needs no GPU: with out == NULL it only reports the
 * size.  hepem_image_check validates an image (magic, version, build
 * compatibility, checksum, bounds).  hepem_create_from_image builds the same
 * context as hepem_create on the same document. */
int  hepem_image_from_json(const char* state_json, size_t len, void* out,
                           size_t capacity, size_t* size);
int  hepem_image_check(const void* image, size_t size, int64_t* arena_bytes);
int  hepem_create_from_image(const void* image, size_t size, hepem_ctx** out);
/* Replaces FreeG4HepEmData / FreeG4HepEmDataOnGPU (G4HepEmData.hh:80-88). */
int  hepem_destroy(hepem_ctx* ctx);
/* Table sizes: number of couples, materials, regions; bytes of the arena. */
int  hepem_info(const hepem_ctx* ctx, int32_t* n_couples, int32_t* n_materials,
                int32_t* n_regions, int64_t* arena_bytes);
const char* hepem_status_string(int status);
/* Last error message of the calling thread (empty if none). */
const char* hepem_last_error(void);

/* ---- electron table lookups (device pointers) ---------------------------- */
/* For each track: restricted macroscopic ionisation and brem cross sections,
 * restricted dE/dx, range, and inverse range at 0.5*range.  Replaces
 * G4HepEmElectronManager::GetRestMacXSec / GetRestDEDX / GetRestRange /
 * GetInvRange (G4HepEm/G4HepEmRun/include/G4HepEmElectronManager.hh:230-248,
 * .icc:486-532).  log(ekin) is computed on the device. */
int  hepem_electron_lookup(const hepem_ctx* ctx, int64_t n, int is_positron,
                           const double* ekin, const int32_t* imc,
                           double* xs_ioni, double* xs_brem, double* dedx,
                           double* range, double* invrange_half, void* stream);
/* The same five quantities from the FP32 tables of the precision form in FP32
 * arithmetic (outputs widened to double): what hepem_step_mixed looks up. */
int  hepem_electron_lookup_mixed(const hepem_ctx* ctx, int64_t n, int is_positron,
                                 const double* ekin, const int32_t* imc,
                                 double* xs_ioni, double* xs_brem, double* dedx,
                                 double* range, double* invrange_half, void* stream);

/* ---- one physics step (device pointers) ---------------------------------- */
/* e+-: G4HepEmElectronManager::HowFar then ::Perform
 *      (G4HepEm/G4HepEmRun/include/G4HepEmElectronManager.hh:71,222).
 * gamma: G4HepEmGammaManager::HowFar, ::SelectInteraction, ::Perform
 *      (G4HepEm/G4HepEmRun/include/G4HepEmGammaManager.hh:32,39,51),
 * in the call order of the reference client
 * (apps/examples/TestEm3/src/G4HepEmProcess.cc:119-200) with the geometrical
 * step equal to the proposed one.  `out` may alias `in` (in-place stepping).
 * counters: device pointer or NULL; accumulated with atomics. */
int  hepem_step(const hepem_ctx* ctx, int64_t n, const hepem_track_state* in,
                hepem_track_state* out, const double* uniforms, int32_t n_uniform,
                uint64_t seed, hepem_step_out* res, hepem_step_counters* counters,
                void* stream);

/* Batched form of hepem_step: same arguments, same results bit for bit.
 * Tracks are sorted by particle, couple and energy and, after the continuous
 * part of the step, into per-interaction queues, so that every warp executes
 * one model at a time (no reference counterpart: a scheduling of the same
 * G4HepEmElectronManager / G4HepEmGammaManager calls).  Uses a stream-ordered
 * workspace of about 48 bytes per track (cudaMallocAsync on `stream`). */
int  hepem_step_batched(const hepem_ctx* ctx, int64_t n, const hepem_track_state* in,
                        hepem_track_state* out, const double* uniforms, int32_t n_uniform,
                        uint64_t seed, hepem_step_out* res, hepem_step_counters* counters,
                        void* stream);

/* Same as hepem_step_batched, except that this library allocates no device
 * memory for the call.  For callers that cannot let a library allocate:
 * applications that give all device memory to their own pool allocator at
 * start-up, serving loops that must not enter an allocator on their latency
 * path, integrations that forbid hidden allocations in third-party libraries.
 * The workspace is a fixed 32 MiB array in the library's device image, held
 * by every GPU that loads the library until the process exits; batches are
 * limited to HEPEM_NOALLOC_MAX_TRACKS tracks (larger ones: HEPEM_BAD_ARG).
 * The first call on a device looks up the array's device address on the
 * current device (make it before any stream capture); the current device must
 * be the context's.  The address is kept for the life of the device's primary
 * context: make no call after a cudaDeviceReset in the same process.  All calls share the array: calls that overlap on the GPU
 * (other streams, other threads) race.  No counterpart in the reference (its
 * host functions need no device workspace). */
#define HEPEM_NOALLOC_MAX_TRACKS 524288
int  hepem_step_batched_noalloc(const hepem_ctx* ctx, int64_t n, const hepem_track_state* in,
                                hepem_track_state* out, const double* uniforms,
                                int32_t n_uniform, uint64_t seed, hepem_step_out* res,
                                hepem_step_counters* counters, void* stream);

/* Many sub-batches (e.g. the track batches of several events) stepped in ONE
 * sorted and queued pass: one sort and one sequence of stage kernels over
 * all of them, instead of one call per sub-batch.  The sub-batches lie in
 * the same SoA arrays: sub-batch b is tracks [offset, offset + n) with
 * uniforms keyed by its own seed (uniforms[i*n_uniform + k] for track i, and
 * hepem_philox_uniform(seed_b, id[i], k) past them).  Ranges must not overlap;
 * tracks outside every range are left as they are (also in `out`).  form:
 * HEPEM_FORM_BATCHED or HEPEM_FORM_MIXED; the results equal one
 * hepem_step_batched / hepem_step_mixed call per sub-batch, bit for bit.
 * `batches` is a host array; counters (device, may be NULL) are the sums
 * over all sub-batches.  Uses a stream-ordered workspace.  No reference
 * counterpart (the reference steps one track at a time). */
typedef struct hepem_subbatch {
  int64_t  offset;   /* first track of the sub-batch in the arrays            */
  int64_t  n;        /* number of its tracks                                  */
  uint64_t seed;     /* key of its tracks' uniform streams                    */
} hepem_subbatch;
int  hepem_step_subbatches(const hepem_ctx* ctx, int form, int32_t n_batches, const hepem_subbatch* batches,
                           const hepem_track_state* in, hepem_track_state* out, const double* uniforms,
                           int32_t n_uniform, hepem_step_out* res, hepem_step_counters* counters,
                           void* stream);

/* Precision form of hepem_step_batched: the e+- HowFar and continuous step
 * (step limits, MSC, energy loss and its fluctuations, the delta-interaction
 * test), the gamma HowFar and interaction choice, and the interaction models
 * but the photoelectric effect and annihilation at rest run from FP32 copies
 * of the tables in FP32 arithmetic; FP64 is kept for the range->energy
 * inversion of the mean loss, the energy and deposit bookkeeping and
 * decisions on exact inputs.  Every discrete decision taken
 * on FP32 values is guarded: a track whose FP32 operands of any decision are
 * closer than 2^-12 relative is re-stepped by the FP64 code
 * (counters->fp64_fallback), so discrete outcomes (interaction, rejection
 * acceptances, sampled counts) equal the FP64 path's, and continuous outputs
 * agree with it within 1e-5 relative (largest measured 6.8e-6, RMS ~1e-7).
 * No reference counterpart (the reference has FP64 only). */
int  hepem_step_mixed(const hepem_ctx* ctx, int64_t n, const hepem_track_state* in,
                      hepem_track_state* out, const double* uniforms,
                      int32_t n_uniform, uint64_t seed, hepem_step_out* res,
                      hepem_step_counters* counters, void* stream);

/* Same with HOST buffers: copies the batch in, steps it (batched form),
 * copies the results back and synchronises.  Pinned host memory is fastest.
 * Reference counterpart: the per-track G4HepEmElectronManager::HowFar/Perform
 * and G4HepEmGammaManager::HowFar/SelectInteraction/Perform calls of
 * apps/examples/TestEm3/src/G4HepEmProcess.cc:144-197 over a host batch. */
int  hepem_step_host(const hepem_ctx* ctx, int64_t n, const hepem_track_state* in,
                     hepem_track_state* out, const double* uniforms,
                     int32_t n_uniform, uint64_t seed, hepem_step_out* res,
                     hepem_step_counters* counters, void* stream);

/* The same through the precision form (hepem_step_mixed). */
int  hepem_step_host_mixed(const hepem_ctx* ctx, int64_t n, const hepem_track_state* in,
                           hepem_track_state* out, const double* uniforms,
                           int32_t n_uniform, uint64_t seed, hepem_step_out* res,
                           hepem_step_counters* counters, void* stream);

/* ---- HowFar and Perform as two calls, with the caller's transport between -- */
/* The reference client calls HowFar, lets Geant4's transport move the track
 * -- the geometry may shorten the step, a field may turn the direction, the
 * step may end on a volume boundary -- and then Perform
 * (apps/examples/TestEm3/src/G4HepEmProcess.cc:119-197).  hepem_howfar and
 * hepem_perform are those two calls over a batch:
 *
 *   hepem_howfar(ctx, form, n, tracks, ..., gstep, limits, ...)
 *       e+-: G4HepEmElectronManager::HowFar (G4HepEmElectronManager.hh:71,
 *       .icc:35-169); gamma: G4HepEmGammaManager::HowFar
 *       (G4HepEmGammaManager.hh:32, .icc:27-48).  gstep[i] (device, n) =
 *       the proposed geometrical step; `limits` (device, hepem_step_limit_bytes(n)
 *       bytes) receives what Perform needs (the reference keeps it in the
 *       thread-local primary track).  The track state is not modified: the
 *       sampled numbers of interaction lengths, the MSC step-limit state and
 *       the uniforms consumed are kept in `limits` until Perform.
 *   -- the caller transports the tracks: it may lower gstep[i] to the step
 *      made (0 <= gstep[i]), write the direction after transport to dir_*,
 *      and set on_boundary[i] to the post-step status (1: the step ended on a
 *      boundary) --
 *   hepem_perform(ctx, form, n, in, out, gstep, limits, ..., res, ...)
 *       e+-: G4HepEmElectronManager::Perform (.hh:222, .icc:171-483), whose
 *       UpdatePStepLength converts a shortened geometrical step back to the
 *       true length (.icc:171-203, :653-691); on a boundary no discrete
 *       interaction happens (.icc:433).  gamma: on a boundary only
 *       UpdateNumIALeft (G4HepEmGammaManager.icc:95-104, the client's
 *       G4HepEmProcess.cc:167-171); otherwise SelectInteraction and Perform
 *       (G4HepEmGammaManager.hh:39,51), as the client calls them back to back
 *       (G4HepEmProcess.cc:187-188).
 *
 * With gstep, direction and on_boundary left as HowFar found them, the pair
 * gives the results of hepem_step bit for bit.  Both calls take the same n,
 * the same track order, the same form, the same uniforms/seed (Perform
 * continues the stream where HowFar stopped), and `in` of hepem_perform is the
 * state given to hepem_howfar with only dir_*, on_boundary (and, for an
 * in-place call, nothing else) changed; `out` may alias `in`.
 * form: HEPEM_FORM_PLAIN (one thread per track, FP64), HEPEM_FORM_BATCHED
 * (the sorted, queued FP64 form of hepem_step_batched; stream-ordered
 * workspace) or HEPEM_FORM_MIXED (the precision form of hepem_step_mixed:
 * results within 1e-5 of the FP64 forms, discrete outcomes identical; e+-
 * steps that transport shortened, and e+- tracks whose FP32 decisions are too
 * close to call, are stepped again in FP64 from the pre-step state).
 * counters (device, may be NULL): hepem_howfar adds the uniforms it consumed;
 * hepem_perform adds the step, its uniforms, interactions and secondaries. */
int64_t hepem_step_limit_bytes(int64_t n);
int  hepem_howfar(const hepem_ctx* ctx, int form, int64_t n, const hepem_track_state* tracks,
                  const double* uniforms, int32_t n_uniform, uint64_t seed, double* gstep, void* limits,
                  hepem_step_counters* counters, void* stream);
int  hepem_perform(const hepem_ctx* ctx, int form, int64_t n, const hepem_track_state* in,
                   hepem_track_state* out, const double* gstep, const void* limits,
                   const double* uniforms, int32_t n_uniform, uint64_t seed, hepem_step_out* res,
                   hepem_step_counters* counters, void* stream);
/* The same two calls with HOST buffers (tracks, uniforms, gstep, limits,
 * results and counters on the host): each copies its inputs to the device,
 * runs, copies its outputs back and synchronises.  Pinned memory is fastest. */
int  hepem_howfar_host(const hepem_ctx* ctx, int form, int64_t n, const hepem_track_state* tracks,
                       const double* uniforms, int32_t n_uniform, uint64_t seed, double* gstep,
                       void* limits, hepem_step_counters* counters, void* stream);
int  hepem_perform_host(const hepem_ctx* ctx, int form, int64_t n, const hepem_track_state* in,
                        hepem_track_state* out, const double* gstep, const void* limits,
                        const double* uniforms, int32_t n_uniform, uint64_t seed, hepem_step_out* res,
                        hepem_step_counters* counters, void* stream);

/* ---- single functions of the path, as the reference's device tests call them */
/* Each takes n energies (device), couple indices and, where a selection is
 * made, uniforms; precision 0 runs the FP64 code of hepem_step, 1 the FP32
 * code of hepem_step_mixed (a selection whose FP32 operands are too close to
 * call is made again in FP64, as in the step).  Inputs outside the tables
 * give NaN (cross sections) or -1 (indices).
 *
 * hepem_electron_xs_stepping: the step-limit macroscopic cross sections of e-
 * (is_positron 0) or e+ -- restricted ionisation and brem at the stepping
 * energy (GetRestMacXSecForStepping), e+ annihilation (0 for e-), e-nuclear,
 * and the transport mean free path (G4HepEmElectronManager.icc:534-599); the
 * reference's device test testing/ElectronXSections/src/ResMacXSecs.cu:16-33
 * and its TestXSectionData. */
int  hepem_electron_xs_stepping(const hepem_ctx* ctx, int64_t n, int is_positron, int precision,
                                const double* ekin, const int32_t* imc, double* xs_ioni, double* xs_brem,
                                double* xs_annih, double* xs_nuc, double* tr_mfp, void* stream);
/* Target element (index in the material's element list, 0 for a one-element
 * material) of Seltzer-Berger (is_sb 1) or relativistic (0) brem for the
 * uniform urnd[i]: G4HepEmElectronInteractionBrem::SelectTargetAtom
 * (G4HepEmElectronInteractionBrem.icc), as in
 * testing/ElectronTargetElementSelector/src/ElemSelector.cu:14-30. */
int  hepem_brem_select_target(const hepem_ctx* ctx, int64_t n, int is_positron, int is_sb, int precision,
                              const double* ekin, const int32_t* imc, const double* urnd, int32_t* elem,
                              void* stream);
/* Target element of pair production for urnd[i] in the couple's material:
 * G4HepEmGammaInteractionConversion::SelectTargetAtom, as in
 * testing/GammaTargetElementSelector/src/GammaElemSelector.cu:14-27. */
int  hepem_conv_select_target(const hepem_ctx* ctx, int64_t n, int precision, const double* ekin,
                              const int32_t* imc, const double* urnd, int32_t* elem, void* stream);
/* Gamma total macroscopic cross section (GetTotalMacXSec), the interaction
 * SampleInteraction selects for urnd[i] (0 conversion, 1 Compton, 2
 * photoelectric, 3 gamma-nuclear) and, when it is the photoelectric effect,
 * its macroscopic cross section (else 0) (G4HepEmGammaManager.icc:108-219);
 * as in testing/GammaXSections/src/GammaMacXSecs.cu:20-30. */
int  hepem_gamma_xs(const hepem_ctx* ctx, int64_t n, int precision, const double* ekin, const int32_t* imc,
                    const double* urnd, double* xs_tot, double* xs_pe, int32_t* winner, void* stream);

/* ---- stage timing (profiling aid; not thread-safe) ------------------------ */
/* enable != 0: the following hepem_step_batched calls on this context record
 * CUDA events around each of their stage kernels (no reference counterpart:
 * the reference has no stage structure).  hepem_stage_times then returns the
 * milliseconds of each stage of the last such call (it waits for it) and,
 * if names is not NULL, static stage names. */
int  hepem_profile_stages(hepem_ctx* ctx, int enable);
int  hepem_stage_times(hepem_ctx* ctx, float* ms, const char** names, int32_t max,
                       int32_t* count);

/* ---- Woodcock gamma tracking in a layered box ----------------------------- */
/* A box |x| <= half_x, |y| <= half_y, z_bounds[0] <= z <= z_bounds[n_layers],
 * made of n_layers slabs along z with couples layer_imc[] (device arrays).
 * wdt_imc is the couple of the heaviest material: its total macroscopic cross
 * section is the Woodcock reference.  Gammas above energy_limit are
 * Woodcock-tracked through the box as G4HepEmWoodcockHelper::KeepTracking
 * does (G4HepEm/G4HepEm/src/G4HepEmWoodcockHelper.cc:146-299): steps of
 * -ln(u) times the reference mean free path, at each point an interaction
 * with probability sigma(point's material)/sigma(reference) (certain in the
 * reference material), until an interaction or 1e-3 mm before the box
 * boundary; the interaction is then selected and performed as in
 * G4HepEmTrackingManager (G4HepEm/G4HepEm/src/G4HepEmTrackingManager.cc:
 * 1000-1110).  Gammas at or below energy_limit make one ordinary HowFar +
 * interaction step in their current layer.  Positions (device, in/out) move
 * by the step; imc becomes the couple at the new position; nia0 is reset.
 * reached_boundary[i] (device, may be NULL) = 1 when the box boundary ended
 * the Woodcock step.  Non-gamma tracks are flagged (flags & 4). */
typedef struct hepem_layered_box {
  double half_x, half_y;        /* transverse half widths [mm]                  */
  int32_t n_layers;
  int32_t wdt_imc;               /* couple of the Woodcock reference material    */
  const double* z_bounds;        /* [n_layers + 1], increasing [mm], device      */
  const int32_t* layer_imc;      /* [n_layers], device                           */
  double energy_limit;           /* Woodcock tracking above this energy [MeV]    */
} hepem_layered_box;
int  hepem_woodcock_gamma(const hepem_ctx* ctx, int64_t n, const hepem_track_state* in,
                          hepem_track_state* out, double* pos_x, double* pos_y, double* pos_z,
                          const hepem_layered_box* box, const double* uniforms, int32_t n_uniform,
                          uint64_t seed, hepem_step_out* res, uint8_t* reached_boundary,
                          void* stream);

/* ---- secondary stacking with production cuts ------------------------------ */
/* Turns the secondaries of a step (res, after hepem_step*) into fresh tracks
 * for the next step, in parent order (parent i: slot 0, then slot 1): type,
 * energy and direction of the secondary, the parent's couple and safety, id =
 * id_base + position, and the ReSet() state of a new track.  With apply_cuts
 * an e- below the couple's electron production cut, an e+ below the positron
 * cut (when m_e c^2 is below the gamma cut) and a gamma below the gamma cut
 * are not stacked; their energy (e+: E + 2 m_e c^2) goes to edep_cut[i]
 * (device, n entries, may be NULL).  *n_out (device) receives the number of
 * stacked secondaries; at most `capacity` of them are written.  Replaces
 * G4HepEmTrackingManager::StackSecondaries
 * (G4HepEm/G4HepEm/src/G4HepEmTrackingManager.cc:1254-1330). */
int  hepem_stack_secondaries(const hepem_ctx* ctx, int64_t n, const hepem_track_state* parents,
                             const hepem_step_out* res, int apply_cuts, int32_t id_base,
                             hepem_track_state* out, int64_t capacity, int64_t* n_out,
                             double* edep_cut, void* stream);

/* ---- per-model sampling ---------------------------------------------------- */
/* n independent draws of one interaction model for a particle of kinetic
 * energy ekin in couple imc (direction +z; draw i uses the pure Philox stream
 * of (seed, id = i)).  out[i] = the sampled energy: model 0 Seltzer-Berger and
 * 1 relativistic brem (e-): the photon energy; 2 Moller (e-) and 3 Bhabha (e+):
 * the delta-ray energy; 4 Klein-Nishina Compton: the scattered photon energy;
 * 5 Bethe-Heitler pair production: the electron kinetic energy (0 when the
 * model produces nothing, e.g. below its threshold).  precision 0: the FP64
 * models of hepem_step; 1: the FP32 models of hepem_step_mixed, where a draw
 * that trips a guard is redone in FP64 (*n_fallback, a device counter, may
 * be NULL).  Replaces the direct calls of the reference's unit tests, e.g.
 * G4HepEmElectronInteractionBrem::SampleETransferSB
 * (G4HepEm/G4HepEmRun/include/G4HepEmElectronInteractionBrem.hh) as called
 * from testElectronInteractionBrem/src/Implementation.cc:268-272. */
int  hepem_sample_model(const hepem_ctx* ctx, int model, int precision, int64_t n,
                        double ekin, int32_t imc, uint64_t seed, double* out,
                        uint64_t* n_fallback, void* stream);

/* ---- launch configuration of the batched form and its autotuner ---------- */
/* The batched form runs eleven stage kernels (index: 0 e+- stage A, 1 gamma
 * stage A, 2..10 the interaction kernels in the order of hepem_stage_times).
 * Each runs with 128, 256 or 512 threads per block and 1..occupancy CTAs per
 * SM; e+- tracks are sorted into 8, 16 or 32 energy bins per couple.  Results
 * do not depend on the configuration (bit-identical).  No reference
 * counterpart: the reference has no batched form. */
typedef struct hepem_launch_config {
  int32_t block[11];          /* threads per block: 128, 256 or 512            */
  int32_t ctas_per_sm[11];    /* 0 = as many as fit                            */
  int32_t sort_energy_bins;   /* 8, 16 or 32                                   */
  float   ms[11];             /* per-kernel time found by hepem_autotune       */
} hepem_launch_config;
int  hepem_get_launch_config(const hepem_ctx* ctx, hepem_launch_config* out);
/* cfg NULL restores the default (256 threads, occupancy grid, 32 bins).  Set
 * it before the context is shared between threads. */
int  hepem_set_launch_config(hepem_ctx* ctx, const hepem_launch_config* cfg);
/* L2 residency of the tables for the batched forms (hepem_step_batched,
 * hepem_step_mixed, the host-buffer steps, the server): enable != 0 sets an
 * L2 access-policy window over the context's table arena on every stage
 * kernel launch (table gathers persisting, up to the device's persisting L2
 * set-aside, which this raises for the process's context to the arena size
 * at most), so the streamed track state does not evict the tables; 0 clears
 * it.  New contexts start without it: on a GB300 it made the precision-form
 * step 4-5% slower and left the FP64 batched step unchanged (the tables, a
 * few hundred KB to a few MB, stay cached without it).  *window_bytes (may be NULL) = the window's size (0: none, e.g. the device
 * has no persisting L2).  Results do not depend on it.  Set it before the
 * context is shared between threads.  No reference counterpart: the
 * reference reads its tables through the ordinary caches
 * (G4HepEm/G4HepEmData/src/G4HepEmData.cc:78-101 copies them to the device). */
int  hepem_set_table_l2_window(hepem_ctx* ctx, int enable, int64_t* window_bytes);
/* Times the FP64 batched step on the caller's batch (device pointers; the
 * batch is read, outputs go to scratch) under every candidate configuration,
 * kernel by kernel, then the whole step with the choice against the default
 * configuration, and returns the faster of the two in `out`; apply != 0 also
 * makes it the context's configuration.  Synchronises the stream. */
int  hepem_autotune(hepem_ctx* ctx, int64_t n, const hepem_track_state* in,
                    const double* uniforms, int32_t n_uniform, uint64_t seed,
                    int apply, hepem_launch_config* out, void* stream);

/* ---- RNG stream helpers --------------------------------------------------- */
/* Philox4x32-10 (Salmon et al., SC'11) uniform in (0,1): counter
 * (k>>1, id, 0, 0x48455045), key (seed lo, seed hi); 52 random bits. */
double hepem_philox_uniform(uint64_t seed, int32_t id, int32_t k);
/* Fill uniforms[i*n_uniform + k] = hepem_philox_uniform(seed, id[i], k) on the
 * device (ids: device pointer). */
int  hepem_fill_uniforms(int64_t n, const int32_t* id, int32_t n_uniform,
                         uint64_t seed, double* uniforms, void* stream);

/* ---- serving form: continuous batching of event requests ------------------- */
/* A request is one event's track batch (host SoA).  The server keeps the
 * tracks of admitted requests resident on the device, steps all of them in
 * one batched step per iteration (requests that arrive while others run join
 * the next iteration), and retires a request when none of its tracks is above
 * min_energy or after max_steps iterations.  Admission is first-come
 * first-served by the memory budget: a request waits until a contiguous slot
 * range of its size is free.  Each track draws pure Philox uniforms keyed by
 * the request's seed and the track's id, and every per-request sum is reduced
 * in a fixed order, so a request's result does not depend on the mix.
 * Reference counterpart: the per-event stepping loop of the TestEm3 tracking
 * (apps/examples/TestEm3/src/G4HepEmProcess.cc:144-197 called per step by
 * Geant4), here for many events at once; the reference has no server. */
typedef struct hepem_server hepem_server;

typedef struct hepem_server_config {
  int64_t memory_budget_bytes;  /* device memory for resident tracks + workspace */
  int32_t max_steps;            /* step budget of a request (iterations)         */
  int32_t max_requests;         /* requests resident at once                     */
  double  min_energy;           /* a track is alive while ekin > min_energy (MeV) */
  int32_t precision;            /* 0: FP64 batched form, 1: precision form       */
  int32_t reserved;             /* 0                                             */
} hepem_server_config;

typedef struct hepem_request_result {
  int64_t n_tracks;
  int32_t steps;                /* iterations the request took part in          */
  int32_t status;               /* HEPEM_OK, HEPEM_CANCELLED or HEPEM_CUDA_ERROR */
  double  edep;                 /* sum of deposited energy over tracks and steps */
  double  e_secondaries;        /* sum of secondary kinetic energies             */
  int64_t n_secondaries;
  int64_t track_steps;          /* sum over tracks of the steps taken            */
  double  t_submit, t_admit, t_done;  /* steady-clock seconds                    */
} hepem_request_result;

typedef struct hepem_server_stats {
  int64_t iterations, track_steps, completed, waiting, active, free_slots;
  double  batch_ms_p50, batch_ms_p99;  /* wall time of one iteration            */
} hepem_server_stats;

/* Starts the server thread; capacity (tracks) follows from the budget. */
int  hepem_server_create(const hepem_ctx* ctx, const hepem_server_config* cfg,
                         hepem_server** out);
int  hepem_server_capacity(const hepem_server* s, int64_t* tracks);
/* Copies the batch; HEPEM_OOM_ADMISSION if n exceeds the whole capacity. */
int  hepem_server_submit(hepem_server* s, int64_t n, const hepem_track_state* tracks,
                         uint64_t seed, int64_t* request_id);
/* done = 1 when finished; then result (and, if not NULL, the final track
 * state, host arrays of n) are filled and the request is forgotten. */
int  hepem_server_poll(hepem_server* s, int64_t request_id, int32_t* done,
                       hepem_request_result* result, hepem_track_state* final_tracks);
/* Waits at most timeout_s seconds (HEPEM_TIMEOUT otherwise), then as poll. */
int  hepem_server_wait(hepem_server* s, int64_t request_id, double timeout_s,
                       hepem_request_result* result, hepem_track_state* final_tracks);
/* A waiting request finishes at once; an admitted one at the next iteration;
 * either way with status HEPEM_CANCELLED. */
int  hepem_server_cancel(hepem_server* s, int64_t request_id);
int  hepem_server_get_stats(hepem_server* s, hepem_server_stats* out);
int  hepem_server_reset_stats(hepem_server* s);
/* Snapshot of the unfinished requests (waiting or resident), taken between
 * two iterations: each request's track state as of its last completed step,
 * its per-track sums (deposit, secondary energy and count, steps) and its
 * step count, with a checksum.  buf == NULL: *size = the bytes needed.  The
 * requests keep running on this server.  Reference counterpart: none (the
 * reference saves only the Geant4 RNG status, apps/examples/TestEm3/src/
 * RunAction.cc:103); the state is plain SoA plus RNG cursors, so a snapshot
 * is a copy. */
int  hepem_server_snapshot(hepem_server* s, void* buf, size_t capacity, size_t* size);
/* Validates a snapshot without a GPU; counts its requests and tracks. */
int  hepem_server_snapshot_check(const void* buf, size_t size, int64_t* n_requests,
                                 int64_t* n_tracks);
/* Submits the requests of a snapshot to server s (built on the same tables):
 * each resumes where it stopped and ends with the result it would have had
 * without the interruption.  old_ids[k] / new_ids[k] (arrays of max_ids) map
 * the snapshot's request ids to this server's; *n_requests = the count
 * (HEPEM_BAD_ARG, nothing submitted, if it is above max_ids). */
int  hepem_server_resume(hepem_server* s, const void* buf, size_t size, int64_t max_ids,
                         int64_t* old_ids, int64_t* new_ids, int64_t* n_requests);
/* Stops the thread after the current iteration and frees the pool. */
int  hepem_server_destroy(hepem_server* s);

#ifdef __cplusplus
}
#endif

#endif /* G4HEPEM_GB300_H */
