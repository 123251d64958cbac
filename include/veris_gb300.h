/*
 * veris_gb300.h - C ABI of the GB300 sea-ice step.
 *
 * One GPU, device pointers only.  Every entry point:
 *   - takes the grid (VerisGrid), the settings (VerisParams) and the state
 *     fields (VerisFieldsF64 / VerisFieldsF32: one device pointer per state
 *     variable, named as the plugin's variables, veris/variables.py:7-105);
 *   - writes its results into caller-allocated device arrays of the same
 *     2-D shape (functional style: inputs are never modified, as the
 *     reference's kernels return new arrays);
 *   - allocates nothing: scratch space is passed in as a workspace whose
 *     size the matching *_workspace_bytes() function returns;
 *   - enqueues its kernels on the given CUDA stream and returns a status
 *     code without synchronising.
 *
 * Arrays are 2-D, (nx + 2*olx) x (ny + 2*oly), x-major (y contiguous), with a
 * row pitch of `ld` elements.  Halos are 2 cells wide (olx = oly = 2, the
 * plugin's default, veris/settings.py:9-10).  Neighbour access wraps
 * periodically over the padded array in both axes, as the reference's
 * `roll` does; the halo fill (veris/fill_overlap.py) then refreshes the
 * halos where the reference does.
 *
 * Each declaration names the reference routine it replaces (file:line in
 * team-ocean/veris).
 */
#ifndef VERIS_GB300_H
#define VERIS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* a cudaStream_t; NULL is the legacy default stream */
typedef void *veris_stream_t;

enum VerisStatus {
    VERIS_OK = 0,
    VERIS_ERR_SHAPE = 1,       /* bad grid sizes, halo widths or pitch */
    VERIS_ERR_ALIGN = 2,       /* a pointer or pitch breaks an alignment rule */
    VERIS_ERR_NAN = 3,         /* a non-finite value was detected */
    VERIS_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
    VERIS_ERR_LAUNCH = 5,      /* a CUDA launch or API call failed */
    VERIS_ERR_ARG = 6,         /* a NULL pointer or an invalid argument */
    VERIS_ERR_UNSUPPORTED = 7, /* settings this entry point does not cover */
    VERIS_ERR_WORKSPACE = 8,   /* workspace missing or too small */
    VERIS_ERR_TOO_LARGE = 9    /* grid larger than a fixed-size entry point's scratch */
};

typedef struct {
    int32_t nx, ny;   /* interior size */
    int32_t olx, oly; /* halo widths (must be 2) */
    int64_t ld;       /* elements between x and x+1; >= ny + 2*oly */
} VerisGrid;

/*
 * Settings (veris/settings.py:4-176) as a flat POD struct.  The fields
 * marked "derived" are computed by the host from other settings exactly as
 * the reference computes them in Python, so that both sides round alike.
 */
#define VERIS_PARAM_DOUBLES(X)                                                        \
    X(deltatTherm) X(recip_deltatTherm) X(deltatDyn) X(recip_deltatDyn)               \
    X(evpAlpha) X(evpBeta) X(aEVPalphaMin) X(EVPcFac)                                 \
    X(rhoIce) X(rhoFresh) X(rhoSea) X(rhoAir) X(rhoSnow)                              \
    X(recip_rhoFresh) X(recip_rhoSea) X(rhoIce2rhoSnow) X(rhoIce2rhoFresh)            \
    X(rhoFresh2rhoSnow)                                                               \
    X(dryIceAlb) X(dryIceAlb_south) X(wetIceAlb) X(wetIceAlb_south)                   \
    X(drySnowAlb) X(drySnowAlb_south) X(wetSnowAlb) X(wetSnowAlb_south)               \
    X(wetAlbTemp) X(lhFusion) X(lhEvap) X(lhSublim) X(cpAir) X(cpWater)               \
    X(stefBoltz) X(iceEmiss) X(snowEmiss) X(iceConduct) X(snowConduct) X(hCut)        \
    X(shortwave) X(tempFrz) X(dtempFrz_dS) X(saltIce_ref) X(minLWdown) X(minTIce)    \
    X(minTAir) X(dalton) X(Area_reg) X(hIce_reg) X(celsius2K) X(stantonNr)            \
    X(uStarBase) X(McPheeTaperFac) X(recip_h0) X(recip_h0_south) X(recip_nITC)        \
    X(sinWin) X(cosWin) X(sinWat) X(cosWat) X(sinWatOcn) X(cosWatOcn)                 \
    X(wSpeedMin) X(hIce_min) X(Area_min) X(airIceDrag) X(airIceDrag_south)            \
    X(waterIceDrag) X(waterIceDrag_south) X(cDragMin) X(seaIceLoadFac) X(gravity)     \
    X(PlasDefCoeff) X(deltaMin) X(pressReplFac) X(pStar) X(cStar)                     \
    X(basalDragU0) X(basalDragK1) X(basalDragK2) X(cBasalStar) X(tensileStrFac)       \
    X(CrMax) X(sideDragCoeff) X(sideDragU0)                                           \
    X(s4t_cc0) X(s4t_cc1) X(s4t_cc2) X(s4t_d1) X(s4t_d1i)                              \
    X(zvir) X(cpdair) X(karman) X(latvap) X(ocean_emissivity) X(gamma_blk) X(grav)

#define VERIS_PARAM_INTS(X)                                                           \
    X(nITC) X(noSlip) X(secondOrderBC) X(useRelativeWind) X(useRealFreshWaterFlux)    \
    X(useAdaptiveEVP) X(veros_fill) X(enable_cyclic_x) X(use_coastline)              \
    X(extensiveFld) X(nEVPsteps) X(pad_)

#define VERIS_DECL_DOUBLE(name) double name;
#define VERIS_DECL_INT(name) int32_t name;
typedef struct {
    VERIS_PARAM_DOUBLES(VERIS_DECL_DOUBLE)
    VERIS_PARAM_INTS(VERIS_DECL_INT)
} VerisParams;

/* State variables carried by VerisFields*, in ABI order. */
#define VERIS_FIELDS(X)                                                               \
    X(hIceMean) X(hSnowMean) X(Area) X(TSurf) X(uIce) X(vIce)                         \
    X(sigma1) X(sigma2) X(sigma12)                                                    \
    X(SeaIceMassC) X(SeaIceMassU) X(SeaIceMassV) X(SeaIceStrength)                    \
    X(AreaW) X(AreaS) X(WindForcingX) X(WindForcingY)                                 \
    X(os_hIceMean) X(os_hSnowMean) X(recip_hIceMean) X(SeaIceLoad) X(IcePenetSW)      \
    X(OceanStressU) X(OceanStressV) X(forc_salt_surface_ice)                          \
    X(uOcean) X(vOcean) X(theta) X(ocSalt) X(Qnet) X(Qsw) X(ssh_an) X(R_low)           \
    X(uWind) X(vWind) X(wSpeed) X(surfPress) X(SWdown) X(LWdown) X(ATemp) X(aqh)      \
    X(precip) X(snowfall) X(evap) X(runoff) X(EmPmR) X(saltflux)                      \
    X(maskInC) X(maskInU) X(maskInV) X(iceMask) X(iceMaskU) X(iceMaskV)               \
    X(k1AtC) X(k2AtC) X(k1AtZ) X(k2AtZ) X(Fu) X(Fv) X(fCori)                          \
    X(dxC) X(dyC) X(dxG) X(dyG) X(dxU) X(dyU) X(dxV) X(dyV)                           \
    X(recip_dxC) X(recip_dyC) X(recip_dxG) X(recip_dyG)                               \
    X(recip_dxU) X(recip_dyU) X(recip_dxV) X(recip_dyV)                               \
    X(rA) X(rAu) X(rAv) X(rAz) X(recip_rA) X(recip_rAu) X(recip_rAv) X(recip_rAz)

#define VERIS_DECL_F64(name) const double *name;
#define VERIS_DECL_F32(name) const float *name;
typedef struct { VERIS_FIELDS(VERIS_DECL_F64) } VerisFieldsF64;
typedef struct { VERIS_FIELDS(VERIS_DECL_F32) } VerisFieldsF32;

/* ---- introspection (lets a binding check its struct layouts) ---------- */
size_t veris_params_size(void);
size_t veris_fields_count(void);
const char *veris_field_name(size_t index);
const char *veris_status_string(int status);
/* 1 when the library was built for sm_103a and a device of that kind is usable */
int veris_device_ok(void);

/* ---- halo fill -------------------------------------------------------- */
/* veris/fill_overlap.py:6-18 fill_overlap(state, A): in place on A */
int veris_fill_overlap_f64(const VerisGrid *g, const VerisParams *p, double *A,
                           veris_stream_t s);
int veris_fill_overlap_f32(const VerisGrid *g, const VerisParams *p, float *A,
                           veris_stream_t s);

/* ---- dynamics preparation (once per step) ---------------------------- */
/* veris/area_mass.py:17-28 SeaIceMass */
int veris_sea_ice_mass_f64(const VerisGrid *g, const VerisParams *p,
                           const VerisFieldsF64 *vs, double *SeaIceMassC,
                           double *SeaIceMassU, double *SeaIceMassV, veris_stream_t s);
/* veris/area_mass.py:5-14 AreaWS */
int veris_area_ws_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                      double *AreaW, double *AreaS, veris_stream_t s);
/* veris/dynsolver.py:7-47 tauXY */
int veris_tau_xy_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                     double *tauX, double *tauY, veris_stream_t s);
/* veris/dynsolver.py:50-84 WindForcingXY */
int veris_wind_forcing_xy_f64(const VerisGrid *g, const VerisParams *p,
                              const VerisFieldsF64 *vs, double *WindForcingX,
                              double *WindForcingY, veris_stream_t s);
/* veris/dynamics_routines.py:5-18 SeaIceStrength */
int veris_sea_ice_strength_f64(const VerisGrid *g, const VerisParams *p,
                               const VerisFieldsF64 *vs, double *SeaIceStrength,
                               veris_stream_t s);

/* ---- EVP building blocks (the inner routines, for parity and reuse) -- */
/* veris/dynamics_routines.py:143-217 strainrates(state, uIce, vIce) */
int veris_strainrates_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                          const double *uIce, const double *vIce, double *e11, double *e22,
                          double *e12, veris_stream_t s);
/* veris/dynamics_routines.py:220-268 viscosities(state, e11, e22, e12) */
int veris_viscosities_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                          const double *e11, const double *e22, const double *e12,
                          double *zeta, double *eta, double *press, veris_stream_t s);
/* veris/averaging.py:4-19 c_point_to_z_point(state, Cfield, noSlip) */
int veris_c_point_to_z_point_f64(const VerisGrid *g, const VerisParams *p,
                                 const VerisFieldsF64 *vs, const double *Cfield,
                                 int32_t noSlip, double *Zfield, veris_stream_t s);
/* veris/dynamics_routines.py:21-52 ocean_drag_coeffs(state, uIce, vIce) */
int veris_ocean_drag_coeffs_f64(const VerisGrid *g, const VerisParams *p,
                                const VerisFieldsF64 *vs, const double *uIce,
                                const double *vIce, double *cDrag, veris_stream_t s);
/* veris/dynamics_routines.py:55-96 basal_drag_coeffs(state, uIce, vIce) */
int veris_basal_drag_coeffs_f64(const VerisGrid *g, const VerisParams *p,
                                const VerisFieldsF64 *vs, const double *uIce,
                                const double *vIce, double *cBot, veris_stream_t s);
/* veris/dynamics_routines.py:99-140 side_drag(state, uIce, vIce) */
int veris_side_drag_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                        const double *uIce, const double *vIce, double *SideDragU,
                        double *SideDragV, veris_stream_t s);
/* veris/dynamics_routines.py:284-303 stressdiv(state, sig11, sig22, sig12) */
int veris_stressdiv_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                        const double *sig11, const double *sig22, const double *sig12,
                        double *stressDivX, double *stressDivY, veris_stream_t s);

/* ---- the EVP solver (the hot loop) ----------------------------------- */
/*
 * veris/evp_solver.py:257-319 evp_solver(state) and its loop body :21-254:
 * `n_subcycles` mEVP subcycles starting from vs->uIce, vIce, sigma1, sigma2,
 * sigma12 (which are also u^{n-1}, v^{n-1}); results in the five outputs.
 * Plain form: one tiled kernel per subcycle, halo fill fused into it.
 */
size_t veris_evp_workspace_bytes(const VerisGrid *g, int32_t elem_size);
int veris_evp_solver_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                         int32_t n_subcycles, double *uIce, double *vIce, double *sigma1,
                         double *sigma2, double *sigma12, void *workspace,
                         size_t workspace_bytes, veris_stream_t s);
int veris_evp_solver_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF32 *vs,
                         int32_t n_subcycles, float *uIce, float *vIce, float *sigma1,
                         float *sigma2, float *sigma12, void *workspace,
                         size_t workspace_bytes, veris_stream_t s);

/*
 * The same loop with the residual diagnostics of veris/evp_solver.py:193-234
 * (settings.computeEvpResidual), as that branch means them: after subcycle
 * k, over the interior,
 *   resSig[k] = sum (d sig11 alphaC iceMask)^2 + (d sig22 alphaC iceMask)^2
 *               + (d sigma12 alphaZ)^2,  sig11/22 = (sigma1 +- sigma2) / 2
 *   resU[k]   = sum (iceMaskU d uIce betaU)^2 + (iceMaskV d vIce betaV)^2
 * (d: the change over the subcycle; alpha, beta: those of that subcycle,
 * adaptive or constant).  resU, resSig: n_subcycles doubles of device
 * memory.  The sums are float64 and deterministic (fixed reduction order).
 */
size_t veris_evp_residual_workspace_bytes(const VerisGrid *g, int32_t elem_size,
                                          int32_t n_subcycles);
int veris_evp_residual_solver_f64(const VerisGrid *g, const VerisParams *p,
                                  const VerisFieldsF64 *vs, int32_t n_subcycles, double *uIce,
                                  double *vIce, double *sigma1, double *sigma2, double *sigma12,
                                  double *resU, double *resSig, void *workspace,
                                  size_t workspace_bytes, veris_stream_t s);
int veris_evp_residual_solver_f32(const VerisGrid *g, const VerisParams *p,
                                  const VerisFieldsF32 *vs, int32_t n_subcycles, float *uIce,
                                  float *vIce, float *sigma1, float *sigma2, float *sigma12,
                                  double *resU, double *resSig, void *workspace,
                                  size_t workspace_bytes, veris_stream_t s);

/*
 * veris/freedrift_solver.py:5-62 freedrift_solver(state): ice velocities
 * without internal stress, from WindForcingX/Y, uOcean, vOcean, hIceMean,
 * fCori, iceMaskU, iceMaskV; every padded point of uIce and vIce is written.
 * veris/dynsolver.py:93-97 selects it when settings.useFreedrift is set.
 */
int veris_freedrift_solver_f64(const VerisGrid *g, const VerisParams *p,
                               const VerisFieldsF64 *vs, double *uIce, double *vIce,
                               veris_stream_t s);
int veris_freedrift_solver_f32(const VerisGrid *g, const VerisParams *p,
                               const VerisFieldsF32 *vs, float *uIce, float *vIce,
                               veris_stream_t s);

/*
 * veris/heat_flux_MITgcm.py:5-123 bulkf_formula_lanl(state, uw, vw, ta, qa,
 * tsf, ocn_mask): bulk fluxes over open ocean at n points (any layout: the
 * formula is pointwise).  Constants from p: zvir, cpdair, karman, latvap,
 * ocean_emissivity, gamma_blk, grav, rhoAir, stefBoltz.  ocn_mask is not
 * read (the reference takes only its shape) and may be NULL; a NULL output
 * is not written.
 */
int veris_bulkf_formula_lanl_f64(const VerisParams *p, int64_t n, const double *uw,
                                 const double *vw, const double *ta, const double *qa,
                                 const double *tsf, const double *ocn_mask, double *flwupa,
                                 double *flha, double *fsha, double *df0dT, double *ust,
                                 double *vst, double *evp, double *ssq, double *dEvdT,
                                 veris_stream_t s);
int veris_bulkf_formula_lanl_f32(const VerisParams *p, int64_t n, const float *uw,
                                 const float *vw, const float *ta, const float *qa,
                                 const float *tsf, const float *ocn_mask, float *flwupa,
                                 float *flha, float *fsha, float *df0dT, float *ust,
                                 float *vst, float *evp, float *ssq, float *dEvdT,
                                 veris_stream_t s);

/*
 * The same loop (veris/evp_solver.py:21-319), fast form: a prep kernel folds
 * the step constants of the float64 state into compact arrays of the
 * arithmetic type, then one shared-memory-staged kernel per subcycle.  Reads
 * the float64 field table; writes the five results in the arithmetic type.
 * Covers the default rheology: veris_evp_fast_settings_check() returns the
 * settings it does not cover (0 = all covered) and veris_evp_fast_check()
 * ORs into *violations_device the state properties it does not cover
 * (non-zero k1/k2 metric terms, masks other than 0/1, grid lengths varying
 * along both axes).  A non-zero answer means: use the plain form.  Bit 128
 * (cell areas rA, rAz, rAu, rAv varying along both axes) concerns only
 * veris_evp_walk_solver_f32 and the float32 tape, which take the areas
 * along j; the tile forms cover it.
 */
size_t veris_evp_fast_workspace_bytes(const VerisGrid *g, int32_t elem_size);
int veris_evp_fast_settings_check(const VerisParams *p);
/* the same for veris_evp_walk_solver_f32, which also runs the adaptive EVP
 * (veris/evp_solver.py:65-73, 97-100, 148-150) */
int veris_evp_walk_settings_check(const VerisParams *p);
int veris_evp_fast_check(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                         int32_t *violations_device, veris_stream_t s);
int veris_evp_fast_solver_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                              int32_t n_subcycles, float *uIce, float *vIce, float *sigma1,
                              float *sigma2, float *sigma12, void *workspace,
                              size_t workspace_bytes, veris_stream_t s);
int veris_evp_fast_solver_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                              int32_t n_subcycles, double *uIce, double *vIce, double *sigma1,
                              double *sigma2, double *sigma12, void *workspace,
                              size_t workspace_bytes, veris_stream_t s);
/*
 * Tile height of the float64 fast-form subcycle kernel (every float64 fast
 * form: solver, tapes, the adjoint's recomputed subcycles): work units of
 * at most 16, 24 or 32 output rows by 32 columns per CTA (4, 3 or 2 CTAs per
 * SM; the launch ends on a round of smaller units), 0 = the library's
 * default.  Process-wide, for every later launch; same values
 * for every height.  VERIS_ERR_ARG for other heights.  A tuning knob with no
 * counterpart in the reference.
 */
int veris_evp_f64_tile_rows(int32_t rows);
/* the float32 fast form without TMA staging (the shared-memory kernel only) */
/*
 * The same float32 loop with the register-walking kernel: one warp per
 * 28-column strip walks `rows` output rows (4..4096; 0: the longest walk
 * that keeps all walks in one wave of resident warps), rows in registers and
 * columns across lanes; no shared memory, no barriers.  `variant` (0..5)
 * picks the compiled form: register budget free (0), 5 (1) or 4 (2, 3)
 * resident 4-warp CTAs per SM, and (3) the own-point constants loaded one
 * walk step early; same values.
 */
int veris_evp_walk_solver_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                              int32_t n_subcycles, int32_t rows, int32_t variant, float *uIce,
                              float *vIce, float *sigma1, float *sigma2, float *sigma12,
                              void *workspace, size_t workspace_bytes, veris_stream_t s);
/*
 * Subcycles per launch of the register-walking float32 kernel (every float32
 * walk solve with at least 3 subcycles): 0 = one launch per subcycle, 1 =
 * all but the last subcycle in one persistent cooperative launch, each walk
 * waiting only for the walks whose rows or columns its stencil shares
 * (per-walk progress counters; a wait that gives up after about half a
 * second sets status bit 1 and ends the launch), then the last subcycle as
 * usual.  Falls back to one launch per subcycle when the walks cannot all
 * be resident at once.  Process-wide, for every later launch; same values.
 * VERIS_ERR_ARG for other values.  A tuning knob with no counterpart in the
 * reference.
 */
int veris_evp_walk_persistent(int32_t on);
int veris_evp_smem_solver_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                              int32_t n_subcycles, float *uIce, float *vIce, float *sigma1,
                              float *sigma2, float *sigma12, void *workspace,
                              size_t workspace_bytes, veris_stream_t s);
/*
 * Device status word of the last fast solve on this workspace (0 = clean;
 * bit 0: a bounded TMA wait gave up and the affected tiles were skipped;
 * bit 1: a persistent walk's bounded wait gave up and the launch ended).
 * Synchronises the stream.
 */
int veris_evp_fast_status(const void *workspace, int32_t *status_host, veris_stream_t s);
/*
 * Failure-detection probe (no counterpart in the reference): one warp waits,
 * with the TMA kernel's bounded mbarrier wait (`limit` polls, at most 2^20),
 * on an mbarrier that it arrives on (`arrive` != 0) or that nothing arrives
 * on; writes 0 or the timeout bit (1) to *status_device and returns.
 */
int veris_mbarrier_wait_probe(int32_t arrive, uint32_t limit, int32_t *status_device, veris_stream_t s);

/*
 * No counterpart in the reference: an allocation-free form of
 * veris_evp_solver_f64 for callers that cannot allocate device memory, e.g.
 * a host model's time loop driving the step through this C ABI with no
 * device allocator of its own, or running under a device-memory budget fixed
 * at start-up.  Same kernels and results as veris_evp_solver_f64; the
 * ping-pong scratch is a fixed array inside the library (VERIS_NOALLOC_MAX_CELLS
 * padded cells, (nx+4) * ld <= 262144, i.e. 10 MiB of device memory held by
 * every GPU that loads the library until the process exits).  Larger grids
 * return VERIS_ERR_TOO_LARGE without launching anything.  The first call on a
 * device looks up the scratch's device address (cudaGetSymbolAddress) with
 * that device current and keeps it for the life of the process: make that
 * first call before any stream capture, and make no call after the device's
 * primary context has been destroyed (cudaDeviceReset) -- the kept address
 * would point at the old context's memory.  Calls share the scratch: calls
 * that overlap on the GPU (different streams, or host threads) race on it
 * and must be serialised by the caller.
 */
#define VERIS_NOALLOC_MAX_CELLS 262144
int veris_evp_solver_f64_noalloc(const VerisGrid *g, const VerisParams *p,
                                 const VerisFieldsF64 *vs, int32_t n_subcycles, double *uIce,
                                 double *vIce, double *sigma1, double *sigma2, double *sigma12,
                                 veris_stream_t s);

/*
 * Adjoint of veris/evp_solver.py:257-319 (fast form, float64): given the
 * adjoints of the five outputs of n subcycles (caller pitch), writes the
 * adjoints of the five inputs (uIce, vIce, sigma1, sigma2, sigma12 at the
 * start; the uIce/vIce ones include the u^{n-1} terms), ADDS the adjoints of
 * the step-constant fields the loop reads into *lfields (a table of adjoint
 * arrays: SeaIceStrength, SeaIceMassC/U/V, WindForcingX/Y, AreaW/S,
 * uOcean/vOcean, and hIceMean/Area through the basal drag; NULL members are
 * skipped), and writes d/d waterIceDrag and d/d waterIceDrag_south to
 * lscalars[0..1].  States are checkpointed every K subcycles (K <= 0: all)
 * and recomputed segment by segment.
 */
size_t veris_evp_adjoint_workspace_bytes(const VerisGrid *g, int32_t elem_size, int32_t n_subcycles,
                                         int32_t K);
int veris_evp_adjoint_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                          int32_t n_subcycles, int32_t K, const double *l_uIce, const double *l_vIce,
                          const double *l_sigma1, const double *l_sigma2, const double *l_sigma12,
                          double *l_uIce0, double *l_vIce0, double *l_sigma10, double *l_sigma20,
                          double *l_sigma120, const VerisFieldsF64 *lfields, double *lscalars,
                          void *workspace, size_t workspace_bytes, veris_stream_t s);

/*
 * Taping forms for gradients of many steps (float64 fast form): the forward
 * keeps every subcycle in a caller buffer of veris_evp_tape_bytes() (slot k,
 * five arrays of internal pitch: uIce and vIce after k subcycles, and the
 * Delta, zeta and ocean-drag coefficient that subcycle k + 1 computes from
 * them; the stresses, which the adjoint does not read, are not kept), and
 * the adjoint reads the tape instead of recomputing the subcycles.  Same
 * values as veris_evp_fast_solver_f64 and veris_evp_adjoint_f64.
 */
size_t veris_evp_tape_bytes(const VerisGrid *g, int32_t elem_size, int32_t n_subcycles);
int veris_evp_fast_tape_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                            int32_t n_subcycles, double *uIce, double *vIce, double *sigma1,
                            double *sigma2, double *sigma12, double *tape, size_t tape_bytes,
                            void *workspace, size_t workspace_bytes, veris_stream_t s);
size_t veris_evp_adjoint_taped_workspace_bytes(const VerisGrid *g, int32_t n_subcycles);
int veris_evp_adjoint_taped_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                                int32_t n_subcycles, const double *tape, size_t tape_bytes,
                                const double *l_uIce, const double *l_vIce, const double *l_sigma1,
                                const double *l_sigma2, const double *l_sigma12, double *l_uIce0,
                                double *l_vIce0, double *l_sigma10, double *l_sigma20,
                                double *l_sigma120, const VerisFieldsF64 *lfields, double *lscalars,
                                void *workspace, size_t workspace_bytes, veris_stream_t s);

/*
 * Float32 forms of the same: the tape holds float32 states written by the
 * register-walking float32 kernel (the engine's float32 forward), eight
 * arrays per slot: the walk's (uIce, vIce, sigma1, sigma2) per point over
 * four arrays and sigma12 after k subcycles, then the Delta, zeta and
 * ocean-drag coefficient the walk computed in subcycle k + 1 (constant
 * alpha; the walk's own values, which the adjoint's gather passes read
 * instead of recomputing them).  The adjoint linearises the fast form at
 * those states.  The adjoints of the five states are float32, those of the
 * constants and the drag coefficients float64.
 */
int veris_evp_fast_tape_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                            int32_t n_subcycles, float *uIce, float *vIce, float *sigma1,
                            float *sigma2, float *sigma12, float *tape, size_t tape_bytes,
                            void *workspace, size_t workspace_bytes, veris_stream_t s);
int veris_evp_adjoint_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                          int32_t n_subcycles, int32_t K, const float *l_uIce, const float *l_vIce,
                          const float *l_sigma1, const float *l_sigma2, const float *l_sigma12,
                          float *l_uIce0, float *l_vIce0, float *l_sigma10, float *l_sigma20,
                          float *l_sigma120, const VerisFieldsF64 *lfields, double *lscalars,
                          void *workspace, size_t workspace_bytes, veris_stream_t s);
size_t veris_evp_adjoint_taped_workspace_bytes_f32(const VerisGrid *g, int32_t n_subcycles);
/*
 * Form of the float32 EVP adjoint subcycle: 0 by grid size (the gather
 * passes from 2^16 padded cells up when reading a tape, from 2^19 when
 * recomputing a segment, where they are memory-bound; below, one tile
 * kernel per subcycle, which beats three to five latency-bound launches),
 * 1 the tile kernel, 2 the gather passes (without a turning angle the last
 * pass of each subcycle runs fused with the first of the subcycle before
 * it), 3 the gather passes each in its own launch (the same values as 2, bit
 * for bit, but for the order of the per-warp drag sums' atomics).
 * Process-wide, for every later call; the tile kernel and the passes agree
 * to float32 rounding.  VERIS_ERR_ARG for other values.
 */
int veris_evp_adjoint_f32_form(int32_t form);
int veris_evp_adjoint_taped_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                                int32_t n_subcycles, const float *tape, size_t tape_bytes,
                                const float *l_uIce, const float *l_vIce, const float *l_sigma1,
                                const float *l_sigma2, const float *l_sigma12, float *l_uIce0,
                                float *l_vIce0, float *l_sigma10, float *l_sigma20, float *l_sigma120,
                                const VerisFieldsF64 *lfields, double *lscalars, void *workspace,
                                size_t workspace_bytes, veris_stream_t s);

/* veris/ocean_stress.py:8-40 OceanStressUV */
int veris_ocean_stress_uv_f64(const VerisGrid *g, const VerisParams *p,
                              const VerisFieldsF64 *vs, double *OceanStressU,
                              double *OceanStressV, veris_stream_t s);

/* ---- advection -------------------------------------------------------- */
/* veris/advection.py:170-175 limiter(Cr), elementwise over n values */
int veris_limiter_f64(const double *Cr, double *phi, int64_t n, veris_stream_t s);
/* veris/advection.py:94-129 calc_ZonalFlux(state, field, uTrans) */
int veris_calc_zonal_flux_f64(const VerisGrid *g, const VerisParams *p,
                              const VerisFieldsF64 *vs, const double *field,
                              const double *uTrans, double *ZonalFlux, veris_stream_t s);
/* veris/advection.py:132-167 calc_MeridionalFlux(state, field, vTrans) */
int veris_calc_meridional_flux_f64(const VerisGrid *g, const VerisParams *p,
                                   const VerisFieldsF64 *vs, const double *field,
                                   const double *vTrans, double *MeridionalFlux,
                                   veris_stream_t s);
/* veris/advection.py:28-91 calc_Advection(state, field) */
size_t veris_advection_workspace_bytes(const VerisGrid *g, int32_t elem_size);
int veris_calc_advection_f64(const VerisGrid *g, const VerisParams *p,
                             const VerisFieldsF64 *vs, const double *field, double *out,
                             void *workspace, size_t workspace_bytes, veris_stream_t s);
/* veris/advection.py:15-25 Advection(state): hIceMean, hSnowMean, Area */
int veris_advection_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                        double *hIceMean, double *hSnowMean, double *Area, void *workspace,
                        size_t workspace_bytes, veris_stream_t s);
/* the same in float32 arithmetic, on a float32 field table */
int veris_advection_f32(const VerisGrid *g, const VerisParams *p, const VerisFieldsF32 *vs,
                        float *hIceMean, float *hSnowMean, float *Area, void *workspace,
                        size_t workspace_bytes, veris_stream_t s);
/* veris/clean_up.py:5-39 clean_up_advection(state) */
int veris_clean_up_advection_f64(const VerisGrid *g, const VerisParams *p,
                                 const VerisFieldsF64 *vs, double *hIceMean,
                                 double *hSnowMean, double *Area, double *TSurf,
                                 double *os_hIceMean, double *os_hSnowMean, veris_stream_t s);
/* veris/clean_up.py:42-47 ridging(state) */
int veris_ridging_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                      double *Area, veris_stream_t s);

/* ---- thermodynamics (float64 throughout) ------------------------------ */
/* veris/solve4temp.py:5-174 solve4temp(state, hIceActual, hSnowActual, TSurfIn, TempFrz) */
int veris_solve4temp_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                         const double *hIceActual, const double *hSnowActual,
                         const double *TSurfIn, const double *TempFrz, double *TSurfOut,
                         double *F_io_net, double *F_ia_net, double *IcePenetSW,
                         double *FWsublim, veris_stream_t s);
/* veris/growth.py:8-397 Growth(state): the eleven outputs in the reference's order */
int veris_growth_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                     double *hIceMean, double *hSnowMean, double *Area, double *TSurf,
                     double *EmPmR, double *forc_salt_surface, double *Qsw, double *Qnet,
                     double *SeaIceLoad, double *IcePenetSW, double *recip_hIceMean,
                     veris_stream_t s);
/*
 * The same on the padded rows [row_begin, row_end) only (Growth is
 * pointwise): a host exchange downloads the rows one launch finished while
 * the next launch computes.  veris_growth_f64 is rows [0, nx+2*olx).
 */
int veris_growth_rows_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                          double *hIceMean, double *hSnowMean, double *Area, double *TSurf,
                          double *EmPmR, double *forc_salt_surface, double *Qsw, double *Qnet,
                          double *SeaIceLoad, double *IcePenetSW, double *recip_hIceMean,
                          int32_t row_begin, int32_t row_end, veris_stream_t s);

/* ---- adjoints of the step's other routines (float64) ------------------ */
/*
 * Each takes the adjoints of its routine's outputs and the table of the
 * routine's INPUT state (the same vs its forward call read); the Jacobians
 * are evaluated at that state, branches (limiters, clipping, masks, the
 * solve4temp Newton iterations) following the values as in the forward.
 */
/* transpose of veris/fill_overlap.py:6-18: lam_out = F^T lam_in (out of place) */
int veris_fill_overlap_adjoint_f64(const VerisGrid *g, const VerisParams *p,
                                   const double *lam_in, double *lam_out, veris_stream_t s);
/*
 * Adjoint of veris/advection.py:15-91 Advection(state) for hIceMean,
 * hSnowMean and Area.  l_* are the adjoints of the three outputs; the
 * adjoints of the three inputs are ADDED into lin_* and those of uIce and
 * vIce (through the transports and the Courant numbers) into l_u, l_v.
 */
size_t veris_advection_adjoint_workspace_bytes(const VerisGrid *g);
int veris_advection_adjoint_f64(const VerisGrid *g, const VerisParams *p,
                                const VerisFieldsF64 *vs, const double *l_hIceMean,
                                const double *l_hSnowMean, const double *l_Area,
                                double *lin_hIceMean, double *lin_hSnowMean, double *lin_Area,
                                double *l_uIce, double *l_vIce, void *workspace,
                                size_t workspace_bytes, veris_stream_t s);
/*
 * Adjoint of veris/clean_up.py:5-47 (clean_up_advection then ridging) for
 * (hIceMean, hSnowMean, Area, TSurf): writes J^T l into o_*.
 */
int veris_cleanup_adjoint_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                              const double *l_hIceMean, const double *l_hSnowMean,
                              const double *l_Area, const double *l_TSurf, double *o_hIceMean,
                              double *o_hSnowMean, double *o_Area, double *o_TSurf,
                              veris_stream_t s);
/*
 * Adjoint of veris/growth.py:8-397 Growth(state) for the ice state
 * (hIceMean, hSnowMean, Area, TSurf) in -> out: writes J^T l into o_*.
 * The forcing fields of vs (Qnet, Qsw, ...) must hold the values the
 * forward call read.
 */
int veris_growth_adjoint_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                             const double *l_hIceMean, const double *l_hSnowMean,
                             const double *l_Area, const double *l_TSurf, double *o_hIceMean,
                             double *o_hSnowMean, double *o_Area, double *o_TSurf,
                             veris_stream_t s);
/*
 * Adjoint of the dynamics preparation: veris/area_mass.py:5-28 SeaIceMass and
 * AreaWS, veris/dynsolver.py:7-84 WindForcingXY (with tauXY) and
 * veris/dynamics_routines.py:5-18 SeaIceStrength, for useRealFreshWaterFlux
 * off.  *lprep holds the adjoints of SeaIceStrength, SeaIceMassC/U/V, AreaW/S
 * and WindForcingX/Y; the adjoints of hIceMean, hSnowMean, Area, uIce and vIce
 * are ADDED into l_*, and d/d pStar, d/d airIceDrag and d/d airIceDrag_south
 * into scalars[0..2].
 */
size_t veris_prep_adjoint_workspace_bytes(const VerisGrid *g);
int veris_prep_adjoint_f64(const VerisGrid *g, const VerisParams *p, const VerisFieldsF64 *vs,
                           const VerisFieldsF64 *lprep, double *l_hIceMean, double *l_hSnowMean,
                           double *l_Area, double *l_uIce, double *l_vIce, double *scalars,
                           void *workspace, size_t workspace_bytes, veris_stream_t s);

/* ---- batched ensemble (float32 fast form) ----------------------------- */
/*
 * n independent domains of uneven sizes (grids[0..n-1], one VerisParams for
 * all) advanced together: per subcycle ONE launch of a persistent kernel
 * whose CTAs pull tiles from a global work queue over all members' tiles
 * (veris/evp_solver.py:21-254 per member, the fast form's arithmetic, so a
 * member's values equal the single-domain shared-memory form's).  The caller
 * provides one device workspace of veris_batch_workspace_bytes().
 *   veris_batch_init            builds the member table (synchronous; call
 *                               it outside any stream capture)
 *   veris_batch_prep_member_f32 folds member m's float64 state (after the
 *                               dynamics preparation) into buffer 0
 *   veris_batch_evp_f32         n_subcycles for all members from buffer
 *                               start_buf; the result is in
 *                               start_buf ^ (n_subcycles & 1).  refold != 0
 *                               first re-forms the momentum constant from
 *                               the current velocities (a new step).  shape
 *                               picks the tile (0: 32x32, 1: 16x32, 2: 32x16,
 *                               3: 16x16 shared-memory tiles; 4-8: register
 *                               walks of 8, 16, 32, 64, 128 rows over 28
 *                               columns, one ticket per warp), blocks_per_sm the persistent
 *                               grid (0: 2 per SM, 4 for walks).  A memset and kernel launches
 *                               only: capturable in a CUDA graph.
 *   veris_batch_copy_state_f32  member m's five state arrays (buffer buf) into
 *                               caller arrays of the member's pitch
 */
size_t veris_batch_workspace_bytes(int32_t n, const VerisGrid *grids);
int veris_batch_init(int32_t n, const VerisGrid *grids, const VerisParams *p, void *workspace,
                     size_t workspace_bytes);
int veris_batch_tiles(int32_t n, const VerisGrid *grids, int32_t shape);
int veris_batch_prep_member_f32(int32_t n, const VerisGrid *grids, const VerisParams *p,
                                void *workspace, size_t workspace_bytes, int32_t m,
                                const VerisFieldsF64 *vs, veris_stream_t s);
int veris_batch_evp_f32(int32_t n, const VerisGrid *grids, const VerisParams *p, void *workspace,
                        size_t workspace_bytes, int32_t n_subcycles, int32_t start_buf,
                        int32_t refold, int32_t shape, int32_t blocks_per_sm, veris_stream_t s);
int veris_batch_copy_state_f32(int32_t n, const VerisGrid *grids, const VerisParams *p,
                               const void *workspace, size_t workspace_bytes, int32_t m,
                               int32_t buf, float *uIce, float *vIce, float *sigma1,
                               float *sigma2, float *sigma12, veris_stream_t s);

/* ---- reductions and conversions -------------------------------------- */
/*
 * veris/global_sum.py:1-4 is an identity on one process; this is the
 * deterministic float64 sum of the interior of A (fixed-order tree), written
 * to *result (device memory).  Workspace: veris_reduce_workspace_bytes().
 */
size_t veris_reduce_workspace_bytes(const VerisGrid *g);
int veris_global_sum_f64(const VerisGrid *g, const double *A, const double *weight,
                         double *result, void *workspace, size_t workspace_bytes,
                         veris_stream_t s);
/*
 * The conservation diagnostics the step's global_sum calls would feed
 * (veris/global_sum.py:1-4, called at veris/evp_solver.py:219,227; the
 * budget quantities of veris/growth.py:296-383): n (1..16) deterministic
 * float64 interior sums sum(fields[q] * weights[q]) (weights NULL, or
 * weights[q] NULL: unweighted), written to ring[slot * 16 + first + q] with
 * slot = *step_counter mod ring_steps (device memory); advance != 0 then
 * increments *step_counter.  Fixed-order trees: bitwise reproducible;
 * capturable in a CUDA graph.  Workspace: veris_budget_workspace_bytes().
 */
size_t veris_budget_workspace_bytes(void);
int veris_budget_sums_f64(const VerisGrid *g, const double *const *fields,
                          const double *const *weights, int32_t n, int32_t first,
                          double *ring, int32_t ring_steps, int32_t *step_counter,
                          int32_t advance, void *workspace, size_t workspace_bytes,
                          veris_stream_t s);
/*
 * No counterpart in the reference (NumPy carries NaN through silently):
 * ORs `flag` into *status_device (device memory, sticky: the caller clears
 * it) when any element of the n (1..8) padded arrays, halos included, is a
 * NaN or an infinity.  Asynchronous; read the word after the stream.  The
 * engine runs it once per step on its prognostic fields and reports
 * VERIS_ERR_NAN.
 */
int veris_check_finite_f64(const VerisGrid *g, const double *const *arrays, int32_t n, int32_t flag,
                           int32_t *status_device, veris_stream_t s);
int veris_check_finite_f32(const VerisGrid *g, const float *const *arrays, int32_t n, int32_t flag,
                           int32_t *status_device, veris_stream_t s);
/* elementwise precision conversion of n values */
int veris_convert_f64_to_f32(const double *src, float *dst, int64_t n, veris_stream_t s);
int veris_convert_f32_to_f64(const float *src, double *dst, int64_t n, veris_stream_t s);
/*
 * No counterpart in the reference: a self-check of the float64 division,
 * reciprocal and square roots that the float64 kernels take from the
 * hardware's approximate reciprocal and reciprocal square root refined by
 * the series of the exact correction (instead of IEEE division and square
 * root).  For n operand pairs (a, b) in device memory it writes 8 planar
 * arrays of n values to out: a/b, a/b, 1/b, 1/b, sqrt(b), sqrt(b),
 * 1/sqrt(b), 1/sqrt(b), each pair in the warp-uniform form (a warp with any
 * operand outside the safe range takes IEEE for all its lanes) and in the
 * per-lane form.  Results are within one unit in the last place of the
 * correctly rounded value (measured over 2^20 operands spanning 2^+-900);
 * zeros, denormals, negatives, infinities and NaN give the IEEE results
 * (sqrt of -0 in the warp form: +0 when the warp takes the series).
 */
int veris_f64_math_check(const double *a, const double *b, int64_t n, double *out, veris_stream_t s);

#ifdef __cplusplus
}
#endif
#endif /* VERIS_GB300_H */
