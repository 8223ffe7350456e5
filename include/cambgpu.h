/*
 * cambgpu.h -- C ABI of the GB300 scalar-perturbation library (libcambgpu.so).
 *
 * The library replaces three OpenMP call sites of the reference's
 * fortran/cmbmain.f90 with CUDA kernels for sm_103a:
 *
 *   (1) the source loop  `do q_ix ... call DoSourcek`      (cmbmain.f90:205-209)
 *       -> cambgpu_evolve_scalar_sources
 *   (2) the transfer loop `do q_ix ... call SourceToTransfers` (cmbmain.f90:287-291),
 *       with the source k-spline of InitSourceInterpolation (cmbmain.f90:1249-1265)
 *       -> cambgpu_los_flat
 *   (3) `call CalcScalCls(State%CLdata%CTransScal)`        (cmbmain.f90:323)
 *       -> cambgpu_calc_scal_cls
 *
 * plus whole-pipeline entry points that mirror CAMB_GetResults
 * (fortran/camb.f90:60-192) for one cosmology or a batch.
 *
 * Conventions (following the reference):
 *   - every array is caller-allocated host memory (GetSourceMem cmbmain.f90:755-782,
 *     Init_ClTransfer results.f90:3110-3123, ClTransferToCl cmbmain.f90:310-356);
 *   - the library owns its device buffers and caches the Bessel table across calls
 *     (as bessels.f90:64-112 caches it on the host);
 *   - return 0 on success, else an error code with the meaning of config.f90:66-74
 *     (4 = error_evolution for ODE failures, 9 = allocation, 2 = unsupported params,
 *     5 = reionization, 3 = recombination);  the library never exits the process.
 *   - threads: every call that uses the device takes one internal lock, so host threads
 *     may call concurrently and their device work runs one call at a time; host-table
 *     building (cambgpu_prepare_tables, cambgpu_tables_create) runs concurrently.  The
 *     process-wide settings (cambgpu_set_precision / _ode_*) apply to every later call of
 *     every thread: set them before concurrent use.
 */
#ifndef CAMBGPU_H
#define CAMBGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define CAMBGPU_OK 0
#define CAMBGPU_ERROR_UNSUPPORTED_PARAMS 2
#define CAMBGPU_ERROR_RECOMBINATION 3
#define CAMBGPU_ERROR_EVOLUTION 4
#define CAMBGPU_ERROR_REIONIZATION 5
#define CAMBGPU_ERROR_ALLOCATION 9
#define CAMBGPU_ERROR_CUDA 10

/* Cosmological and accuracy parameters: the subset of CAMBParams / AccuracyParams
 * (fortran/model.f90:27-209) that the scalar flat path reads. */
typedef struct CambGpuParams {
    double H0, ombh2, omch2, omk, TCMB, YHe;
    double nnu;                  /* total effective number of neutrinos N_eff */
    double mnu;                  /* sum of the massive neutrino masses in eV (0: all massless) */
    int num_massive_neutrinos;   /* degenerate massive eigenstate holds this many neutrinos */
    double optical_depth;        /* reionization tau (re_use_optical_depth = T) */
    double reion_delta_redshift; /* tanh width, default 0.5 */
    double As, ns, nrun, pivot_scalar, Alens;
    int max_l;                   /* CP%Max_l */
    double max_eta_k;            /* CP%Max_eta_k */
    int do_lensing;              /* lensing-potential source (3 sources) */
    double AccuracyBoost, lAccuracyBoost, lSampleBoost, IntTolBoost, TimeStepBoost;
    double SourcekAccuracyBoost, IntkAccuracyBoost, BesselBoost, BessIntBoost;
    double TimeSwitchBoost, LimberBoost, BackgroundTimeStepBoost;
    int accurate_polarization, accurate_reionization;
    double LensingBoost;         /* AccuracyParams%LensingBoost (lensing theta sampling and range) */
    /* matter transfer functions (CAMBparams%Transfer, model.py set_matter_power) */
    int want_cls;                /* 1: CMB sources and C_l; 0: matter transfer functions only */
    int want_transfer;           /* 1: transfer functions at transfer_redshifts (with want_cls = 0) */
    int transfer_high_precision; /* Transfer%high_precision (set_matter_power sets it) */
    double transfer_kmax;        /* Transfer%kmax in 1/Mpc */
    int num_transfer_redshifts;  /* 1..256 (max_transfer_redshifts), decreasing, as set_matter_power sorts them */
    double transfer_redshifts[256];
    int reion_use_optical_depth; /* 1: optical_depth fixes the reionization redshift; 0: reion_redshift does */
    double reion_redshift;
    int recfast_no_rosenbrock;   /* 1: Recfast%use_rosenbrock = F (Dormand-Prince with the Saha hold
                                    throughout); 0 (default): the Rosenbrock phase until x_H = 0.976 */
} CambGpuParams;

/* Per-k-mode setup: the hierarchy sizes of GetNumEqns (equations.f90:860-1070)
 * and the start/tight-coupling times of GetTauStart (cmbmain.f90:706-729) and
 * initial (equations.f90:1940-1950). */
typedef struct CambGpuModeSpec {
    double q;
    double taustart;
    double tight_switch_tau;
    int lmaxg, lmaxgpol, lmaxnr;
    int lmaxnu;                /* massive-neutrino hierarchy lmax (0 without massive neutrinos) */
    int nq0[3];                /* momentum bins evolved from the start, per mass eigenstate */
    int pad;
    double nu_l_boost[3];      /* MassiveNuTransferLAccuracyBoost (equations.f90:484-500) */
    double nu_approx_time[3];  /* MassiveNuApproxTime set in initial (equations.f90:2091-2102) */
} CambGpuModeSpec;

/* Read-only view of everything the hot path consumes for one cosmology: the
 * background scalars of CAMBdata (results.f90:188-216), the thermal-history tables
 * of TThermoData (results.f90:75-111), the source time grid (SetTimeSteps), the
 * source and integration k grids, the l sampling and the flat Bessel table.
 * All pointers are host pointers owned by the handle that filled the view. */
typedef struct CambGpuTables {
    /* background */
    double grhog, grhor, grhornomass, grhoc, grhob, grhov, grhok;
    double adotrad, tau0, DMt0, taurst, taurend, tau_maxvis, matter_verydom_tau;
    double akthom, fHe;
    /* massive neutrinos (one or two mass eigenstates; MassiveNu module) */
    int nu_eig, nqmax;
    double nu_masses[3], grhormass[3], nu_tau_nonrel[3];
    const double* nu_q;               /* [nqmax] momenta */
    const double* nu_int_kernel;      /* [nqmax] quadrature weights */
    const double* nu_tau_notmassless; /* [nu_eig][nqmax] */
    /* thermal history */
    int nthermo;
    double tauminn, dlntau, dlntau_inv, tight_tau;
    const double* thermo_horner; /* [nthermo][16]: cs2b(4) opacity(4) a/tau(4) dopacity(4) */
    const double* dotmu;         /* [nthermo] */
    const double* ddotmu;        /* [nthermo] */
    const double* cs2;           /* [nthermo] */
    const double* dddotmu;       /* [nthermo] */
    const double* ddddotmu;      /* [nthermo] */
    const double* emmu;          /* [nthermo] */
    const double* demmu;         /* [nthermo] */
    /* source time steps (TimeSteps%points / dpoints) */
    int ntau;
    const double* tau_points;
    const double* tau_dpoints;
    /* source k grid (Evolve_q) and per-mode setup */
    int nk;
    const double* q_evolve;
    const CambGpuModeSpec* modes;
    /* integration q grid (ThisCT%q) */
    int nq;
    const double* q_int;
    const double* dq_int;
    /* sampled l (ThisCT%ls%l) */
    int nl;
    const int* ls;
    /* flat Bessel table: bessel_horner(4, num_xx-1, nl) laid out [l][x][4] */
    int num_xx;
    const double* bess_x;
    const double* bessel_horner;
    /* settings */
    int nsrc;                /* 2 unlensed, 3 with lensing potential */
    int want_late_time;      /* WantLateTime (cmbmain.f90:138) */
    double max_etak_scalar;  /* InitVars cmbmain.f90:812-813 */
    double tol1;             /* ODE tolerance, cmbmain.f90:1018 */
    double max_bessels_etak; /* maximum_qeta */
    double AccuracyBoost, IntTolBoost, TimeSwitchBoost, BessIntBoost, LimberBoost;
    double lAccuracyBoost;
    int accurate_polarization, accurate_reionization;
    double As, ns, nrun, pivot_scalar, Alens;
    /* C_l interpolation and lensing */
    int max_l;                  /* CP%Max_l (last sampled l) */
    int do_lensing;             /* lens the C_l (CP%DoLensing) */
    double cl_template_scale;   /* lSamples%template_l_scale (results.f90:1517-1520) */
    double lens_accuracy_boost; /* AccuracyBoost * LensingBoost */
    /* transfer functions only: q_evolve/modes are then the transfer k grid (InitTransfer,
     * cmbmain.f90:564-704) and every mode is evolved to each transfer time (GetTransfer,
     * cmbmain.f90:1167-1188) */
    int transfer_only;
    int num_transfer_times;
    const double* transfer_times; /* tau of the transfer redshifts, increasing */
    double hubble_h;              /* H0/100 */
    int want_cls;
    int transfer_high_precision;       /* Transfer%high_precision with transfers requested */
    double late_phot_switch_boost_min; /* 2 for high-precision transfers (equations.f90:318-320), else 0 */
    /* A run that wants the CMB and transfer functions keeps evolving its source modes, and
     * storing their sources, at late times until tau passes this time, the last transfer
     * time (CalcScalarSources, cmbmain.f90:1032-1035); -1 otherwise. */
    double src_keep_tau;
    /* The transfer half of such a run: its first transfer_source_modes modes are the source
     * grid's, which stop at every source time as well, in CalcScalarSources' order
     * (cmbmain.f90:1020-1070); 0 otherwise. */
    int transfer_source_modes;
} CambGpuTables;

/* Fills p with the reference's defaults (model.f90:36-209, Python set_params). */
void cambgpu_default_params(CambGpuParams* p);

/* ---- host-side tables (background, RECFAST, reionization, grids, Bessel table) ---- */
/* Replaces CAMBdata%SetParams + InitVars (results.f90:332-628, cmbmain.f90:785-862),
 * SetkValuesForSources (cmbmain.f90:864-936), lSamples_init (results.f90:1505-1704),
 * SetkValuesForInt (cmbmain.f90:1267-1349) and InitSpherBessels (bessels.f90:64-112). */
int cambgpu_tables_create(const CambGpuParams* p, void** handle);
int cambgpu_tables_view(void* handle, CambGpuTables* view);
/* The transfer-function half of a handle whose parameters want the CMB and transfer
 * functions (want_cls = want_transfer = 1): the source k grid followed by the transfer
 * grid's points above it (InitTransfer with WantCls, cmbmain.f90:681-699), transfer_only
 * set for the device's transfer path; code 2 for any other handle. */
int cambgpu_tables_transfer_view(void* handle, CambGpuTables* view);
void cambgpu_tables_destroy(void* handle);
/* Background quantities for checks: tau0, DMt0, taurst, taurend, tau_maxvis,
 * zre (reionization mid redshift), x_e(z) at the requested redshifts. */
int cambgpu_tables_derived(void* handle, double* out8);
int cambgpu_recfast_xe(void* handle, const double* z, int n, double* xe);
/* Conformal time from the big bang to each redshift z[i], in Mpc: CAMBdata_TimeOfz
 * (results.f90:673-681, DeltaTime(0, 1/(1+z)) at its default tolerance), which
 * camb.CAMBdata.conformal_time (camb/results.py:1779) calls. */
int cambgpu_conformal_time(void* handle, const double* z, int n, double* eta);

/* ---- hot path on the GPU (host buffers in and out) ---- */
/* (1) cmbmain.f90:205-209: LinearSrc laid out [ntau][nsrc][nk] (k fastest, as the
 *     reference's LinearSrc(nk, nsrc, ntau) in Fortran order). */
int cambgpu_evolve_scalar_sources(const CambGpuTables* t, double* linear_src);
/* (2) cmbmain.f90:1249-1265 + 287-291: Delta_p_l_k laid out [nq][nl][nsrc]
 *     (src fastest, as Delta_p_l_k(nsrc, nl, nq) in Fortran order). */
int cambgpu_los_flat(const CambGpuTables* t, const double* linear_src, double* delta_p_l_k);
/* (3) cmbmain.f90:3179-3343: iCl laid out [nl][6] with columns TT EE TE PP PT PE
 *     (C_Temp..C_PhiE), l(l+1)C_l/2pi at the sampled l. */
int cambgpu_calc_scal_cls(const CambGpuTables* t, const double* delta_p_l_k, double* icl);

/* Allocation-free variant of cambgpu_los_flat (no counterpart in the reference): for
 * callers that cannot call cudaMalloc -- code inside a framework that owns all device
 * memory, or a service that must not allocate after start-up.  Every array pointer in
 * `t` (q_evolve, tau_points, tau_dpoints, q_int, ls, bess_x, bessel_horner) and both
 * buffers are DEVICE (or managed) pointers owned by the caller -- a host pointer is
 * rejected with code 2; the spline scratch lives in a 16 MiB static device array inside
 * the library.  Problems with 5*nk + ntau*nsrc*nk beyond it, or with ntau above 3722
 * (the projection stages ntau*44 + 64 bytes of the time grid in at most 160 KiB of
 * shared memory), are rejected with code 2 and a message before any device call.  Work
 * is enqueued on `stream` (a cudaStream_t, NULL = the default stream) and the call
 * blocks until that stream has finished it.  All calls share the scratch: calls that
 * overlap on the GPU race, so serialise them.  The first call on a device sets up the
 * scratch address (under a lock, so concurrent first calls do it once); make it before
 * any stream capture. */
int cambgpu_los_flat_noalloc(const CambGpuTables* t, const double* linear_src_dev, double* delta_dev, void* stream);

/* ---- whole pipeline (CAMB_GetResults for the scalar flat path) ---- */
/* cl_out: [lmax_out+1][4] TT EE BB TE of l(l+1)C_l/2pi (dimensionless), BB = 0,
 * as results.py get_unlensed_scalar_cls. */
int cambgpu_get_results(const CambGpuParams* p, int lmax_out, double* cl_out);
/* n cosmologies in one persistent launch per stage; cl_out [n][lmax_out+1][4];
 * status [n] (per-cosmology error code). */
int cambgpu_get_results_batch(const CambGpuParams* p, int n, int lmax_out, double* cl_out, int* status);

/* Spectra of n cosmologies: camb.get_results followed by the CAMBdata getters
 * get_unlensed_scalar_cls, get_lensed_scalar_cls and get_lens_potential_cls
 * (camb_python.f90:585-632).  Any output pointer may be NULL to skip it.
 *   unlensed, lensed: [n][lmax_out+1][4] TT EE BB TE of l(l+1)C_l/2pi;
 *   lens_potential:   [n][lmax_out+1][3] PP PT PE ([L(L+1)]^2 C_L/2pi and crosses).
 * C_l at every l come from the sampled l by InterpolateCls (cmbmain.f90:3523-3540,
 * spline on the difference from the high-L template); lensing is CorrFuncFullSkyApodized
 * (lensing.f90:338-678, the reference default with AccurateBB off) and needs
 * do_lensing = 1; lensed spectra are zero above each cosmology's lmax_lensed, written to
 * lmax_lensed[n] (0 for cosmologies without lensing) when that pointer is not NULL. */
int cambgpu_get_spectra_batch(const CambGpuParams* p, int n, int lmax_out, double* unlensed, double* lensed,
                              double* lens_potential, int* lmax_lensed, int* status);

/* The same call in two halves, so that a caller can build the host tables of the next
 * batch while the device works on the current one (the reference builds them inside
 * CAMB_GetResults, results.f90:1924-2779, cmbmain.f90:785-936).
 * cambgpu_prepare_tables: background, thermal history, grids and Bessel table of n
 * cosmologies on the host threads; touches no device state and may run concurrently
 * with any other entry point.  cambgpu_get_spectra_prepared: upload, device pipeline
 * and outputs as cambgpu_get_spectra_batch (the tables stay valid and may be run
 * again); cambgpu_free_prepared releases them. */
typedef struct CambGpuPrepared CambGpuPrepared;
int cambgpu_prepare_tables(const CambGpuParams* p, int n, CambGpuPrepared** out, int* status);
int cambgpu_get_spectra_prepared(const CambGpuPrepared* t, int lmax_out, double* unlensed, double* lensed,
                                 double* lens_potential, int* lmax_lensed, int* status);
void cambgpu_free_prepared(CambGpuPrepared* t);
/* Matter transfer functions of n cosmologies with want_cls = 0 and want_transfer = 1
 * (camb.get_results after set_matter_power; outtransf, equations.f90:2256-2271, and
 * Transfer_Get_sigmas, results.f90:4115-4182).  Per cosmology, with nq_max entries
 * reserved per redshift:
 *   transfer: [n][nz][nq_max][13] float, MatterTransferData%TransferData(13, nq, nz) in
 *             Fortran order (k/h, then CDM, baryon, photon, massless nu, massive nu, total,
 *             total without nu, total with dark energy, Weyl k^2 Phi, Newtonian CDM and
 *             baryon velocities, baryon-CDM velocity, each over k^2), single precision as
 *             the reference stores it;
 *   nq:       [n] number of transfer wavenumbers used;
 *   sigma8, sigma2_vdelta_8: [n][nz] at R = 8 Mpc/h (the redshift order of the input).
 * Any output pointer may be NULL. */
int cambgpu_get_transfer_batch(const CambGpuParams* p, int n, int nq_max, float* transfer, int* nq, double* sigma8,
                               double* sigma2_vdelta_8, int* status);

/* A run that wants the CMB and transfer functions (want_cls = want_transfer = 1 for every
 * cosmology), in the reference's single evolution: one transfer-path launch evolves each
 * source mode once, storing its CMB sources at the source times and its transfer
 * variables at the transfer times (CalcScalarSources with WantTransfer,
 * cmbmain.f90:1020-1070), and the transfer grid's modes above the source grid
 * (TransferOut, cmbmain.f90:1136-1165); the projection, C_l, interpolation and lensing then
 * run on those sources.  Outputs as cambgpu_get_spectra_batch and
 * cambgpu_get_transfer_batch. */
int cambgpu_get_results_with_transfers(const CambGpuParams* p, int n, int lmax_out, double* unlensed, double* lensed,
                                       double* lens_potential, int* lmax_lensed, int nq_max, float* transfer, int* nq,
                                       double* sigma8, double* sigma2_vdelta_8, int* status);

/* Lensing l range of a cosmology's tables: out3 = {lmax of the lensing sums
 * (LensingExtrapLmax, lensing.f90:161-177), lmax_lensed (InitLensedClArrays,
 * lensing.f90:230-247), number of theta points}. */
int cambgpu_lensing_range(const CambGpuTables* t, int* out3);

/* ---- resident batch: tables staged in device memory once, then timed runs ---- */
/* Builds and uploads n cosmologies; the batch stays resident until released or until
 * another call stages a batch (the arena is shared): the calls below then return 2. */
int cambgpu_batch_prepare(const CambGpuParams* p, int n);
/* The same batch on grids shared by all its cosmologies (no counterpart in the reference,
 * where every cosmology has its own grids): one comoving-distance grid chi_n, each
 * member's time steps tau_n = tau0 - chi_n (nodes with tau >= taurst/2), following at every
 * chi the finest native time spacing of any member; the source k grid, integration q grid
 * and Bessel table of the member with the median tau0.  Needed by the tensor-core
 * projection (cambgpu_set_precision(2)); the FP64 and mixed forms run on it too, so the
 * projections compare on the same grids.  CMB runs of one l sampling
 * and one set of sources; nchi_out (optional) receives the number of shared nodes. */
int cambgpu_batch_prepare_shared(const CambGpuParams* p, int n, int* nchi_out);
/* The shared grids of cambgpu_batch_prepare_shared applied to n existing table handles of
 * cambgpu_tables_create (host only; their views change). */
int cambgpu_tables_share_grids(void** handles, int n, int* nchi_out);
/* Runs ODE, source spline + LOS, C_l on the resident batch; ms3 = device ms per stage. */
int cambgpu_batch_run(double* ms3);
/* C_l of the last run, [n][lmax_out+1][4] as cambgpu_get_results. */
int cambgpu_batch_fetch(int lmax_out, double* cl_out);
/* CAMBdata.power_spectra_from_transfer (camb/results.py, camb.f90:25-58): new primordial
 * power (per-cosmology As, ns, nrun, pivot_scalar; a NULL array keeps the current
 * values) applied to the resident batch's transfer functions Delta_p_l_k without
 * re-evolving: C_l k-integral, interpolation and lensing rerun on the device.  Outputs as
 * cambgpu_get_spectra_batch (any may be NULL). */
int cambgpu_batch_spectra_from_transfer(const double* As, const double* ns, const double* nrun,
                                        const double* pivot_scalar, int lmax_out, double* unlensed, double* lensed,
                                        double* lens_potential, int* lmax_lensed);
void cambgpu_batch_release(void);

/* ---- runtime ---- */
/* Arithmetic of the line-of-sight projection (no counterpart in the reference, which is
 * FP64 throughout).  0 (default): FP64 everywhere -- the plain form whose transfer
 * functions and C_l match the reference's algorithm to rounding.  1: mixed precision --
 * the staged sources (an FP32 copy of the source k-spline), the Bessel weights, the
 * Bessel table and the products in FP32, summed in FP32 over 16 time steps per lane and
 * accumulated as compensated FP32 pairs, converted to FP64 once per (q, l); the ODE, the
 * spline itself, the window set-up, the Limber branch, the C_l k-integral, interpolation
 * and lensing stay FP64.  C_l agree with the FP64 form to ~1e-6. */
int cambgpu_set_precision(int mode);
/* Mode 2 (no counterpart in the reference): the projection of a batch on shared grids
 * (cambgpu_batch_prepare_shared) as split hi/lo BF16 products on the tensor cores --
 * Delta[l][c] = sum_n j_l(q chi_n) dchi_n S_c(q, tau0_c - chi_n) per q and source, one
 * matrix product for the whole batch, FP32 accumulation in tensor memory, the FP64 kernel's
 * windows, cuts and Limber values applied around it; other batches return 2. */
int cambgpu_get_precision(void);
/* ODE kernel variant: 32/16/8 = lanes per k-mode with the state in registers (massless
 * neutrinos, CMB sources); 6 = one warp per k-mode with the state rows in shared memory
 * (any layout: massive neutrinos, transfer functions); 1/2/3/4/5 = one thread per k-mode
 * compiled for 3/4/5/6/8 resident blocks of 128 per SM; 7 = one thread per k-mode compiled
 * for 2 resident blocks (CMB sources; transfer-function runs fall back to 2); 0 = the
 * autotuned choice. */
int cambgpu_set_ode_team(int lanes_per_mode);
/* ODE launch shape: queue order (-1 = the autotuned one, else as for the autotuner) and a
 * cap on resident threads per SM in units of 128 (0 = as many as fit; a lower cap leaves
 * modes in the work queue for threads that finish early). */
int cambgpu_set_ode_launch(int queue_order, int blocks_per_sm);
/* ODE schedule (no counterpart in the reference): 0 = each thread's first mode from its
 * index, later ones from an atomic queue counter; 1 = static stride (thread t of T takes
 * queue entries t, t + T, t + 2T, ...); -1 = the autotuned choice. */
int cambgpu_set_ode_schedule(int schedule);
/* In-library autotuner: times ODE variants, work-queue orders and resident-block caps on
 * n cosmologies and keeps the fastest for that batch-size class.  Queue orders: 0 = decreasing q,
 * 1 = increasing q, 2 = bands of q with the cosmologies of each band ordered by neutrino
 * mass, 3 = decreasing cost measured by the batch's previous run (evaluations x system
 * size; order 2 until a run has recorded it), 4 = order 2 cut into bundles of 32 modes
 * dealt to the warps of a static-stride launch by the previous run's costs, longest
 * first, so that every warp gets the same work (thread-per-mode kernels with the
 * static-stride schedule; order 2 otherwise).  Before a batch's first run, order 4 uses
 * the evaluations per ln q recorded from the first run of the last batch of the same kind
 * (same lmax, sources, massive neutrinos or not, transfer functions or not), and order 2
 * when there is none; from the batch's second run its own measured costs.  Queue orders
 * never change results, only which thread runs which mode.
 * best = [team, order, class, cap]; times (optional, >= 16 entries) receives ms per
 * candidate (0 for candidates that do not apply to the batch). */
int cambgpu_autotune_ode(const CambGpuParams* p, int n, int* best, double* times);
/* Wall-clock split of the last cambgpu_get_spectra_batch / get_results_batch /
 * get_spectra_prepared call, in ms: [host tables (for a prepared batch: its
 * cambgpu_prepare_tables), staging (pinned copy + uploads enqueued), device pipeline,
 * packing + D2H]. */
int cambgpu_last_host_timings(double* out4);
/* Kernel timing of the last GPU call, in ms: [ode, spline, los, cls, h2d, d2h]. */
int cambgpu_last_timings(double* out6);
/* Derivative evaluations of the last ODE launch (all modes of all cosmologies). */
long long cambgpu_last_ode_evals(void);
/* Host<->device bytes moved by the last pipeline call: out2 = [h2d, d2h]. */
int cambgpu_last_transfer_bytes(long long* out2);
/* Measures the device's FP64 FMA throughput (TFLOP/s) with a DFMA-chain kernel. */
int cambgpu_probe_fp64_tflops(double* tflops);
/* Split hi/lo BF16 matrix product on the tensor cores (tcgen05.mma, FP32 accumulation in
 * tensor memory; no counterpart in the reference, whose projection is FP64 loops):
 * D[m][n] = sum_k A[m][k] B[n][k] for row-major host buffers A [M][K], B [N][K], D [M][N],
 * each FP32 operand split into a BF16 pair and D = A_hi B_hi + A_hi B_lo + A_lo B_hi.
 * The primitive of the shared-grid projection; sizes 1-65536. */
int cambgpu_gemm_bf16x3(const float* A, const float* B, int M, int N, int K, float* D);
/* The FP64 issue model behind the ODE kernels' design (no counterpart in the reference):
 * one block per SM with warps_per_sm warps, active_lanes lanes of each warp running
 * `chains` (1, 4 or 8) independent DFMA chains; returns the lane FMAs retired per SM
 * cycle (clock64 around the loop, mean over SMs).  On a GB300 a warp issues one DFMA per
 * 64 cycles whatever its lanes or chains, and an SM saturates near 1.7 lane FMAs per
 * cycle with four warps. */
int cambgpu_probe_fp64_pipe(int warps_per_sm, int active_lanes, int chains, double* lane_fma_per_sm_cycle);
/* Number of kernels the library launched since the counter was reset. */
long long cambgpu_kernel_launches(int reset);
/* Message of the calling thread's last error (empty if none). */
const char* cambgpu_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
