/* dpgpu.h -- C ABI of libdpgpu.so, the GB300 (sm_103a) implementation of the
 * DiffPumas.jl data-parallel hot path: backward Monte Carlo muon transport
 * (run_backward_mc) and the voxel-density tomography forward model with its
 * density adjoint.
 *
 * Plain C types only.  Every entry point returns 0 on success, a negative
 * DP_ERR_* code on misuse or CUDA failure (dp_last_error() gives the text),
 * never aborts.  One CUDA stream per context; calls on one context must be
 * serialised by the caller; contexts may be used from different threads.
 * Device memory is owned by the handles.  Host arrays are borrowed for the
 * duration of a call.  "_dev" variants take device pointers that must stay
 * valid until the call returns (the call synchronises its stream).
 *
 * Reference citations are paths inside the DiffPumas.jl project.
 */
#ifndef DPGPU_H
#define DPGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DPGPU_VERSION 1

/* Return codes */
#define DP_OK 0
#define DP_ERR_ARG (-1)     /* ArgumentError in the reference */
#define DP_ERR_CUDA (-2)
#define DP_ERR_DOMAIN (-3)  /* DomainError in the reference (table domain) */
#define DP_ERR_ALLOC (-4)
#define DP_ERR_STATE (-5)   /* loop/iteration cap reached: status words tell which */

/* Per-history status bits (MC kernels write one int32 per history when asked).
 * They map to the reference throw sites and loop caps:
 *   DP_ST_STEP_CAP    2,000,000 transport steps (no reference counterpart: the
 *                     reference loop is unbounded; src/Geometry.jl:553)
 *   DP_ST_OUTER_CAP   1000 mode-loop passes (src/Geometry.jl:553 is unbounded)
 *   DP_ST_EVENT_CAP   100000 hard events (src/MixedTransport.jl:157,193)
 *   DP_ST_DOMAIN_HI   energy above the prepared tables (src/MixedTransport.jl:45,155,196)
 *   DP_ST_DOMAIN_LO   energy below the prepared tables (src/MixedTransport.jl:44)
 *   DP_ST_ZERO_RATE   non-positive hard-event rate (src/MixedTransport.jl:113)
 *   DP_ST_BAD_WEIGHT  invalid adjoint hard-event weight (src/MixedTransport.jl:186)
 *   DP_ST_TABLE_WAIT  a table-staging wait gave up (no reference counterpart)
 *   DP_ST_NO_PROGRESS a fixed-path step made no spatial progress
 *                     (src/Tomography.jl:916,965)
 *   DP_ST_BAD_MEDIUM  a fixed-path segment names a medium outside the media
 *                     set (device-array calls; host calls reject it up front)
 * A history with any bit but DP_ST_OUTER_CAP contributes zero flux; the call
 * then returns DP_ERR_DOMAIN (domain, rate, weight bits) or DP_ERR_STATE
 * (caps, no progress), where the reference would throw. */
#define DP_ST_OK 0
#define DP_ST_STEP_CAP 1
#define DP_ST_OUTER_CAP 2
#define DP_ST_EVENT_CAP 4
#define DP_ST_DOMAIN_HI 8
#define DP_ST_DOMAIN_LO 16
#define DP_ST_ZERO_RATE 32
#define DP_ST_BAD_WEIGHT 64
#define DP_ST_TABLE_WAIT 128
#define DP_ST_NO_PROGRESS 256
#define DP_ST_BAD_MEDIUM 512

typedef struct dp_ctx dp_ctx;
typedef struct dp_physics dp_physics;

/* ------------------------------------------------------------------ context */
int dp_version(void);
/* Creates a context on CUDA device `device` with its own stream. */
int dp_init(int device, dp_ctx** out);
int dp_destroy(dp_ctx* ctx);
/* Text of the last error raised on this context ("" if none). */
const char* dp_last_error(const dp_ctx* ctx);
/* Makes the context launch on the caller's cudaStream_t (e.g. a CUDA.jl or
 * torch stream); NULL restores the context's own stream. */
int dp_set_stream(dp_ctx* ctx, void* cuda_stream);
void* dp_get_stream(const dp_ctx* ctx);
/* Per-kernel timing with CUDA events recorded on the context stream around
 * each main kernel (off by default; recording adds no host synchronisation,
 * dp_kernel_time resolves the events).  Names: "csda_mc", "tomo_trace",
 * "tomo_forward", "tomo_adjoint", "tomo_transpose". */
int dp_set_timing(dp_ctx* ctx, int enable);
int dp_kernel_time(dp_ctx* ctx, const char* kernel, double* ms_total);
/* The same with the number of timed launches of that kernel (may be NULL). */
int dp_kernel_stats(dp_ctx* ctx, const char* kernel, double* ms_total, long long* launches);
/* Number of kernels this context has launched. */
long long dp_launch_count(const dp_ctx* ctx);
/* Bytes of device scratch this context holds (its grow-on-demand slots,
 * reused across calls and freed by dp_destroy); a diagnostic. */
long long dp_scratch_bytes(const dp_ctx* ctx);
/* blocking = 1 (default): device-pointer calls synchronise and report kernel
 * errors before returning.  blocking = 0: they return once enqueued (no host
 * synchronisation, e.g. for CUDA-graph capture or back-to-back solver
 * iterations); dp_sync then waits and reports.  Host-pointer calls always
 * synchronise. */
int dp_set_blocking(dp_ctx* ctx, int blocking);
int dp_sync(dp_ctx* ctx);
/* Failure-path limits of this context, for tests of the error paths (no
 * reference counterpart; the reference's loops throw at fixed counts,
 * src/MixedTransport.jl:157,193).  step_cap: transport steps of one history
 * (default 2,000,000; DP_ST_STEP_CAP); event_cap: hard events of one mixed
 * step (default 100,000 as in the reference; DP_ST_EVENT_CAP); wait_iters:
 * polls of a table-staging wait before the block gives up (default 2^22;
 * DP_ST_TABLE_WAIT, the copy in flight is still awaited before the block
 * leaves).  A negative value restores the default.  Every limit ends its loop
 * with a status the call reports (DP_ERR_STATE); none of them faults. */
int dp_set_debug_limits(dp_ctx* ctx, int step_cap, int event_cap, int wait_iters);

/* ------------------------------------------------------------------ launch shapes
 * CTA size of the persistent transport kernels per kernel family and
 * precision (DP_PREC_FP64 / DP_PREC_MIXED).  They run one CTA per SM, so the
 * size trades registers per thread for warps per SM.  threads = 0 selects the
 * default; dp_mc_thread_choices lists the compiled sizes (first: default). */
#define DP_KERNEL_MC 0   /* dp_mc_histories, dp_mc_los: two-layer transport */
#define DP_KERNEL_DIR 1  /* dp_dir_mc: fixed-path transport */
int dp_mc_thread_choices(int precision, int* threads, int cap);  /* returns the count */
int dp_set_mc_threads(dp_ctx* ctx, int family, int precision, int threads);
int dp_get_mc_threads(const dp_ctx* ctx, int family, int precision, int* threads);
/* Autotuner.  For every compiled CTA size of (family, precision): run(user)
 * once untimed and once timed (CUDA events on the context stream; run
 * enqueues the caller's workload on this context and returns a dp status).
 * Keeps the fastest size on the context and writes it to best_threads;
 * ms[i] receives the time of choice i (up to cap entries).  A nonzero status
 * from run ends the search, restores the previous size and is returned. */
int dp_autotune(dp_ctx* ctx, int family, int precision, int (*run)(void* user), void* user,
                int* best_threads, double* ms, int cap);
/* The full launch shape of those kernels: the CTA size, where the media
 * tables live (staging 0: copied to shared memory once per CTA when they fit,
 * the default in FP64; 1: read through L1/L2, the default in DP_PREC_MIXED,
 * whose kernels size their shared memory to the smallest carve-out step and
 * leave the rest of the SM's 256 KB to the L1 cache) and the order histories are handed out
 * in (order 0: longest first, by a per-history estimate of its steps, the
 * default; 1: index order).  sync is a mask of the transport phases (bit 0:
 * below the mode switch, bit 1: above it) whose steps the warps of a CTA take
 * in lockstep, one block barrier per step, so that they fetch the same code
 * at the same time, and whose hard-event DCS sums the whole CTA evaluates
 * together; it applies to DP_PREC_MIXED (default: 3 for DP_KERNEL_MC, 2 for
 * DP_KERNEL_DIR).  A thread refills itself one history at a time from a
 * warp-aggregated counter.  Every history keeps its own stream, so staging
 * and order change no result (bit for bit).  The DCS sums of a lockstep phase
 * are compiled separately from those of a free-running one, and the code
 * generator may fuse their FP32 multiply-adds differently, so results under
 * another sync mask agree statistically, not bit for bit.  Each CTA size is a
 * separately compiled kernel whose FP32 multiply-adds the code generator may
 * fuse differently, so results at another size agree statistically too. */
typedef struct {
  int threads, staging, order, sync;
} dp_mc_shape;
int dp_set_mc_shape(dp_ctx* ctx, int family, int precision, const dp_mc_shape* shape);
int dp_get_mc_shape(const dp_ctx* ctx, int family, int precision, dp_mc_shape* shape);
/* dp_autotune over the whole shape, one dimension at a time (CTA size, then
 * staging, then order, then for DP_PREC_MIXED the sync mask, each from the
 * best so far): every candidate runs
 * run(user) once untimed and once timed.  The best shape stays on the context
 * and goes to *best; tried[i] / ms[i] list the candidates and their times (up
 * to cap), *n_tried their count. */
int dp_autotune_shape(dp_ctx* ctx, int family, int precision, int (*run)(void* user), void* user,
                      dp_mc_shape* best, dp_mc_shape* tried, double* ms, int cap, int* n_tried);

/* ------------------------------------------------------------------ physics tables
 * Column layout of one material table (src/Physics.jl:64-102 MaterialTable).
 * Every column holds n_energies doubles on the material's kinetic-energy grid. */
enum dp_column {
  DP_COL_E = 0,          /* kinetic energy, GeV */
  DP_COL_LOGE,           /* log(E) */
  DP_COL_CSDA_S,         /* CSDA stopping power, GeV/(kg/m^2) */
  DP_COL_CSDA_R,         /* CSDA range, kg/m^2 */
  DP_COL_CSDA_T,         /* CSDA proper-time integral, kg/m^2 */
  DP_COL_MIXED_S,        /* restricted (soft) stopping power */
  DP_COL_MIXED_R,        /* restricted range */
  DP_COL_STRAG,          /* straggling variance, GeV^2/(kg/m^2) */
  DP_COL_ION,            /* ionisation stopping power */
  DP_COL_BREMS,
  DP_COL_PAIR,
  DP_COL_PHOTO,
  DP_COL_XS,             /* hard-event cross section, m^2/kg */
  DP_COL_LB1,            /* first transport path, kg/m^2 */
  DP_COL_LBE,            /* elastic path x p^2 */
  DP_COL_ECUT,           /* elastic cutoff angle */
  DP_COL_MAGROT,         /* magnetic rotation */
  DP_COL_MU0,            /* Coulomb screening parameter */
  DP_COL_FSPIN,          /* spin factor */
  DP_NCOL
};

typedef struct {
  double Z, A, I;        /* atomic number, mass number (g/mol), mean excitation (GeV) */
  double fraction;       /* mass fraction */
} dp_element;

typedef struct {
  const char* name;
  double density;        /* reference density, kg/m^3 */
  double I;              /* mean excitation energy, GeV */
  double ZoA;            /* <Z/A> (0: computed from the elements) */
  int n_elements;
  const dp_element* elements;
} dp_material;

typedef struct {
  double mass;           /* GeV/c^2 (muon 0.10565839) */
  double ctau;           /* m (muon 658.654) */
  double cutoff;         /* relative soft/hard cutoff (0.05) */
  double elastic_ratio;  /* (0.05) */
} dp_settings;

/* Uploads caller-built tables (the Julia create_physics output) to the device.
 * columns: n_materials x DP_NCOL x n_energies doubles, row-major in that order.
 * All materials share one energy grid.  recipes may be NULL (then hard-event
 * sampling, which needs the elemental recipes, is unavailable).
 * Replaces the table handover of src/Physics.jl:534-599 (create_physics). */
int dp_physics_upload(dp_ctx* ctx, const dp_settings* settings, int n_materials,
                      int n_energies, const double* columns, const dp_material* recipes,
                      dp_physics** out);

/* Builds tables on the host exactly as create_physics(MUON) does without PUMAS
 * dE/dx files (empirical DCS integration, src/Physics.jl:280-408, 534-599),
 * on a log grid of n_energies nodes in [K_min, K_max], then uploads them. */
int dp_physics_create(dp_ctx* ctx, const dp_settings* settings, int n_materials,
                      const dp_material* materials, int n_energies, double K_min, double K_max,
                      dp_physics** out);
int dp_physics_free(dp_physics* phys);
int dp_physics_info(const dp_physics* phys, int* n_materials, int* n_energies);
/* Copies column `col` of material `mat` (host copy of the device tables). */
int dp_physics_column(const dp_physics* phys, int mat, int col, double* out);
/* Index of the material with this name, or -1 (src/Physics.jl:609 get_material_index). */
int dp_physics_material_index(const dp_physics* phys, const char* name);
/* create_physics with PUMAS dE/dx files (src/Physics.jl:146-273
 * create_material_table_from_dedx, src/DEDXLoader.jl:100-190
 * load_dedx_file): material m's energy grid, CSDA stopping power and range
 * and energy-loss components come from dedx_paths[m]; the restricted
 * stopping power, straggling, hard cross section and Coulomb columns are
 * integrated from the recipe (with the file's <Z/A>).  All files must share
 * one energy grid. */
int dp_physics_create_dedx(dp_ctx* ctx, const dp_settings* settings, int n_materials,
                           const dp_material* materials, const char* const* dedx_paths,
                           dp_physics** out);
/* The same tables on the host only (no device): *n_energies receives the
 * grid size; with cols (capacity cap doubles) the n_materials x DP_NCOL x
 * n_energies columns.  Returns DP_ERR_ARG for unreadable files, differing
 * grids or a small cap. */
int dp_tables_from_dedx(const dp_settings* settings, int n_materials,
                        const dp_material* materials, const char* const* dedx_paths,
                        int* n_energies, double* cols, long cap);
/* Portable table file, the counterpart of the reference's Julia-only
 * .pumas serialisation (src/Loader.jl:30-105): settings, recipes and every
 * column in FP64, little-endian; loading reproduces the tables bit for bit
 * on x86-64 and AArch64 hosts. */
int dp_physics_save(const dp_physics* phys, const char* path);
int dp_physics_load(dp_ctx* ctx, const char* path, dp_physics** out);
/* The settings of a table set, and material m's name (copied into buf,
 * NUL-terminated; returns its length, or -1 without recipes or if cap is
 * too small). */
int dp_physics_settings(const dp_physics* phys, dp_settings* out);
int dp_physics_material_name(const dp_physics* phys, int mat, char* buf, int cap);

/* ------------------------------------------------------------------ backward MC
 * run_backward_mc (src/Geometry.jl:1286-1338) on a two-layer rock + air column. */
typedef struct {
  double rock_thickness;     /* m */
  double rock_density;       /* kg/m^3 */
  double elevation;          /* degrees */
  double energy_min;         /* GeV */
  double energy_max;         /* GeV (<= energy_min: single energy) */
  long n_samples;
  uint64_t seed;             /* Philox key; stream keyed by (seed, sample id) */
  int straggling;            /* 0: CSDA */
  int scattering;
  int compute_gradient;
  double energy_threshold_low; /* GeV (100) */
  double source_energy_max;  /* GeV, <= 0: min(1e9, table max) */
  double primary_altitude;   /* m (3e4) */
  int rock_material;         /* -1: "StandardRock" or 0 */
  int air_material;          /* -1: "Air" or the last table */
  int precision;             /* DP_PREC_FP64 (0): the reference's FP64
                                operations; DP_PREC_MIXED (1): FP32 stochastic
                                transport, and CSDA histories walked in FP32
                                with float-pair range and altitude, the final
                                energy and the flux in FP64 (within ~1e-6 of
                                FP64 per history) */
  /* Shallow porous layer of TwoLayerGeometry (src/Geometry.jl:47-72,
   * compute_flux's porous_* keywords, :899): the top porous_thickness m of
   * the rock column are material porous_material at porous_density.  Active
   * when porous_material >= 0 and porous_thickness > 0; the column then runs
   * through the stochastic kernels (CSDA steps when straggling = scattering
   * = 0), without the CSDA gradient. */
  int porous_material;       /* -1: none */
  double porous_density;     /* kg/m^3 */
  double porous_thickness;   /* m */
} dp_mc_params;

typedef struct {
  double flux, sigma;        /* estimate and standard error */
  double gradient;           /* d(CSDA sample-average flux)/d(rock_density) */
  double gradient_flux;      /* the CSDA surrogate's flux */
  double source_energy_max;
  long n_samples;
  long n_status_nonzero;     /* histories that hit a cap (see DP_ST_*) */
} dp_mc_result;

/* Whole estimator (_compute_flux_estimate, src/Geometry.jl:818-896): device
 * sampling, transport, deterministic reduction.
 * straggling = scattering = 0: deterministic CSDA transport; otherwise the
 * stochastic dual-mode transport (straggled with scattering below
 * energy_threshold_low, mixed above, src/Geometry.jl:534-672) of the rock
 * and air materials.  compute_gradient adds the CSDA sample-average gradient
 * over the same samples (src/Geometry.jl:933-945). */
int dp_backward_mc(dp_ctx* ctx, const dp_physics* phys, const dp_mc_params* p,
                   dp_mc_result* out);

/* Deterministic CSDA flux of explicit histories (compute_flux_differentiable,
 * src/Geometry.jl:958-986, and its Zygote gradient :1007-1028): contrib[i] =
 * w[i]*flux_i and dcontrib[i] = w[i]*d flux_i/d rho, in p->precision.  Host
 * pointers. */
int dp_csda_flux_samples(dp_ctx* ctx, const dp_physics* phys, const dp_mc_params* p,
                         long n, const double* energy, const double* charge,
                         const double* weight, double* contrib, double* dcontrib,
                         int32_t* steps);
/* Same with device pointers (inputs resident in HBM). */
int dp_csda_flux_samples_dev(dp_ctx* ctx, const dp_physics* phys, const dp_mc_params* p,
                             long n, const double* energy, const double* charge,
                             const double* weight, double* contrib, double* dcontrib,
                             int32_t* steps);
/* compute_flux_csda_direct (src/Geometry.jl:1126-1209): the two-layer CSDA
 * flux in closed form (one range inversion per layer, closed-form air
 * grammage, decay at the mean energy of each layer), as used by
 * compute_flux_differentiable_csda / compute_flux_gradient_csda
 * (:1220-1280): contrib[i] = w[i]*flux_i, dcontrib[i] = w[i]*d flux_i/d rho
 * (optional).  Geometry, materials and primary altitude from p.  Host pointers. */
int dp_csda_direct_samples(dp_ctx* ctx, const dp_physics* phys, const dp_mc_params* p, long n,
                           const double* energy, const double* charge, const double* weight,
                           double* contrib, double* dcontrib);
/* Philox samples exactly as dp_backward_mc draws them (log-uniform energy,
 * +-1 charge, weight 2*E*log(Emax/Emin)), for parity checks.  Host pointers. */
int dp_mc_samples(dp_ctx* ctx, const dp_mc_params* p, long n, double* energy,
                  double* charge, double* weight);

/* ------------------------------------------------------------------ stochastic MC
 * Propagation medium: one material or a runtime mixture with mass fractions
 * (MaterialMixture, src/Types.jl:357-376; mixture properties of
 * src/Physics.jl:1058-1323), with its MIXED transport kernel
 * (prepare_mixed_kernel, src/MixedTransport.jl:51-97: 8-fold refined log grid,
 * restricted stopping power, hard-event rate regularised below its onset,
 * cumulative range, hazard and proper-time integrals, elemental recipe).
 * The materials must share the physics energy grid and carry recipes. */
typedef struct dp_mixture dp_mixture;
int dp_mixture_prepare(dp_ctx* ctx, const dp_physics* phys, int n_materials,
                       const int* materials, const double* fractions, dp_mixture** out);
int dp_mixture_free(dp_mixture* mix);
/* Host copy of MIXED kernel column col (0 energy, 1 stopping power, 2 hard
 * rate, 3 range, 4 hazard, 5 proper time) into out (up to cap values); *n
 * receives the node count and *onset the hard-event onset energy. */
int dp_mixture_kernel(const dp_mixture* mix, int col, double* out, int cap, int* n,
                      double* onset);

/* Options of a stochastic run (run_backward_mc kwargs, src/Geometry.jl:1286). */
typedef struct {
  int straggling;              /* 1: straggled below / mixed above the threshold */
  int scattering;              /* 1: EHS, DEL angles and soft scattering below it */
  double energy_threshold_low; /* GeV (100) */
  double source_energy_max;    /* GeV; <= 0: min(1e9, table maximum) */
  uint64_t seed;               /* Philox key: stream (seed, history id) */
  int precision;               /* DP_PREC_FP64: the reference's FP64 operations;
                                  DP_PREC_MIXED: FP32 transport, FP64 positions,
                                  event kinematics, flux and tallies */
} dp_mc_config;

/* Explicit histories, the parity form of compute_flux_single with an rng
 * (src/Geometry.jl:694-757) on a rock (mixture) layer under air: history i has
 * final energy E[i], charge q[i], sampling weight w[i] and geometry
 * thickness/density/elevation/primary_altitude[i] (index 0 for every history
 * when geo_stride is 0); its random stream is (seed, id0 + i).  Outputs
 * contrib[i] = w[i]*flux_i and optionally status[i], steps[i] and the final
 * state (4 values per history: energy, altitude, direction cosine u_z,
 * transport weight).  Host pointers. */
int dp_mc_histories(dp_ctx* ctx, const dp_physics* phys, const dp_mixture* rock,
                    const dp_mixture* air, const dp_mc_config* cfg, long n, const double* E,
                    const double* q, const double* w, const double* thickness,
                    const double* density, const double* elevation,
                    const double* primary_altitude, int geo_stride, uint64_t id0,
                    double* contrib, int32_t* status, int32_t* steps, double* final_state);

/* One line of sight of a batched run: n_samples histories with log-uniform
 * final energies and +-1 charges drawn as run_backward_mc draws them
 * (src/Geometry.jl:863-875).  Geometry: rock thickness, bulk density and
 * elevation; when a *_max field exceeds its base value, each history draws
 * the value uniformly in [base, max] instead (Philox blocks 1-2).  Primary
 * altitude: thickness + air_height when air_height > 0, else
 * primary_altitude (<= 0: 3e4 m). */
typedef struct {
  double thickness, thickness_max;
  double density, density_max;
  double elevation, elevation_max;
  double primary_altitude, air_height;
  double energy_min, energy_max;
  long n_samples;
  /* the shallow porous layer's thickness and density (src/Geometry.jl:47-72),
   * used by the *_layers calls with a porous medium; 0: no layer */
  double porous_thickness, porous_density;
} dp_los;

typedef struct {
  double flux, sigma;          /* estimate and standard error (src/Geometry.jl:883-893) */
  double gradient;             /* d(CSDA sample-average flux)/d(density), when asked */
  double gradient_flux;        /* that CSDA surrogate flux */
  long n_samples;
  long n_status_nonzero;       /* histories with a status bit */
} dp_los_result;

/* Batched stochastic backward MC over many lines of sight in one persistent
 * launch (histories of all lines of sight share the device; the history id
 * is the running sample index over the batch).  compute_gradient adds the
 * deterministic CSDA sample-average flux and its derivative with respect to
 * each line's density over the same samples (src/Geometry.jl:933-945); it
 * needs fixed (undrawn) geometry and single-material rock and air.  Host
 * pointers. */
int dp_mc_los(dp_ctx* ctx, const dp_physics* phys, const dp_mixture* rock, const dp_mixture* air,
              const dp_mc_config* cfg, long n_los, const dp_los* los, int compute_gradient,
              dp_los_result* out);
/* Same with los and out in device memory; total_samples must equal the sum
 * of n_samples. */
int dp_mc_los_dev(dp_ctx* ctx, const dp_physics* phys, const dp_mixture* rock,
                  const dp_mixture* air, const dp_mc_config* cfg, long n_los, const dp_los* los,
                  long total_samples, int compute_gradient, dp_los_result* out);
/* The same columns with the shallow porous top layer of TwoLayerGeometry
 * (src/Geometry.jl:617-635): z in [thickness - porous_thickness, thickness)
 * is the prepared medium `porous` at each line's porous_density.  NULL
 * porous: dp_mc_los.  No CSDA gradient (compute_gradient must be 0). */
int dp_mc_los_layers(dp_ctx* ctx, const dp_physics* phys, const dp_mixture* rock,
                     const dp_mixture* porous, const dp_mixture* air, const dp_mc_config* cfg,
                     long n_los, const dp_los* los, int compute_gradient, dp_los_result* out);
int dp_mc_los_layers_dev(dp_ctx* ctx, const dp_physics* phys, const dp_mixture* rock,
                         const dp_mixture* porous, const dp_mixture* air,
                         const dp_mc_config* cfg, long n_los, const dp_los* los,
                         long total_samples, int compute_gradient, dp_los_result* out);

/* ---------------------------------------------------------- fixed-path MC
 * compute_directional_flux_mc (src/Tomography.jl:979-1041) over many
 * directions at once.  A media set lists the distinct prepared media the
 * paths use (cell mixtures from mc_cell_mixture_and_density,
 * src/Tomography.jl:826-845, the rock beyond the cells and the air); the
 * kernel copies the leading media to shared memory when they fit, so list
 * the most used first.  Replaces the per-call kernel preparation of
 * src/Tomography.jl:995-1003. */
typedef struct dp_dir_media dp_dir_media;
int dp_dir_media_create(dp_ctx* ctx, const dp_physics* phys, int n_media,
                        const dp_mixture* const* media, dp_dir_media** out);
int dp_dir_media_free(dp_dir_media* media);

/* One batch of directions (DirectionalPath, src/Tomography.jl:214-223). */
typedef struct {
  long n_dirs;
  const double* cos_theta;       /* cosd(zenith) per direction */
  const double* remaining_rock;  /* remaining_rock_distance (m) per direction */
  const double* air_distance;    /* metres of air: max(0, primary_altitude - surface_exit_z)
                                    / max(cos_theta, 1e-3) (src/Tomography.jl:1020) */
  const int32_t* valid;          /* NULL: all valid; 0: flux and sigma NaN */
  const int64_t* seg_ptr;        /* n_dirs + 1 running segment offsets (< 2^31 segments) */
  const int32_t* seg_medium;     /* media-set index per segment (the cell's mixture) */
  const double* seg_density;     /* kg/m^3 per segment (the cell's density) */
  const double* seg_length;      /* m per segment (CellSegment.distance) */
  const int64_t* sample_ptr;     /* n_dirs + 1 running sample offsets */
  const double* energy;          /* final energy (GeV) per sample; NULL: drawn per history */
  const double* charge;          /* +-1 per sample */
  const double* weight;          /* EnergySample.weight per sample */
  double energy_min, energy_max; /* draw range when energy == NULL (sample_energy_set,
                                    src/Tomography.jl:236-248, on Philox block 0) */
  int rock_medium, air_medium;   /* media-set indices of the rock beyond the cells, the air */
  double rock_density;           /* MaterialConfig.rock_density (kg/m^3) */
  double detector_elevation;     /* SiteConfig.detector_elevation (m): air density altitude */
} dp_dir_batch;

/* Flux and sigma (n - 1 form, src/Tomography.jl:1036-1039) per direction into
 * out[n_dirs] (gradient fields 0).  cfg: straggling, energy_threshold_low,
 * seed, precision; scattering must be 0 (the reference's ArgumentError);
 * source_energy_max 0 selects min(1e9, last table energy), the reference's
 * energy limit.  History i of the batch draws from Philox stream (seed, i).
 * contrib and status (optional, one per sample) receive 2 w_i w flux_i and
 * the DP_ST_* bits, final_state (optional, two per sample) the final energy
 * and transport weight. */
int dp_dir_mc(dp_ctx* ctx, const dp_physics* phys, dp_dir_media* media, const dp_dir_batch* batch,
              const dp_mc_config* cfg, dp_los_result* out, double* contrib, int32_t* status,
              double* final_state);
/* The same with every batch array and out in device memory (the struct
 * itself on the host); total_samples = sample_ptr[n_dirs]. */
int dp_dir_mc_dev(dp_ctx* ctx, const dp_physics* phys, dp_dir_media* media,
                  const dp_dir_batch* batch, long total_samples, const dp_mc_config* cfg,
                  dp_los_result* out);

/* ------------------------------------------------------------ voxel paths
 * trace_path(::VoxelVolume) / precompute_paths (examples/lvd_tomography.jl:
 * 583-627, 738-779, 835-861): the straight path from the detector (origin)
 * along (zenith, azimuth) through a voxel volume with the reference's
 * POINT_EPS march, cut at the slant distance of the surface exit.  Edges are
 * increasing (n + 1 per axis), cells x fastest.  Host arrays; a call with
 * seg_cell = seg_length = NULL only counts (seg_ptr[n_dirs]).  A direction
 * with surface_distance <= 0 or NaN is invalid (no segments, NaN outputs).
 * ctx may be NULL (no device work; it only receives the error message). */
typedef struct {
  int nx, ny, nz;
  const double* x_edges;
  const double* y_edges;
  const double* z_edges;
} dp_voxel_volume;
int dp_voxel_trace(dp_ctx* ctx, const dp_voxel_volume* volume, long n_dirs, const double* zenith,
                   const double* azimuth, const double* surface_distance, int64_t* seg_ptr,
                   int32_t* seg_cell, double* seg_length, int64_t seg_cap, double* traveled,
                   double* remaining_rock);

/* ------------------------------------------------ terrain and tetrahedral meshes
 * Host geometry (no device work).  An elevation map (Turtle ElevationMap,
 * src/Turtle.jl:455-481): z[iy * nx + ix] at node x0 + ix dx, y0 + iy dy.
 * map_elevation (:520-557) bilinear, map_gradient (:559-634); inside[i] = 0
 * off the map. */
typedef struct {
  int nx, ny;
  double x0, y0, dx, dy;
  const double* z;
} dp_elevation_map;
int dp_map_elevation(const dp_elevation_map* map, long n, const double* x, const double* y,
                     double* z, int32_t* inside);
int dp_map_gradient(const dp_elevation_map* map, long n, const double* x, const double* y,
                    double* gx, double* gy, int32_t* inside);
/* The terrain above a detector at the origin: the surface height at local
 * metres (x, y) is map_elevation(map, x xy_scale, y xy_scale) -
 * detector_elevation (examples/lvd_tomography.jl:214-217; the LVD map is in
 * km, xy_scale 1e-3).  ray_surface_exit_distance (:219-252) marches in
 * steps of `step` m up to max_distance (40 m, 25 km there), then bisects 40
 * times; dp_surface_exit gives per direction the slant distance, the exit
 * altitude above the detector and ok = 0 for a direction that leaves the
 * map or points down. */
typedef struct {
  dp_elevation_map map;
  double xy_scale, detector_elevation, step, max_distance;
} dp_terrain;
int dp_surface_exit(const dp_terrain* terrain, long n_dirs, const double* zenith,
                    const double* azimuth, double* distance, double* exit_z, int32_t* ok);
/* Ray-triangle intersection (src/TriangleIntersect.jl:78-115, Moller-Trumbore):
 * returns 1 and the distance (and the point, 3 doubles, if given) on a hit, 0
 * otherwise. */
int dp_ray_triangle(const double* origin, const double* dir, const double* p1, const double* p2,
                    const double* p3, double* distance, double* point);
/* A tetrahedral mesh (TetraVolume, examples/lvd_tomography.jl:172-179):
 * points[3 i + k], tets[4 t + v] 1-based point indices (TetGen's
 * connectivity; the mesh is built by the caller).  dp_tetra_neighbors fills
 * neighbors[4 t + f] with the 1-based tetrahedron across face f of
 * tetra_face_indices (:415-422), 0 on the boundary (build_tetra_neighbors,
 * :431-453).  dp_tetra_trace is trace_path(::TetraVolume) (:694-736) for
 * every direction: the POINT_EPS walk from the tetrahedron containing the
 * start point through neighbours, cut at the terrain's surface exit; cells
 * are 1-based tetrahedra; the count / fill protocol of dp_voxel_trace. */
typedef struct {
  long n_points;
  const double* points;
  long n_tets;
  const int32_t* tets;
} dp_tetra_mesh;
int dp_tetra_neighbors(const dp_tetra_mesh* mesh, int32_t* neighbors);
int dp_tetra_trace(dp_ctx* ctx, const dp_tetra_mesh* mesh, const int32_t* neighbors,
                   const dp_terrain* terrain, long n_dirs, const double* zenith,
                   const double* azimuth, int64_t* seg_ptr, int32_t* seg_cell,
                   double* seg_length, int64_t seg_cap, double* traveled,
                   double* surface_distance, double* remaining_rock, double* exit_z,
                   int32_t* valid);

/* ------------------------------------------------ water-fraction CSDA model
 * compute_directional_flux_csda (src/Tomography.jl:667-727),
 * directional_flux_and_grad_csda (:736-762) and assemble_forward_and_jacobian
 * (:773-820): per direction, the CSDA flux of a path through cells of water
 * mass fraction w, and d flux / d w.  MaterialConfig and SiteConfig
 * (src/Tomography.jl:179-201) and the CSDA corrections of
 * set_csda_correction! / set_csda_material_correction! (:136-175). */
typedef struct {
  int rock_material, water_material, air_material, porous_material; /* 0-based; porous < 0: none */
  double rock_density, water_density, porous_density, porous_top_thickness;
  double detector_elevation, primary_altitude;  /* SiteConfig (m) */
  int correction;                                /* CsdaCorrection.enabled */
  double kappa_strag, kappa_hard, resid_a, resid_b, resid_c, resid_d;
  int material_correction;                       /* CsdaMaterialCorrection.enabled */
  double material_linear, material_quadratic;
} dp_csda_config;

/* Directions and the energy samples they share (EnergySample list, at most 256). */
typedef struct {
  long n_bins;
  const double* cos_theta;       /* cosd(zenith) */
  const double* remaining_rock;  /* remaining_rock_distance (m) */
  const double* surface_exit_z;  /* surface_exit_z (m above the detector) */
  const int32_t* valid;          /* NULL: all valid; invalid or cos_theta <= 0: flux NaN */
  const int64_t* seg_ptr;        /* n_bins + 1 running segment offsets */
  const int32_t* seg_cell;       /* 0-based cell index per segment */
  const double* seg_length;      /* m per segment */
  int n_energy;
  const double* energy;
  const double* charge;
  const double* weight;
} dp_csda_batch;

/* flux[n_bins]; jac (optional) one value per segment in segment order: the
 * derivative of the direction's flux with respect to the water fraction of
 * the segment's cell through that segment (summed over a cell's segments it
 * is d flux / d w_cell, the entries of the reference's sparse Jacobian).
 * shallow: one flag per cell (NULL: none shallow).  precision DP_PREC_FP64:
 * the reference's FP64 operations; DP_PREC_MIXED: FP32 steps and tangents,
 * FP64 adjoint prefix sums, flux and reductions.  Host pointers. */
int dp_dir_csda(dp_ctx* ctx, const dp_physics* phys, const dp_csda_config* cfg,
                const dp_csda_batch* batch, long n_cells, const uint8_t* shallow,
                const double* water_fraction, double* flux, double* jac, int precision);
/* The same with every array in device memory (the structs on the host). */
int dp_dir_csda_dev(dp_ctx* ctx, const dp_physics* phys, const dp_csda_config* cfg,
                    const dp_csda_batch* batch, long n_cells, const uint8_t* shallow,
                    const double* water_fraction, double* flux, double* jac, int precision);

/* ------------------------------------------------------------------ tomography
 * Voxel-density CSDA forward model (examples/diff_flux_cube.jl:304-557):
 * ray march through a regular grid, per-segment range inversion, decay,
 * side-exit rock remainder, closed-form air, GCCLY flux, integrated over
 * energy nodes: flux_r = (1/N) sum_n 2 w_n f(E_n, q_n). */
typedef struct {
  int nx, ny, nz;
  double x0, y0, z0;         /* lower corner; z0 is the detector level */
  double dx, dy, dz;         /* pitch, m */
} dp_grid;

typedef struct {
  double ox, oy, oz;         /* start point */
  double ux, uy, uz;         /* unit direction, upward (uz > 0) */
  double cos_theta;          /* cosine of the zenith angle */
} dp_ray;

typedef struct {
  int rock_material, air_material;
  int side_cell;             /* side-exit remainder density: rho[side_cell], or
                                side_density when side_cell < 0 */
  double side_density;
  double primary_altitude;   /* m */
  int n_nodes;
  const double* node_energy; /* host pointers, n_nodes each */
  const double* node_charge;
  const double* node_weight;
  int precision;             /* DP_PREC_FP64 (0) or DP_PREC_MIXED (1) for the
                                host-pointer entry points */
} dp_tomo_params;

/* Per-ray flux.  rho: nx*ny*nz doubles (x fastest).  Host pointers. */
int dp_tomo_forward(dp_ctx* ctx, const dp_physics* phys, const dp_grid* grid,
                    const dp_tomo_params* tp, const double* rho, long n_rays,
                    const dp_ray* rays, double* flux);
/* Per-ray flux and the sparse Jacobian d flux_r / d rho_c in CSR form:
 * row_ptr[n_rays+1]; col/val hold one entry per traversed segment (a cell
 * crossed twice appears twice), in traversal order.  nnz_cap bounds col/val;
 * *nnz receives the count (DP_ERR_ARG if it exceeds nnz_cap).  Host pointers.
 * Replaces assemble_forward_and_jacobian (src/Tomography.jl:773-820) and the
 * Zygote gradient of compute_flux_gradient_cube (examples/diff_flux_cube.jl:489). */
int dp_tomo_jacobian(dp_ctx* ctx, const dp_physics* phys, const dp_grid* grid,
                     const dp_tomo_params* tp, const double* rho, long n_rays,
                     const dp_ray* rays, double* flux, int64_t* row_ptr, int32_t* col,
                     double* val, int64_t nnz_cap, int64_t* nnz);
/* Vector-Jacobian product: grad_rho[c] = sum_r cot[r] d flux_r / d rho_c,
 * with a deterministic segmented reduction (no floating-point atomics):
 * the result is bitwise reproducible.  Also returns the per-ray flux.
 * Host pointers. */
int dp_tomo_vjp(dp_ctx* ctx, const dp_physics* phys, const dp_grid* grid,
                const dp_tomo_params* tp, const double* rho, long n_rays,
                const dp_ray* rays, const double* cot, double* flux, double* grad_rho);
/* Device-pointer form of dp_tomo_vjp (traces the rays on every call; the node
 * arrays of tp are device pointers here). */
int dp_tomo_vjp_dev(dp_ctx* ctx, const dp_physics* phys, const dp_grid* grid,
                    const dp_tomo_params* tp, const double* rho, long n_rays,
                    const dp_ray* rays, const double* cot, double* flux, double* grad_rho);

/* Ray paths: the rays are traced once (geometry does not depend on rho) into a
 * device-resident CSR segment list with the CSC permutation of J^T r, the
 * analogue of precompute_paths (examples/lvd_tomography.jl:835-861).  The
 * side-exit remainder density is rho[side_cell], or the side_density of the
 * evaluation when side_cell < 0 (then its Jacobian entry has col -1). */
typedef struct dp_paths dp_paths;
int dp_tomo_paths_create(dp_ctx* ctx, const dp_grid* grid, long n_rays, const dp_ray* rays,
                         int side_cell, dp_paths** out);                 /* host rays */
int dp_tomo_paths_create_dev(dp_ctx* ctx, const dp_grid* grid, long n_rays,
                             const dp_ray* rays, int side_cell, dp_paths** out);  /* device rays */
int dp_tomo_paths_free(dp_paths* paths);
int dp_tomo_paths_info(const dp_paths* paths, long* n_rays, int64_t* nnz, int* max_segments);
/* Host copies of the segment lists (any pointer may be NULL). */
int dp_tomo_paths_csr(const dp_paths* paths, int64_t* row_ptr, int32_t* col, double* len);

#define DP_PREC_FP64 0   /* the reference's operations in FP64 (parity mode) */
#define DP_PREC_MIXED 1  /* per-segment work in FP32, FP64 range carry and flux integral */
/* One evaluation on device pointers (node arrays of tp are device pointers):
 * flux[n_rays]; if cot/grad are given, grad[ncell] = J^T cot (deterministic);
 * if jac is given, the Jacobian values in the CSR order of the paths. */
int dp_tomo_eval_dev(dp_ctx* ctx, const dp_physics* phys, const dp_paths* paths,
                     const dp_tomo_params* tp, const double* rho, const double* cot,
                     double* flux, double* grad_rho, double* jac, int precision);
/* The same with host pointers (tp->precision selects the arithmetic); the
 * inputs are copied in and the outputs out inside the call.  This is the
 * reference-facing call of an iterative solver: trace once, evaluate often. */
int dp_tomo_eval(dp_ctx* ctx, const dp_physics* phys, const dp_paths* paths,
                 const dp_tomo_params* tp, const double* rho, const double* cot, double* flux,
                 double* grad_rho, double* jac);

/* Allocation-free variant of dp_tomo_eval_dev (mixed precision): per-ray flux
 * and, when cot/grad are given, grad = J^T cot on resident paths, with device
 * pointers, without calling cudaMalloc or any allocating routine.  It has no
 * counterpart in the reference.  It is meant for callers that may not allocate
 * device memory during a call: a service holding a fixed device-memory budget,
 * or a plugin whose host process owns device memory through its own pool.
 * Its only scratch, the per-segment Jacobian values, lives in a fixed 8 MiB
 * array inside the library (held by every GPU that loads it, until exit), so
 * paths with more than 2,097,152 segments are rejected (DP_ERR_ARG) -- use
 * dp_tomo_eval_dev for those.  The first call on a device looks up that
 * array's device address (cudaGetSymbolAddress) with the device current; make
 * that first call before any stream capture.  All calls share the array and
 * every value is rewritten before it is read, so nothing needs clearing, but
 * calls that overlap on the GPU (other contexts or streams at the same time)
 * race on it.  The address looked up is the one in the device's primary
 * context (the CUDA runtime's): after a cudaDeviceReset the process must not
 * call this entry point again. */
int dp_tomo_eval_noalloc_dev(dp_ctx* ctx, const dp_physics* phys, const dp_paths* paths,
                             const dp_tomo_params* tp, const double* rho, const double* cot,
                             double* flux, double* grad_rho);

/* ------------------------------------------------------------------ plain baseline
 * Plain FP64 GPU form used as the speed-up denominator: one kernel launch per
 * ray, one thread per energy node, tables read from global memory with binary
 * search, no staging, no batching.  Device pointers; flux only. */
int dp_tomo_forward_plain_dev(dp_ctx* ctx, const dp_physics* phys, const dp_grid* grid,
                              const dp_tomo_params* tp, const double* rho, long n_rays,
                              const dp_ray* rays, double* flux);

/* ------------------------------------------------------------------ inversion loops
 * Consumers of the forward model and its Jacobian (src/Tomography_inverse.jl)
 * on resident paths, the unknown being the voxel density:
 *   DP_SOLVE_SART  rho <- clamp(rho + relaxation D_col J^T D_row (obs - f(rho)), box),
 *                  D_row = 1/sum_j|J_ij|, D_col = 1/sum_i|J_ij| (sart_reconstruct,
 *                  :98-132), with J re-evaluated at every iterate;
 *   DP_SOLVE_GN    Gauss-Newton / Levenberg-Marquardt on 0.5 sum_i W_i (f_i - obs_i)^2
 *                  (gauss_newton_reconstruct, :448-603, legacy acceptance), the
 *                  damped normal equations solved matrix-free by preconditioned
 *                  conjugate gradients on the device (no dense J^T W J);
 *   DP_SOLVE_MLEM  mlem_reconstruct (:153-188) on the model linearised at the
 *                  iterate: with A = -J (the density lowers the flux, so A >= 0)
 *                  and b = max(f(rho_k) + A rho_k - obs, 0) (obs = f(rho) is
 *                  then A rho = b), rho <- clamp(rho * A^T (b / max(A rho, 1e-12))
 *                  / (A^T 1 + max(dR/drho, 0)), box), zero column sums counting
 *                  as 1, the start lifted to at least 1e-6.  The multiplicative
 *                  step solves the linearised problem: it need not lower the
 *                  flux misfit of the nonlinear model;
 *   DP_SOLVE_GD    gradient_descent_reconstruct (:324-400) with its optimizers:
 *                  g = J^T W (f - obs) + dR/drho; PGD scales g by the
 *                  Gauss-Newton + prior diagonal and takes the exact step of the
 *                  local quadratic along it, capped at lr, and stops when the
 *                  objective changes by at most 1e-5 of itself; Adam (0.9,
 *                  0.999, 1e-8) and plain steps of lr otherwise.
 * MLEM and GD re-evaluate f and J at every iterate, or with fixed_linearization
 * use f0 + J0 (rho - rho0) (the reference's relinearize = false; MLEM's fixed
 * A, b).  history[k] is the flux misfit ||f(rho_k) - obs|| at iterate k (GD
 * with fixed_linearization: of the linear model it iterates on; NaN past an
 * early stop).  No
 * reference entry point takes this exact form: it replaces the solver loops
 * around make_csda_operator (:614-626) for the voxel-density model. */
#define DP_SOLVE_SART 0
#define DP_SOLVE_GN 1
#define DP_SOLVE_MLEM 2
#define DP_SOLVE_GD 3
#define DP_GD_PGD 0      /* diagonally preconditioned projected gradient, exact step */
#define DP_GD_ADAM 1
#define DP_GD_PLAIN 2    /* w <- clamp(w - lr g, box) */
typedef struct {
  int method;            /* DP_SOLVE_SART, DP_SOLVE_GN, DP_SOLVE_MLEM or DP_SOLVE_GD */
  int n_iter;            /* outer iterations */
  int cg_iter;           /* GN: conjugate-gradient iterations per solve (<= 0: 10) */
  int precision;         /* forward model: DP_PREC_FP64 or DP_PREC_MIXED */
  double relaxation;     /* SART relaxation (<= 0: 0.2) */
  double lm_damping;     /* GN initial damping (<= 0: 1e-3) */
  double box_lo, box_hi; /* density bounds, kg/m^3 */
  double prior_weight;   /* > 0: smoothness prior weight * sum over the grid's
                            6-neighbour edges of (rho_i - rho_j)^2 (SmoothnessPrior,
                            src/Tomography_inverse.jl:17-79): GN objective term,
                            SART smoothing sweep */
  double smooth_strength; /* SART sweep strength (<= 0: 0.1) */
  int no_speculation;     /* GN: 0 (default) evaluates the first line-search trial
                             with its Jacobian while the iterations' first trials
                             keep being accepted (the accepted trial's Jacobian is
                             the next iteration's); 1 never does.  The iterates
                             are the same either way. */
  int optimizer;          /* GD: DP_GD_PGD (default), DP_GD_ADAM or DP_GD_PLAIN */
  int fixed_linearization; /* MLEM, GD: 0 re-evaluates f and J at every iterate
                              (relinearize = true); 1 linearises once at the start,
                              f(rho) ~ f0 + J0 (rho - rho0) (relinearize = false) */
  double lr;              /* GD: step (PGD: step-length cap); <= 0: 1 for PGD, 1e-2 else */
} dp_solve_params;
/* obs: n_rays observed fluxes, weight: n_rays data weights (NULL: 1), rho:
 * the start density in, the estimate out (all device pointers; node arrays of
 * tp on the device).  history (host, n_iter + 1 values, may be NULL): the misfit
 * ||obs - f(rho)|| before each iteration and after the last; NaN where a
 * Gauss-Newton loop stopped early (no accepted step). */
int dp_tomo_solve_dev(dp_ctx* ctx, const dp_physics* phys, const dp_paths* paths,
                      const dp_tomo_params* tp, const double* obs, const double* weight,
                      double* rho, const dp_solve_params* sp, double* history);

#ifdef __cplusplus
}
#endif
#endif /* DPGPU_H */
