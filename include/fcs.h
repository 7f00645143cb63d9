/*
 * fcs.h -- C ABI of the GB300 stiff-chemistry library (libfcs_cuda.so).
 *
 * This is the boundary an OpenFOAM-side chemistry model binds to.  It
 * replaces, for a whole batch of cells at once, the per-cell solver contract
 * of the FastChemistrySolver plugin:
 *
 *   virtual void solve(scalar& p, scalar& T, scalarField& Y, label li,
 *                      scalar& deltaT, scalar& subDeltaT) const;
 *       (src/ChemistryModel/FastChemistryModel.H:375-383, implemented by
 *        src/ODE/OptRodas34/OptRodas34.C:57-121,
 *        src/ODE/OptRosenbrock34/OptRosenbrock34.C:61-125,
 *        src/ODE/OptSeulex/OptSeulex.C:103-169)
 *
 * together with the cell loop that drives it,
 *
 *   scalar FastChemistryModel::solve(const scalar deltaT)
 *       (src/ChemistryModel/FastChemistryModel_transientSolve.H:2-104)
 *
 * and the mechanism loader OptReaction::readInfo
 *       (src/Reaction/OptReaction.C:348-1339).
 *
 * Conventions
 *   - Every function returns an fcs_status; nothing aborts.  A failure in
 *     individual cells is reported per cell through cell_status and by the
 *     FCS_ERR_CELLS return code; the other cells are still written.
 *   - All arrays are owned by the caller.  Unless FCS_PTR_DEVICE is passed
 *     they are host pointers and the library copies them to and from its own
 *     device buffers.  With FCS_PTR_DEVICE they are device pointers on the
 *     context's GPU and are used in place.
 *   - Species-major layout: Y[i * n_cells + c] is species i of cell c (one
 *     contiguous OpenFOAM field per species).
 *   - One context per host thread; calls on one context are serialised.
 *     While a step of fcs_integrate_async is in flight, the entry points that
 *     use the context's buffers return FCS_ERR_STATE until fcs_sync.
 */
#ifndef FCS_H
#define FCS_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fcs_ctx fcs_ctx;
typedef int32_t fcs_status;

enum {
    FCS_OK = 0,
    FCS_ERR_INVALID = 1,      /* bad argument or option                       */
    FCS_ERR_CUDA = 2,         /* CUDA runtime error (see fcs_last_error_string)*/
    FCS_ERR_NOMEM = 3,        /* device or host allocation failed             */
    FCS_ERR_STATE = 4,        /* call out of order (e.g. no mechanism loaded) */
    FCS_ERR_CELLS = 5,        /* some cells failed; see cell_status           */
    FCS_ERR_UNSUPPORTED = 6,  /* reaction type or size not supported          */
    FCS_ERR_PARSE = 7,        /* OpenFOAM dictionary could not be read        */
    FCS_ERR_TIMEOUT = 8       /* fcs_sync_timeout: the step is still running  */
};

/* Per-cell status codes (cell_status output). */
enum {
    FCS_CELL_OK = 0,
    FCS_CELL_MAX_STEPS = 1,   /* maxSteps exceeded (fatal in the reference, OptRodas34.C:193) */
    FCS_CELL_NONFINITE = 2,   /* NaN/Inf met in the state or the error norm          */
    FCS_CELL_DT_UNDERFLOW = 3,/* step size collapsed / too many rejected attempts    */
    FCS_CELL_SKIPPED = 4      /* T <= Treact: not integrated, RR = 0                  */
};

/* Reaction kinds of fcs_mechanism_desc.type (OpenFOAM type names without the
 * reversible/irreversible prefix). */
enum {
    FCS_RXN_ARRHENIUS = 0,           /* (ir)reversibleArrhenius                    */
    FCS_RXN_THIRD_BODY = 1,          /* (ir)reversibleThirdBodyArrhenius           */
    FCS_RXN_PLOG = 2,                /* (ir)reversibleArrheniusPLOG                */
    FCS_RXN_LINDEMANN_FALLOFF = 3,   /* (ir)reversibleArrheniusLindemannFallOff    */
    FCS_RXN_TROE_FALLOFF = 4,        /* (ir)reversibleArrheniusTroeFallOff         */
    FCS_RXN_SRI_FALLOFF = 5,         /* (ir)reversibleArrheniusSRIFallOff          */
    FCS_RXN_NONEQ = 6,               /* nonEquilibriumReversibleArrhenius: forward
                                        and reverse rates both Arrhenius (no Kc)  */
    FCS_RXN_NONEQ_THIRD_BODY = 7     /* nonEquilibriumReversibleThirdBodyArrhenius */
};

enum { FCS_SOLVER_RODAS34 = 0, FCS_SOLVER_ROSENBROCK34 = 1, FCS_SOLVER_SEULEX = 2,
       FCS_SOLVER_RODAS23 = 3,        /* src/ODE/OptRodas23/OptRodas23.C:202-315       */
       FCS_SOLVER_ROSENBROCK23 = 4 }; /* src/ODE/OptRosenbrock23/OptRosenbrock23.C:208-298 */
enum { FCS_JACOBIAN_EXACT = 0, FCS_JACOBIAN_FAST = 1 };
/* FCS_PRECISION_MIXED: the iteration matrix factored in FP32 (power-of-two
 * row and column equilibration), one FP64-residual refinement sweep per
 * linear solve against the FP64 Jacobian; an attempt whose correction is not
 * small is redone in FP64.  Rates, thermo, equilibrium constants, the
 * Jacobian assembly, state and the step controller stay FP64. */
enum { FCS_PRECISION_FP64 = 0, FCS_PRECISION_MIXED = 1 };
/* Cell-to-thread mapping: AUTO lets the autotuner choose.  LANE: one thread
 * per cell, the cells' working sets in a global-memory workspace interleaved
 * across the lanes of a warp (Rosenbrock-family solvers, FP64 or mixed); the others:
 * a group of 32..256 threads per cell with its working set in shared memory
 * (or in global memory when it does not fit). */
enum { FCS_MAPPING_AUTO = 0, FCS_MAPPING_LANE = 1, FCS_MAPPING_WARP = 32, FCS_MAPPING_BLOCK64 = 64,
       FCS_MAPPING_BLOCK128 = 128, FCS_MAPPING_BLOCK256 = 256 };

/* flags for fcs_integrate */
enum {
    FCS_PTR_DEVICE = 1,        /* all array arguments are device pointers       */
    FCS_NO_QUEUE_SORT = 2,     /* keep natural cell order in the work queue
                                  (default: reacting cells ordered by predicted
                                  step count delta_t / sub_delta_t, largest first) */
    FCS_CUDA_GRAPH = 4         /* with FCS_PTR_DEVICE: run the step as one CUDA
                                  graph (counters, classify, queue, integrator,
                                  statistics), captured on the first call and
                                  replayed while the arrays, n_cells, delta_t and
                                  options stay the same; the mapping is the
                                  option's, else one the autotuner already chose,
                                  else the default */
};

/*
 * Mechanism in OpenFOAM file order.  The library reorders the reactions into
 * the type blocks of OptReaction::readInfo (OptReaction.C:348-1339): constant
 * Arrhenius (beta == 0 and Ta == 0) first, then the other Arrhenius,
 * non-equilibrium, non-equilibrium third-body, third-body, fall-off, then
 * PLOG.  Stoichiometric coefficients are expanded
 * into repeated species entries exactly as readReactionInfo does
 * (OptReaction.C:29-173).  The host keeps ownership; the library copies.
 */
typedef struct fcs_mechanism_desc {
    int32_t n_species;
    int32_t n_reactions;
    const double* W;             /* [Ns] molecular weight, kg/kmol              */
    const double* T_low;         /* [Ns]                                        */
    const double* T_high;        /* [Ns]                                        */
    const double* T_common;      /* [Ns]                                        */
    const double* high_coeffs;   /* [Ns*7] NASA-7 (janaf) high-T coefficients   */
    const double* low_coeffs;    /* [Ns*7] NASA-7 low-T coefficients            */
    const int32_t* type;         /* [R] FCS_RXN_*                               */
    const int32_t* reversible;   /* [R] 1 = reversible, 0 = irreversible        */
    const int32_t* lhs_offset;   /* [R+1]                                       */
    const int32_t* lhs_species;  /* reactant species, repeated by coefficient   */
    const int32_t* rhs_offset;   /* [R+1]                                       */
    const int32_t* rhs_species;  /* product species, repeated by coefficient    */
    const double* arrhenius;     /* [R*3] A, beta, Ta (k0 for fall-off, the
                                    forward rate for non-equilibrium)           */
    const double* arrhenius2;    /* [R*3] kInf A, beta, Ta for fall-off, the
                                    reverse rate for non-equilibrium; may be NULL
                                    when neither kind occurs                    */
    const double* efficiencies;  /* [R*Ns] third-body efficiencies (row used for
                                    third-body, fall-off and non-equilibrium
                                    third-body reactions; the latter use it for
                                    both directions, as the reference reads the
                                    reverse list from the forward dictionary,
                                    OptReaction.C:678); may be NULL */
    const double* falloff_params;/* [R*5] Troe alpha,Ts,Tss,Tsss / SRI a,b,c,d,e */
    const int32_t* plog_offset;  /* [R+1] rows of plog_table per reaction       */
    const double* plog_table;    /* [rows*4] p, A, beta, Ta (ArrheniusData)     */
} fcs_mechanism_desc;

/* chemistryProperties keys: chemistryType{solver}, jacobian, Treact,
 * initialChemicalTimeStep (used by the caller to seed subDeltaT),
 * maxChemicalTimeStep, <Solver>Coeffs{absTol, relTol, maxSteps}; plus the
 * GPU-only keys precision and mapping. */
typedef struct fcs_options {
    int32_t solver;              /* FCS_SOLVER_*                      */
    int32_t jacobian;            /* FCS_JACOBIAN_*                    */
    int32_t precision;           /* FCS_PRECISION_*                   */
    int32_t mapping;             /* FCS_MAPPING_*                     */
    double abs_tol;
    double rel_tol;
    int32_t max_steps;           /* default 10000                     */
    int32_t max_rejects;         /* bound on rejected retries per step (GPU-only, default 1000) */
    double T_react;              /* cells with T <= Treact are skipped */
    double delta_t_chem_max;     /* maxChemicalTimeStep (default 1e300) */
} fcs_options;

/* Per-call statistics, summed over cells. */
typedef struct fcs_step_stats {
    int64_t cells_integrated;
    int64_t cells_skipped;
    int64_t cells_failed;
    int64_t attempts;            /* attempted steps (accepted + rejected) */
    int64_t accepted;
    int64_t jacobians;
    int64_t lu_decompositions;
    int64_t rhs_evaluations;
    int64_t linear_solves;
    int64_t fp64_fallbacks;      /* mixed precision: attempts (Rosenbrock) or cells (Seulex)
                                    redone in FP64 after a failed refinement check */
    double  kernel_ms;           /* device time of the integration kernel */
    double  call_ms;             /* device time of the whole call on the library's
                                    stream, host<->device copies included */
    int32_t mapping;             /* threads per cell used (autotuned for AUTO) */
    int32_t reserved;
} fcs_step_stats;

fcs_status fcs_create(fcs_ctx** ctx, int device);
fcs_status fcs_destroy(fcs_ctx* ctx);
const char* fcs_last_error_string(const fcs_ctx* ctx);
const char* fcs_version(void);

/* Replaces OptReaction::readInfo (OptReaction.C:348-1339). */
fcs_status fcs_load_mechanism(fcs_ctx* ctx, const fcs_mechanism_desc* desc);

/* Reads an OpenFOAM `reactions` dictionary file and a physicalProperties /
 * speciesThermo file (species list + per-species specie/thermodynamics
 * sub-dictionaries) and loads the mechanism, like the plugin constructor
 * (FastChemistryModel.C:110 -> OptReaction.C:348). */
fcs_status fcs_load_mechanism_foam(fcs_ctx* ctx, const char* reactions_path,
                                   const char* thermo_path);

/* Host only (no context, no device): parses the same two files as
 * fcs_load_mechanism_foam and hands the flat description and the species
 * names (thermo-file order) to `visit`, whose status is returned.  The arrays
 * are valid during the call only.  For callers that inspect, convert or keep
 * a mechanism without loading it. */
typedef fcs_status (*fcs_mechanism_visitor)(const fcs_mechanism_desc* desc,
                                            const char* const* species_names, void* user);
fcs_status fcs_parse_mechanism_foam(const char* reactions_path, const char* thermo_path,
                                    fcs_mechanism_visitor visit, void* user);

/* Reads the chemistryProperties keys of the plugin (FastChemistryModel.C:45-168,
 * OptRodas34.C:34-50) into opts: chemistryType{solver}, jacobian, Treact,
 * <Solver>Coeffs{absTol,relTol,maxSteps}, maxChemicalTimeStep and the optional
 * FastChemistryGPU{precision, mapping} sub-dictionary.  Unknown keys (balance,
 * Iter, DLBthreshold, ...) are accepted and ignored.  initial_sub_dt receives
 * initialChemicalTimeStep (or -1 when absent). */
fcs_status fcs_read_chemistry_properties(const char* path, fcs_options* opts,
                                         double* initial_sub_dt);

fcs_status fcs_default_options(fcs_options* opts);
fcs_status fcs_set_options(fcs_ctx* ctx, const fcs_options* opts);

/* Number of species / reactions of the loaded mechanism. */
fcs_status fcs_mechanism_size(const fcs_ctx* ctx, int32_t* n_species, int32_t* n_reactions);

/* hf[Ns]: each species' formation enthalpy at 298.15 K in J/kg, as
 * specieThermo::Hf() gives it; the chemistry model's Qdot() is
 * -sum_i hf_i RR_i over the last solve's RR (FastChemistryModel.C:656-685). */
fcs_status fcs_formation_enthalpy(fcs_ctx* ctx, double* hf);

/*
 * Integrate n_cells independent constant-pressure cells over delta_t.
 * Batched form of FastChemistryModel::solve(deltaT) (transientSolve.H:30-104):
 *   in:  p[n], rho0[n], T[n], Y[Ns*n], sub_delta_t[n] (deltaTChem_)
 *   out: T, Y (new state, Y clamped >= 0), sub_delta_t (next initial sub-step,
 *        capped at maxChemicalTimeStep), RR[Ns*n] = (Y - Y0) * rho0 / delta_t
 *        (may be NULL), cell_status[n] (may be NULL), stats (may be NULL),
 *        delta_t_min = min(min over integrated cells of the uncapped
 *        sub-step, 2*delta_t) (may be NULL).
 */
fcs_status fcs_integrate(fcs_ctx* ctx, int64_t n_cells, double delta_t,
                         const double* p, const double* rho0,
                         double* T, double* Y, double* sub_delta_t,
                         double* RR, int32_t* cell_status,
                         fcs_step_stats* stats, double* delta_t_min,
                         int32_t flags);

/*
 * fcs_integrate over caller-owned DEVICE arrays, enqueued on `cuda_stream`
 * (a cudaStream_t of the context's device; NULL = the context's own stream)
 * without waiting for it: the flow solver can overlap the chemistry with its
 * own work, and order its next kernels after it on the same stream.  The
 * step's results are in T, Y, sub_delta_t, RR, cell_status once the stream
 * reaches them; fcs_sync waits for the step and returns its statistics and
 * delta_t_min (same meaning as fcs_integrate's).  One step in flight per
 * context: a second fcs_integrate_async before fcs_sync returns
 * FCS_ERR_STATE.  The mapping is the option's, else one the autotuner already
 * chose for this context, else the default (the autotuner needs a host round
 * trip and is not run here).  flags: FCS_NO_QUEUE_SORT.
 */
fcs_status fcs_integrate_async(fcs_ctx* ctx, int64_t n_cells, double delta_t,
                               const double* p, const double* rho0,
                               double* T, double* Y, double* sub_delta_t,
                               double* RR, int32_t* cell_status, int32_t flags,
                               void* cuda_stream);
fcs_status fcs_sync(fcs_ctx* ctx, fcs_step_stats* stats, double* delta_t_min);

/*
 * fcs_sync with a bounded host-side wait (no counterpart in the reference,
 * whose only failure path is the fatal maxSteps, OptRodas34.C:193): waits at
 * most timeout_ms for the step of fcs_integrate_async.  If the step has not
 * completed by then it returns FCS_ERR_TIMEOUT and the step stays in flight
 * (the kernels are not interrupted); a later fcs_sync or fcs_sync_timeout
 * collects it.  While a step is in flight every other entry point that uses
 * the context's buffers returns FCS_ERR_STATE.
 */
fcs_status fcs_sync_timeout(fcs_ctx* ctx, double timeout_ms, fcs_step_stats* stats, double* delta_t_min);

/* Same, with a per-cell delta_t (the local-time-stepping variant
 * FastChemistryModel::solve(const scalarField& deltaT),
 * FastChemistryModel_localEulerSolve.H:3-101). */
fcs_status fcs_integrate_lts(fcs_ctx* ctx, int64_t n_cells, const double* delta_t,
                             const double* p, const double* rho0,
                             double* T, double* Y, double* sub_delta_t,
                             double* RR, int32_t* cell_status,
                             fcs_step_stats* stats, double* delta_t_min,
                             int32_t flags);

/*
 * fcs_integrate_noalloc -- no counterpart in the reference.
 *
 * fcs_integrate over caller-owned DEVICE arrays that allocates no device
 * memory: no cudaMalloc/cudaFree and no allocating library routine, on any
 * call.  For callers that cannot allocate during a time step: a flow solver
 * that gives all free device memory to its own pool at start-up, and one
 * whose other streams must not be stalled by the device-wide synchronisation
 * of cudaMalloc/cudaFree when fcs_integrate's grow-only buffers grow.
 *
 * Same arguments and results as fcs_integrate with FCS_PTR_DEVICE (p, rho0,
 * T, Y, sub_delta_t, RR, cell_status are device or managed memory of the
 * context's device; stats and delta_t_min are host).  The step counters,
 * minimum sub-step, work-queue head and queue of reacting cells live in one
 * fixed device array of this library, per device, so:
 *   - n_cells is at most FCS_NOALLOC_MAX_CELLS (4 MiB of queue); larger
 *     calls return FCS_ERR_INVALID without doing anything;
 *   - the per-cell workspace must fit in shared memory (about 140 species
 *     for the Rosenbrock solvers in FP64, 120 mixed, 100 for Seulex, with
 *     about seven reactions per species); otherwise FCS_ERR_UNSUPPORTED;
 *   - the call zeroes the counters and queue head itself before its kernels;
 *     nothing has to be cleared by the caller;
 *   - calls that overlap in time on the same device (two host threads, or two
 *     contexts) race on that array and must be serialised by the caller;
 *     consecutive calls from one thread are safe (each call returns after its
 *     work has finished);
 *   - the mapping autotuner is not run (it allocates trial copies): the
 *     mapping is fcs_options.mapping, else one the autotuner already cached in
 *     this context, else the default for the mechanism size;
 *   - the first call on a device looks up the array's address (which may load
 *     this library's device code); make it before any stream capture begins.
 */
#define FCS_NOALLOC_MAX_CELLS 1048576
/* (continued) The first launch of each kernel variant (mapping x precision x
 * solver family) in a process may make the CUDA driver enlarge the
 * context's local-memory reservation for the kernel's stack frame.  Make one
 * call for each mapping and precision the run will use before the flow
 * solver's pool takes the remaining device memory. */
fcs_status fcs_integrate_noalloc(fcs_ctx* ctx, int64_t n_cells, double delta_t,
                                 const double* p, const double* rho0,
                                 double* T, double* Y, double* sub_delta_t,
                                 double* RR, int32_t* cell_status,
                                 fcs_step_stats* stats, double* delta_t_min);

/*
 * Test hook (host side only; no counterpart in the reference): the next
 * `count` growths of the library's device buffers, in any context of this
 * process, fail as if cudaMalloc had returned cudaErrorMemoryAllocation.  The
 * entry point that needed the buffer returns FCS_ERR_NOMEM; the mechanism,
 * the options and the other buffers stay as they were, and the next call
 * allocates again.  0 clears it.
 */
fcs_status fcs_test_fail_allocations(int32_t count);

/*
 * Right-hand side of the mass-fraction ODE system at each cell state:
 * dydt[(Ns+1)*n] (species-major, row Ns is dT/dt).  Mirrors
 * FastChemistryModel::derivatives (FastChemistryModel.C:194-273) on top of
 * OptReaction::dNdtByV (ReactionRate.C:732-1503).  Y is read-only here (the
 * in-place max(Y,0) clamp of the reference acts on a copy).
 */
fcs_status fcs_rhs(fcs_ctx* ctx, int64_t n_cells, const double* p, const double* T,
                   const double* Y, double* dydt, int32_t flags);

/*
 * Analytic Jacobian of the mass-fraction system: J[n][(Ns+1)*(Ns+1)] row-major
 * per cell, and f = dydt[(Ns+1)*n] species-major.  Mirrors
 * FastChemistryModel::jacobian (FastChemistryModel.C:489-572) on top of
 * OptReaction::ddNdtByVdcTp (Jacobian.C:5-1004) and the dC/dY conversion
 * (Jacobian.C:1943-2059, 2814-2858, 3709-3793, 4541-4568).
 */
fcs_status fcs_jacobian(fcs_ctx* ctx, int64_t n_cells, const double* p, const double* T,
                        const double* Y, double* J, double* dydt, int32_t flags);

/*
 * Instantaneous source terms (FastChemistryModel::calculate(),
 * FastChemistryModel.C:715-755): c_i = rho Y_i / W_i (Y not clamped),
 * RR[i*n+c] = dNdtByV_i * W_i (kg/m^3/s), and the heat release
 * Qdot[c] = -sum_i Hf_i RR_i with Hf_i the formation enthalpy at 298.15 K
 * (FastChemistryModel.C:656-685).  Qdot may be NULL.
 */
fcs_status fcs_rates(fcs_ctx* ctx, int64_t n_cells, const double* p, const double* T,
                     const double* rho, const double* Y, double* RR, double* Qdot,
                     int32_t flags);

/*
 * Chemical time scale per cell (FastChemistryModel::tc(),
 * FastChemistryModel.C:589-651, over OptReaction::Tc, Tc.C:3-834):
 * c_i = rho Y_i / W_i; for every reaction wf = n_products Kf prod(c_reactants)
 * and wr = n_reactants Kr prod(c_products) (Kc clamped at 1.49011611938476e-8);
 * tc = sum(wf + wr) / sum(wf^2 + wr^2) * sum_i c_i, or 1e300 when no reaction
 * runs.  tc[n].
 */
fcs_status fcs_tc(fcs_ctx* ctx, int64_t n_cells, const double* p, const double* T, const double* rho,
                  const double* Y, double* tc, int32_t flags);

#ifdef __cplusplus
}
#endif
#endif /* FCS_H */
