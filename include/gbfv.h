/*
 * gbfv.h -- C ABI of the GB300-native ECFV/TPFA linearizer and Newton linear
 * solve (BiCGStab + block ILU0).
 *
 * Everything here is plain C: pointers, sizes and status codes.  Host arrays
 * are in the reference's natural (grid index) order; device-side layouts are
 * private to the library.
 *
 * Reference interfaces each group of entry points replaces (paths inside
 * OPM/opm-models):
 *   - problem description   : tests/problems/lensproblem.hh:227-627,
 *                             tests/problems/reservoirproblem.hh:215-736
 *                             (what Problem::intrinsicPermeability/porosity/
 *                             materialLawParams/boundary/constraints return)
 *   - gbfv_linearize & co.  : opm/models/discretization/common/
 *                             fvbaselinearizer.hh:133-375 (FvBaseLinearizer)
 *   - gbfv_solve & co.      : opm/simulators/linalg/parallelbasebackend.hh:
 *                             137-290 (prepare/setResidual/setMatrix/solve)
 *   - gbfv_newton_*         : opm/models/nonlinear/newtonmethod.hh:228-845,
 *                             opm/models/blackoil/blackoilnewtonmethod.hh:
 *                             176-427
 *   - gbfv_time_integration : opm/models/discretization/common/
 *                             fvbaseproblem.hh:512-606
 */
#ifndef GBFV_H
#define GBFV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* status codes (the reference throws; every entry point here returns)  */
/* ------------------------------------------------------------------ */
enum gbfv_status {
    GBFV_OK = 0,
    GBFV_ERR_ARG = 1,           /* invalid argument / size                  */
    GBFV_ERR_CUDA = 2,          /* CUDA runtime error                       */
    GBFV_ERR_OOM = 3,           /* device allocation failed                 */
    GBFV_ERR_NUMERICAL = 4,     /* Opm::NumericalProblem equivalent         */
    GBFV_ERR_NONFINITE = 5,     /* non-finite residual / update             */
    GBFV_ERR_BREAKDOWN = 6,     /* BiCGStab breakdown (bicgstabsolver.hh)   */
    GBFV_ERR_NOT_CONVERGED = 7, /* linear solver returned false             */
    GBFV_ERR_TIMEOUT = 8,       /* a bounded device-side wait expired       */
    GBFV_ERR_UNSUPPORTED = 9,   /* input outside what the kernels handle    */
    GBFV_ERR_SINGULAR = 10,     /* ILU0 pivot block could not be inverted   */
    GBFV_ERR_NO_DEVICE = 11     /* no CUDA device visible                   */
};

/* models (Properties::Model of the reference's type tags) */
enum gbfv_model {
    GBFV_MODEL_IMMISCIBLE_2P = 0, /* opm/models/immiscible, 2 phases, b = 2 */
    GBFV_MODEL_BLACKOIL_3P = 1    /* opm/models/blackoil, 3 phases,  b = 3  */
};

/* material laws (opm-common MaterialLaw of the problems) */
enum gbfv_law {
    GBFV_LAW_REG_VAN_GENUCHTEN = 0, /* EffToAbsLaw<RegularizedVanGenuchten> */
    GBFV_LAW_REG_BROOKS_COREY = 1,  /* EffToAbsLaw<RegularizedBrooksCorey>  */
    GBFV_LAW_COREY3P = 2            /* 3-phase Corey kr, zero p_c (black-oil)*/
};

/* boundary condition kinds (ImmiscibleBoundaryRateVector setters) */
/* flux module (Properties::FluxModule): Darcy (darcyfluxmodule.hh:183-525,
 * the default) or two-point transmissibilities (transfluxmodule.hh:201-480,
 * used by lens_immiscible_ecfv_ad_trans.cc:55-58; immiscible model only)   */
enum gbfv_flux {
    GBFV_FLUX_DARCY = 0,
    GBFV_FLUX_TRANS = 1
};

enum gbfv_bc {
    GBFV_BC_NOFLOW = 0,   /* setNoFlow()                                    */
    GBFV_BC_FREEFLOW = 1, /* setFreeFlow(fs): Dirichlet state (p_w, S_w)    */
    GBFV_BC_MASSRATE = 2  /* setMassRate(rate) [kg/(m^2 s)] per equation    */
};

/* black-oil primary-variable meanings (blackoilprimaryvariables.hh) */
enum gbfv_pv_meaning {
    GBFV_WATER_SW = 0,
    GBFV_PRESSURE_PO = 0,
    GBFV_GAS_SG = 0,
    GBFV_GAS_RS = 1,
    GBFV_GAS_RV = 2
};

/* solve precision */
enum gbfv_precision {
    GBFV_PREC_FP64 = 0,  /* everything FP64 (plain form)                      */
    GBFV_PREC_MIXED = 1  /* FP64 outer refinement around FP32 BiCGStab/ILU0    */
};

/* material-law parameter record: GBFV_MAT_STRIDE doubles per material */
#define GBFV_MAT_STRIDE 8
/*  [0] law (enum gbfv_law, stored as double)
 *  two-phase laws:  [1] S_wr  [2] S_nr
 *    van Genuchten: [3] alpha [1/Pa]   [4] n
 *    Brooks-Corey:  [3] entry pressure p_e [Pa]   [4] lambda
 *  3-phase Corey:   [4] exponent  (residual saturations zero)              */

/* black-oil PVT (BlackOilFluidSystem with LiveOilPvt / DryGasPvt /
 * ConstantCompressibilityWaterPvt, reservoirproblem.hh:223-327)          */
typedef struct gbfv_blackoil_pvt {
    double rho_ref_oil, rho_ref_water, rho_ref_gas; /* surface densities     */
    int32_t n_oil;            /* rows of the saturated live-oil table        */
    const double* oil_p;      /* [n_oil] pressure [Pa], increasing           */
    const double* oil_rs;     /* [n_oil] saturated R_s, increasing           */
    const double* oil_bo;     /* [n_oil] saturated B_o                       */
    const double* oil_mu;     /* [n_oil] saturated viscosity [Pa s]          */
    double oil_compressibility; /* undersaturated d(1/B_o)/dp / (1/B_o) [1/Pa]*/
    int32_t n_gas;
    const double* gas_p;      /* [n_gas] pressure [Pa], increasing           */
    const double* gas_bg;     /* [n_gas] B_g                                 */
    const double* gas_mu;     /* [n_gas] viscosity [Pa s]                    */
    double water_p_ref, water_bw_ref, water_compressibility, water_mu;
} gbfv_blackoil_pvt;

/* The problem: geometry, rock, boundary and constraint data of one grid.
 * Cells and faces follow the reference's element / intersection order
 * (YaspGrid: x fastest; intersections -x,+x,-y,+y,-z,+z).                */
typedef struct gbfv_problem {
    int32_t model;            /* enum gbfv_model                             */
    int32_t num_cells;
    int32_t num_conn;         /* interior intersections (2 per interior face)*/
    int32_t num_bfaces;       /* boundary intersections                      */
    /* cells */
    const double* center;     /* [num_cells*3] cell centre (z = 0 in 2D)     */
    const double* volume;     /* [num_cells]                                 */
    const double* porosity;   /* [num_cells]                                 */
    const double* perm;       /* [num_cells*3] diagonal of K                 */
    const int32_t* material;  /* [num_cells] index into material_params      */
    /* interior intersections, grouped per cell, in intersection order     */
    const int32_t* conn_ptr;  /* [num_cells+1]                               */
    const int32_t* conn_nbr;  /* [num_conn] neighbour cell                   */
    const int32_t* conn_dir;  /* [num_conn] local intersection index (0..5)  */
    const double* conn_normal;/* [num_conn*3] unit outer normal              */
    const double* conn_center;/* [num_conn*3] integration point              */
    const double* conn_area;  /* [num_conn]                                  */
    /* boundary intersections, grouped per cell, in intersection order     */
    const int32_t* bface_ptr; /* [num_cells+1]                               */
    const double* bface_normal;/* [num_bfaces*3]                             */
    const double* bface_center;/* [num_bfaces*3]                             */
    const double* bface_area; /* [num_bfaces]                                */
    const int32_t* bface_type;/* [num_bfaces] enum gbfv_bc                   */
    const double* bface_value;/* [num_bfaces*4] FREEFLOW: p_w, S_w;
                                 MASSRATE: rate per equation                 */
    /* constraints (FvBaseConstraints; wells of the reservoir problem)     */
    const int32_t* constraint;/* [num_cells] -1 = free, else row of below     */
    int32_t num_constraints;
    const double* constraint_pv;        /* [num_constraints*3]               */
    const int32_t* constraint_meaning;  /* [num_constraints] gas meaning      */
    /* parameters */
    double gravity[3];
    int32_t num_materials;
    const double* material_params;      /* [num_materials*GBFV_MAT_STRIDE]   */
    double rho[2], mu[2];     /* immiscible: constant liquid density/visc.   */
    const gbfv_blackoil_pvt* pvt; /* black-oil only, else NULL               */
    double temperature;
    int32_t flux_module;      /* enum gbfv_flux: Properties::FluxModule      */
    /* Vertex-centred finite volumes (VcfvDiscretization with the stencil of
     * vcfvstencil.hh:466-1390): num_elements > 0 selects it; 2D
     * axis-aligned quadrilaterals, the immiscible model.  The cells above
     * are then the grid's vertices, its degrees of freedom: centre = the
     * vertex position, porosity / perm / material at the vertex, volume not
     * read (the library sums each vertex's sub-control volumes), num_conn 0,
     * no constraints.  Each element lists its corner vertices in the
     * reference element's order: corner c at lower + (c&1, (c>>1)&1) .*
     * (upper - lower).  The boundary arrays then hold the boundary
     * sub-control-volume faces grouped per element (bface_ptr has
     * num_elements + 1 entries): per boundary intersection of the element
     * in intersection order, one face per corner of the intersection, with
     * that corner (bface_corner), the face's integration point
     * (bface_center: half way from the corner to the intersection's
     * centre), the intersection's unit outer normal, half its area, and the
     * condition the problem's boundary() gives at the integration point.   */
    int32_t num_elements;
    const int32_t* elem_corner;  /* [num_elements*4] vertex of each corner  */
    const int32_t* bface_corner; /* [num_bfaces] corner of each boundary face */
    int32_t p1_gradients;        /* UseP1FiniteElementGradients: 1 = gradients
                                    of the P1 (Q1) finite-element interpolant
                                    at the sub-control-volume faces (the lens
                                    VCFV tests), 0 = two-point gradients     */
} gbfv_problem;

/* run-time parameters; names and defaults follow the reference's
 * Opm::Parameters (newtonmethodparameters.hh:31-53, linalgparameters.hh:
 * 41-78, blackoilnewtonmethodparameters.hh, fvbaseparameters.hh)        */
typedef struct gbfv_params {
    double newton_tolerance;          /* NewtonTolerance            1e-8    */
    int32_t newton_max_iterations;    /* NewtonMaxIterations        20      */
    int32_t newton_target_iterations; /* NewtonTargetIterations     10      */
    double newton_max_error;          /* NewtonMaxError             1e100   */
    double linear_tolerance;          /* LinearSolverTolerance      1e-3    */
    double linear_abs_tolerance;      /* LinearSolverAbsTolerance  -1       */
    int32_t linear_max_iterations;    /* LinearSolverMaxIterations  1000    */
    double linear_max_error;          /* LinearSolverMaxError       1e7     */
    int32_t precision;                /* enum gbfv_precision                */
    double inner_tolerance;           /* mixed: FP32 inner reduction  1e-3  */
    int32_t max_refinements;          /* mixed: outer FP64 refinement steps */
    double dp_max_rel;                /* DpMaxRel                   0.3     */
    double ds_max;                    /* DsMax                      0.2     */
    double pv_oscillation_threshold;  /* PriVarOscilationThreshold  1e-5    */
    double pressure_min, pressure_max;/* PressureMin/PressureMax            */
    double max_water_saturation;      /* MaximumWaterSaturation     1.0     */
    double water_only_threshold;      /* WaterOnlyThreshold         1.0     */
    double min_time_step;             /* MinTimeStepSize            0       */
    double max_time_step;             /* MaxTimeStepSize            inf     */
    int32_t max_time_step_divisions;  /* MaxTimeStepDivisions       10      */
    int32_t local_linearizer;         /* LocalLinearizerSplice: enum gbfv_local_linearizer */
    int32_t numeric_difference_method;/* NumericDifferenceMethod (FD)  +1     */
    int32_t linear_solver;            /* LinearSolverSplice: enum gbfv_linear_solver */
    int32_t amg_coarsen_target;       /* AmgCoarsenTarget           5000    */
    int32_t linearizer;               /* Properties::Linearizer: enum gbfv_linearizer */
} gbfv_params;

/* local linearizer (Properties::LocalLinearizerSplice): automatic
 * differentiation (FvBaseAdLocalLinearizer, the default) or finite
 * differences (FvBaseFdLocalLinearizer, fvbasefdlocallinearizer.hh:
 * 135-523: one cell's primary variable perturbed by BaseEpsilon /
 * primaryVarWeight at a time; numeric_difference_method +1 forward,
 * 0 central, -1 backward differences)                                     */
enum gbfv_local_linearizer {
    GBFV_LIN_AD = 0,
    GBFV_LIN_FD = 1
};

/* linear-solver backend (Properties::LinearSolverSplice):
 * ParallelBiCGStabSolverBackend (BiCGStab + block ILU(0), the default) or
 * ParallelAmgBackend (parallelamgbackend.hh:85-330: BiCGStab preconditioned
 * by one V-cycle of an aggregation AMG; SOR smoothing, Galerkin coarse
 * matrices, coarsening down to amg_coarsen_target rows).  The AMG's
 * aggregates, colours and coarse patterns are built from the first matrix a
 * context or linear solver solves and kept for its later matrices; coarse
 * values are recomputed at every solve.                                    */
enum gbfv_linear_solver {
    GBFV_LINSOLVER_ILU0 = 0,
    GBFV_LINSOLVER_AMG = 1
};

/* linearizer (Properties::Linearizer): the element-wise FvBaseLinearizer
 * (the default: every residual row and Jacobian row divided by its cell's
 * volume) or TpfaLinearizer with BlackOilLocalResidualTPFA
 * (tpfalinearizer.hh:711-866, blackoillocalresidualtpfa.hh:234-505): cell
 * by cell over precomputed neighbour records, transmissibility fluxes times
 * the face area, storage times volume / dt, rows not divided by the volume.
 * TPFA takes the black-oil model with automatic differentiation, a problem
 * without constraint cells (TpfaLinearizer applies none) and boundary faces
 * that are no-flow or mass-rate; contexts only (not batches).            */
enum gbfv_linearizer {
    GBFV_LINEARIZER_ELEMENT = 0,
    GBFV_LINEARIZER_TPFA = 1
};

/* fill *p with the reference's defaults */
void gbfv_default_params(gbfv_params* p);

/* ------------------------------------------------------------------ */
/* context: one grid (or a batch of grids, see gbfv_batch_*)            */
/* ------------------------------------------------------------------ */
typedef struct gbfv_ctx gbfv_ctx;

/* Largest grid (cells) or matrix (block rows) one context or linear solver
 * takes: device arrays are planes of a row count padded to 64 and indexed
 * with 32-bit integers, and the largest holds 63 planes (7 block slots of
 * 3 x 3), so 64 x the padded row count must stay below 2^31.  Larger inputs
 * return GBFV_ERR_UNSUPPORTED before any device work.                      */
#define GBFV_MAX_CELLS 33554368

/* Create a context on the current CUDA device and upload the problem.
 * Mirrors FvBaseLinearizer::init + createMatrix_ (fvbaselinearizer.hh:
 * 418-452): the sparsity pattern, level sets and block-slot maps are built
 * once here.  *status receives the result; NULL is returned on error.
 * Before any device call the description is checked for consistency
 * (offsets start at 0, do not decrease and end at their counts; enum
 * fields, material laws, constraint rows and gas meanings are known values;
 * arrays a used feature needs are not NULL; PVT tables of 2..32 rows with
 * strictly increasing pressures and R_s, positive B_o and B_g) and so are
 * the enum-valued parameters: GBFV_ERR_ARG, with gbfv_last_error() naming
 * the field, when one fails.                                              */
gbfv_ctx* gbfv_create(const gbfv_problem* prob, const gbfv_params* params,
                      int* status);
int gbfv_destroy(gbfv_ctx* ctx);
int gbfv_set_params(gbfv_ctx* ctx, const gbfv_params* params);
/* equations per cell (2 or 3) and number of cells */
int gbfv_dims(const gbfv_ctx* ctx, int* num_cells, int* block_size,
              int* nnz_blocks);

/* model().solution(timeIdx) (fvbasediscretization.hh): primary variables in
 * natural order, [num_cells*b]; meanings [num_cells] (black-oil gas
 * meaning, enum gbfv_pv_meaning; ignored for the immiscible model).
 * GBFV_ERR_ARG, with nothing changed, for a black-oil gas meaning other
 * than Sg, Rs or Rv.                                                      */
int gbfv_set_solution(gbfv_ctx* ctx, const double* pv,
                      const int32_t* meaning);
int gbfv_get_solution(gbfv_ctx* ctx, double* pv, int32_t* meaning);

/* simulator().timeStepSize() and newtonMethod().numIterations(), which the
 * storage cache reads (fvbaselocalresidual.hh:535-571)                    */
int gbfv_set_timestep(gbfv_ctx* ctx, double dt);
int gbfv_set_newton_iteration(gbfv_ctx* ctx, int iteration);

/* FvBaseLinearizer::linearizeDomain (fvbaselinearizer.hh:201-241):
 * residual and Jacobian of the current solution, on the device.  Applies
 * the constraints to the solution first and to the system afterwards
 * (:630-666).                                                             */
int gbfv_linearize(gbfv_ctx* ctx);
/* linearizer.residual() -> [num_cells*b], natural order                   */
int gbfv_get_residual(gbfv_ctx* ctx, double* residual);
/* linearizer.jacobian().istlMatrix() as BCRS, natural order, columns sorted
 * ascending in each row; blocks row-major b*b, entry [eq][pv].
 * row_ptr[num_cells+1], col_idx[nnz], blocks[nnz*b*b]                     */
int gbfv_get_jacobian(gbfv_ctx* ctx, int32_t* row_ptr, int32_t* col_idx,
                      double* blocks);

/* NewtonMethod::preSolve_ error: max_{dof,eq} |r * eqWeight| over
 * unconstrained cells (newtonmethod.hh:572-607)                           */
int gbfv_newton_error(gbfv_ctx* ctx, double* error);

/* ParallelBiCGStabSolverBackend: prepare + setResidual + setMatrix + solve
 * (parallelbasebackend.hh:182-284) on the current linearization.  Solves
 * J dx = r; dx [num_cells*b] natural order (may be NULL to keep it on the
 * device for gbfv_newton_update).  iterations: BiCGStab iterations (sum of
 * inner iterations in mixed precision).  Returns GBFV_OK when converged,
 * GBFV_ERR_NOT_CONVERGED / GBFV_ERR_BREAKDOWN otherwise.                  */
int gbfv_solve(gbfv_ctx* ctx, double* dx, int* iterations);

/* NewtonMethod::update_ / BlackOilNewtonMethod::updatePrimaryVariables_:
 * x <- x - dx with chopping and primary-variable switching, using the dx
 * of the last gbfv_solve.  num_switched may be NULL.                      */
int gbfv_newton_update(gbfv_ctx* ctx, int* num_switched);

/* NewtonMethod::apply (newtonmethod.hh:228-438) for one time step of size
 * dt.  converged: 1/0.  iterations: numIterations() after the call
 * (2*target on failure, as failed_()).  linear_iterations: total.         */
typedef struct gbfv_newton_report {
    int32_t converged;
    int32_t iterations;
    int32_t linear_iterations;
    int32_t linearizations;
    int32_t refinements;       /* mixed precision: outer refinement steps   */
    int32_t status;            /* GBFV_OK or the error that ended it        */
    double error;              /* last Newton error                         */
} gbfv_newton_report;
int gbfv_newton_apply(gbfv_ctx* ctx, double dt, gbfv_newton_report* rep);

/* NewtonMethod::suggestTimeStepSize (newtonmethod.hh:448-465)              */
double gbfv_suggest_time_step(const gbfv_ctx* ctx, double old_dt,
                              int newton_iterations);

/* FvBaseProblem::timeIntegration + Simulator time loop (fvbaseproblem.hh:
 * 512-606): num_steps time steps starting at dt0 (dt halving on failure,
 * dt control by Newton iterations unless fixed_dt != 0).  Per-step stats
 * (each may be NULL): dt used, Newton iterations, linear iterations.      */
int gbfv_time_integration(gbfv_ctx* ctx, int num_steps, double dt0,
                          double end_time, int fixed_dt, double* step_dt,
                          int32_t* step_newton, int32_t* step_linear,
                          int32_t* total_linearizations);

/* ------------------------------------------------------------------ */
/* stand-alone linear-solver backend over a host BCRS matrix            */
/* (ParallelBiCGStabSolverBackend used without the linearizer)          */
/* ------------------------------------------------------------------ */
typedef struct gbfv_linsolver gbfv_linsolver;
/* prepare(M): pattern of an n x n block matrix, blocks b x b (b = 2, 3),
 * columns sorted ascending per row, diagonal present.                     */
gbfv_linsolver* gbfv_linsolver_create(int n, int b, const int32_t* row_ptr,
                                      const int32_t* col_idx,
                                      const gbfv_params* params, int* status);
int gbfv_linsolver_destroy(gbfv_linsolver* s);
/* setMatrix(M): values [nnz*b*b] row-major blocks                         */
int gbfv_linsolver_set_matrix(gbfv_linsolver* s, const double* blocks);
/* setResidual(b) + solve(x): x = A^-1 rhs, iterations as gbfv_solve       */
int gbfv_linsolver_solve(gbfv_linsolver* s, const double* rhs, double* x,
                         int* iterations);
/* AMG backend (linear_solver GBFV_LINSOLVER_AMG), diagnostics: the
 * hierarchy (built from the matrix last set if there is none yet) --
 * rows (sizes) and colours (colors, may be NULL) of every level, at most
 * 15; returns the level count or -status -- and one FP64 V-cycle
 * v = M^-1 d of the preconditioner (natural order, n*b values).           */
int gbfv_linsolver_amg_levels(gbfv_linsolver* s, int32_t* sizes,
                              int32_t* colors);
/* the same for a context: 0 levels before its first AMG solve            */
int gbfv_amg_levels(gbfv_ctx* ctx, int32_t* sizes, int32_t* colors);
int gbfv_linsolver_amg_apply(gbfv_linsolver* s, const double* d, double* v);
/* Patterns beyond the 5/7-point stencil's -- more than 7 distinct column
 * offsets (at most 27, symmetric), or an ILU(0) whose lower entries update
 * more than the diagonal, like the vertex-centred 9-point Jacobian -- are
 * solved with the general block ILU(0) (natural-order blockILU0Decomposition,
 * level-scheduled).  Diagnostic: one FP64 application v = (LU)^-1 d of it
 * after factoring the matrix last set (natural order, n*b values);
 * GBFV_ERR_UNSUPPORTED for a structured pattern.                          */
int gbfv_linsolver_ilu0_apply(gbfv_linsolver* s, const double* d, double* v);

/* ------------------------------------------------------------------ */
/* diagnostics                                                          */
/* ------------------------------------------------------------------ */
/* kernel launches issued by this library since load                       */
int64_t gbfv_kernel_launches(void);
/* last CUDA error string for the calling thread ("" if none)              */
const char* gbfv_last_error(void);
/* per-phase device time of the last gbfv_newton_apply, milliseconds:
 * [0] linearize, [1] solver-format conversion + ILU0 factorization,
 * [2] Krylov iterations, [3] Newton update + error                       */
int gbfv_phase_times(const gbfv_ctx* ctx, double* ms4);

/* the CUDA stream (cudaStream_t) all work of this context is issued on    */
void* gbfv_stream(gbfv_ctx* ctx);

/* device-side snapshot of the solution, its meanings and the switching
 * flags, and its restore (keeps a run's inputs resident on the device)    */
int gbfv_save_state(gbfv_ctx* ctx);
int gbfv_restore_state(gbfv_ctx* ctx);

/* cumulative kernel statistics since creation or the last reset.
 * Durations are CUDA-event times on the context's stream.  Algorithmic
 * bytes are what each kernel must move at least once for its work:
 *   solve: per factorization  N*(S*b*b + (d+1)*b*b)*s + 4*N*d
 *          per iteration      N*(2*S*b*b + 4*d*b*b + 2*b*b)*s
 *                             + 4*N*(2*S + 4*d) + 30*N*b*s
 *          (S = 2d+1 blocks per row, d = lower blocks, s = 4 or 8 bytes)
 *   linearize: IQ pass (reads x, writes the intensive quantities) plus the
 *          assembly pass (reads them, the face geometry and the storage
 *          cache; writes residual and all S Jacobian blocks)            */
typedef struct gbfv_kernel_stats {
    double solve_ms;           /* persistent BiCGStab/ILU0 kernels        */
    int64_t solve_launches;
    int64_t solve_iterations;
    int64_t solve_factorizations;
    double solve_bytes;
    double linearize_ms;       /* IQ + assembly kernels                   */
    int64_t linearize_launches;
    double linearize_bytes;
} gbfv_kernel_stats;
int gbfv_get_kernel_stats(const gbfv_ctx* ctx, gbfv_kernel_stats* out);
/* launch configuration the autotuner chose for the persistent solve kernel
 * of a precision (GBFV_PREC_FP64 / GBFV_PREC_MIXED): cluster (mode 1),
 * cooperative grid (mode 0) or hybrid (mode 2), possibly with
 * GBFV_SOLVER_TILES, blocks, and the candidate timings [ms] in tune_ms
 * (room for 16; *num_tuned of them are written; any output may be NULL)  */
int gbfv_solver_config(const gbfv_ctx* ctx, int precision, int* mode, int* blocks,
                       double* tune_ms, int* num_tuned);
/* fix the launch configuration of the persistent solve kernel of a
 * precision (mode 1 = cluster of `blocks` blocks, 0 = cooperative grid,
 * 2 = hybrid: `blocks` in clusters of 16 over the GPU, the first cluster
 * factorizes and sweeps, all blocks share SpMV, updates and reductions) and
 * skip the autotuner; GBFV_ERR_UNSUPPORTED beyond what the device allows.
 * Modes 1 and 2 or-ed with GBFV_SOLVER_TILES deal the rows of every ILU
 * level to the sweeping cluster's blocks by the spatial tile of their cell
 * (grid contexts only; GBFV_ERR_UNSUPPORTED where a tile's level is wider
 * than a block or the tables exceed shared memory)                        */
#define GBFV_SOLVER_TILES 4
/* or-ed into mode 2 for GBFV_PREC_MIXED: the hybrid launch with blocks of
 * 256 threads instead of 512 (a cheaper level step where a level's share per
 * block fits 256 rows; one of the autotuner's candidates)                  */
#define GBFV_SOLVER_NARROW 8
/* reported by gbfv_solver_config only: the precision's solves run in the
 * general block ILU(0) kernel (vertex-centred grids, narrow systems, and
 * the FP32 inner solves of systems wider than one block), with
 * GBFV_SOLVER_TAGGED where its sweeps publish every row's result with a tag
 * its consumers wait for instead of a barrier per wavefront level          */
#define GBFV_SOLVER_GILU 16
#define GBFV_SOLVER_TAGGED 32
int gbfv_set_solver_config(gbfv_ctx* ctx, int precision, int mode, int blocks);
int gbfv_reset_kernel_stats(gbfv_ctx* ctx);
/* with GBFV_PROFILE set in the environment at creation: nanoseconds spent
 * by the persistent solve kernel per phase since the last call ([0]
 * factorization, [1] forward sweeps, [2] backward sweeps, [3] SpMV + dots,
 * [4] vector updates + norms, [5] remaining); zeros otherwise            */
int gbfv_solver_phase_ns(gbfv_ctx* ctx, unsigned long long* ns8);
/* with GBFV_PROFILE: SM cycles one working thread of the forward sweeps
 * spent per level since the last call: [0] waiting for its data, [1]
 * computing, [2] pushing results and storing, [3] in the level barrier;
 * [4] the number of levels sampled.  With GBFV_SOLVER_TILES (thread 0 of
 * block 5): [0] staging the level's operands, [1] waiting for the halo
 * values, [2] computing, pushing and storing, [3] the level barrier       */
int gbfv_solver_level_cycles(gbfv_ctx* ctx, unsigned long long* c8);

/* ------------------------------------------------------------------ */
/* Batched systems (ensemble realizations, served requests).  No single
 * counterpart in the reference, which advances one problem per simulator
 * (Simulator::run, simulator.hh:738); each system here follows exactly the
 * reference's time loop and Newton method (fvbaseproblem.hh:512-606,
 * newtonmethod.hh:228-806) as gbfv_time_integration does.  The device work
 * of all systems is issued together: one batched launch per phase (IQ +
 * assembly + Newton error; FP64 residual; one persistent BiCGStab/ILU0
 * launch in which clusters of cluster_size blocks take systems from a work
 * queue, largest first; Newton update), each phase a captured CUDA graph
 * replayed every round.  A system's results equal those of the same
 * problem run alone with gbfv_set_solver_config(ctx, precision, 1,
 * cluster_size).  All systems share params and the model.               */
typedef struct gbfv_batch gbfv_batch;
typedef struct gbfv_batch_stats {
    int32_t num_systems;
    int32_t cluster_size;      /* blocks per cluster of the batched solve  */
    int32_t num_clusters;      /* clusters resident at once               */
    int32_t pad;
    int64_t rounds;            /* Newton rounds                           */
    int64_t graph_launches;
    int64_t kernel_launches;
    int64_t solve_launches;    /* batched persistent solve launches        */
    double solve_ms;           /* device time of those launches            */
    double solve_bytes;        /* their algorithmic bytes                  */
    double linearize_ms;       /* device time of the linearization graphs  */
} gbfv_batch_stats;
/* cluster_size 0: 8 (or the device maximum below it)                    */
gbfv_batch* gbfv_batch_create(const gbfv_problem* problems, int num_systems,
                              const gbfv_params* params, int cluster_size, int* status);
int gbfv_batch_destroy(gbfv_batch* batch);
/* the context of system i (set_solution / get_solution / save_state ...;
 * owned by the batch)                                                    */
gbfv_ctx* gbfv_batch_system(gbfv_batch* batch, int i);
/* every system: num_steps time steps from dt0 (gbfv_time_integration
 * semantics); returns the first failing system's status or GBFV_OK      */
int gbfv_batch_time_integration(gbfv_batch* batch, int num_steps, double dt0,
                                double end_time, int fixed_dt);
/* autotuner of the batched solve: linearizes every system at its current
 * state, times one batched solve for each cluster size 2, 4, 8, 16 (up to
 * the device limit) and keeps the fastest; the systems' states are not
 * changed.  ms[k] = the solve time of candidate k (up to 8)              */
int gbfv_batch_autotune(gbfv_batch* batch, double dt, int* cluster_size, double* ms, int* num_candidates);
/* system i's last time integration: its status, the steps it completed
 * (*steps_done, at most the num_steps of that gbfv_batch_time_integration
 * call, or the steps of a served request) and per completed step its dt,
 * Newton and linear iterations, written to arrays of at least *steps_done
 * entries; any output may be NULL (a first call with NULL arrays gives the
 * count)                                                                  */
int gbfv_batch_system_report(const gbfv_batch* batch, int i, int* status, int* steps_done,
                             double* step_dt, int32_t* step_newton, int32_t* step_linear,
                             int* linearizations);
int gbfv_batch_get_stats(const gbfv_batch* batch, gbfv_batch_stats* out);
void* gbfv_batch_stream(gbfv_batch* batch);

/* ------------------------------------------------------------------ */
/* Serving: a batch whose slots are filled and emptied while it runs
 * (continuous batching).  A request (one system, its initial state and
 * its time steps) is admitted into a free slot between rounds; every
 * gbfv_serve_step runs one round for all running systems, so requests that
 * arrive while others are on the GPU join at the next round and their work
 * overlaps on the device.  A finished slot keeps its state (read it through
 * gbfv_batch_system) until gbfv_serve_release frees its device memory.
 * Admission by HBM footprint is the caller's policy, with
 * gbfv_footprint_bytes as the estimate of one system.                    */
/* estimated device bytes of one system (context + solver buffers) as a
 * batch or a server holds it; -1 for a size no context takes (num_cells
 * outside 1..GBFV_MAX_CELLS, block size other than 2 or 3, dim other than
 * 2 or 3).  A stand-alone context of more than 65,536 cells whose
 * autotuner picks the tagged sweeps also holds their copy of the factors
 * and vectors (about 320 B per cell in FP32, 650 B in FP64 at b = 3, dim = 3, plus
 * 48 B of tagged words), not counted here.                                */
int64_t gbfv_footprint_bytes(int num_cells, int block_size, int dim);
gbfv_batch* gbfv_serve_create(int capacity, int model, const gbfv_params* params,
                              int cluster_size, int max_cells, int* status);
int gbfv_serve_admit(gbfv_batch* server, const gbfv_problem* problem, const double* pv,
                     const int32_t* meaning, int num_steps, double dt0, int fixed_dt, int* slot);
/* one round; running = systems still iterating                           */
int gbfv_serve_step(gbfv_batch* server, int* running);
/* state: 0 empty, 1 running, 2 done, 3 failed (status = its error)       */
int gbfv_serve_slot(const gbfv_batch* server, int slot, int* state, int* status);
int gbfv_serve_release(gbfv_batch* server, int slot);
int64_t gbfv_serve_footprint(const gbfv_batch* server);

/* ------------------------------------------------------------------ */
/* Restart files in the reference's text format (Opm::Restart,
 * opm/models/io/restart.hh:101-265, written by Simulator::serialize,
 * simulator.hh:906-962): the magic cookie (restart.hh:57-75), the
 * "Simulator" section (simulator.hh:930-943), the problem's
 * "VTKMultiWriter" section when it writes VTK output (fvbaseproblem.hh:
 * 755-760, vtkmultiwriter.hh:408-437; no .pvd meta file here: length and
 * position 0) and the ECFV "Entities: Codim 0" section, one line per cell
 * in natural order (ecfvdiscretization.hh:212-226): the primary variables
 * (fvbasediscretization.hh:1440-1454), for black-oil followed by the gas,
 * water and pressure meanings and the PVT region (blackoilmodel.hh:
 * 468-493).  Floating point as "%.20g" (the stream's precision(20)).      */
typedef struct gbfv_restart_info {
    int32_t num_cpus;            /* gridView.comm().size() (cookie)          */
    int32_t rank;                /* gridView.comm().rank() (cookie)          */
    int32_t num_edges;           /* gridView.size(dim - 1) (cookie)          */
    int32_t num_vertices;        /* gridView.size(dim) (cookie)              */
    int32_t episode_index;       /* Simulator section                        */
    int32_t time_step_index;
    double episode_start_time;
    double episode_length;
    double start_time;
    double time;
    int32_t vtk_section;         /* 1: with the VTKMultiWriter section       */
    int32_t vtk_writer_num;      /* its curWriterNum_                        */
    int32_t entity_codim;        /* codimension of the entities: 0 elements
                                    (ECFV), the grid dimension for vertices
                                    (VCFV, vcfvdiscretization.hh:185-200)   */
    int32_t num_elements;        /* gridView.size(0) (cookie) when the
                                    entities are vertices; with codim 0 the
                                    cells are the elements                   */
} gbfv_restart_info;
/* the file's text for num_cells entities (cells, or the vertices of a
 * vertex-centred grid) of b primary variables (natural order) and, for
 * black-oil, their gas meanings (NULL: immiscible); *len =
 * its size in bytes; buf NULL asks for the size only                      */
int gbfv_format_restart(const gbfv_restart_info* info, int32_t num_cells, int32_t b, const double* pv,
                        const int32_t* gas_meaning, char* buf, size_t cap, size_t* len);
/* read a file's text back (Restart::deserialize*, restart.hh:166-265):
 * `expect` gives the cookie's grid counts, out the Simulator section (and
 * whether a VTK section was present); GBFV_ERR_ARG on any mismatch        */
int gbfv_parse_restart(const char* text, size_t len, const gbfv_restart_info* expect, int32_t num_cells, int32_t b,
                       double* pv, int32_t* gas_meaning, gbfv_restart_info* out);
/* restartFileName_ (restart.hh:80-95): <dir/>sim_name_time=<t>_rank=<r>.ers */
int gbfv_restart_file_name(const char* output_dir, const char* sim_name, double time, int32_t rank, char* buf,
                           size_t cap);
/* write the context's current solution to a restart file; read one back
 * into the context (solution and its previous time level, as
 * BlackOilModel::deserialize sets solution(1) = solution(0)); info: cookie
 * counts in, Simulator section out                                        */
int gbfv_write_restart(gbfv_ctx* ctx, const char* path, const gbfv_restart_info* info);
int gbfv_read_restart(gbfv_ctx* ctx, const char* path, gbfv_restart_info* info);

/* ------------------------------------------------------------------ */
/* VTK output (the reference's VtkMultiWriter with its primary-variable and
 * multi-phase modules: opm/models/io/vtkmultiwriter.hh:64-540,
 * vtkprimaryvarsmodule.hh:54-170, vtkmultiphasemodule.hh:84-460).       */
/* The output quantities of the context's current solution, evaluated on
 * the device as the intensive quantities are: out[q*num_cells + cell],
 * natural cell order, for plane q = 3*k + phase with k = 0 pressure,
 * 1 density, 2 saturation, 3 mobility, 4 relative permeability,
 * 5 viscosity (phases: wetting / non-wetting for the immiscible model, the
 * third plane zero; water / oil / gas for black-oil), and q = 18 the
 * porosity.                                                              */
#define GBFV_OUTPUT_PLANES 19
int gbfv_output_fields(gbfv_ctx* ctx, double* out);

/* fields of a VTK file, the reference's VtkWrite* parameters; the default
 * set is theirs: pressures, densities, saturations, relative
 * permeabilities and porosity                                            */
enum gbfv_vtk_field {
    GBFV_VTK_PRESSURE = 1,        /* VtkWritePressures              true  */
    GBFV_VTK_DENSITY = 2,         /* VtkWriteDensities              true  */
    GBFV_VTK_SATURATION = 4,      /* VtkWriteSaturations            true  */
    GBFV_VTK_MOBILITY = 8,        /* VtkWriteMobilities             false */
    GBFV_VTK_RELPERM = 16,        /* VtkWriteRelativePermeabilities true  */
    GBFV_VTK_VISCOSITY = 32,      /* VtkWriteViscosities            false */
    GBFV_VTK_POROSITY = 64,       /* VtkWritePorosity               true  */
    GBFV_VTK_PRIMARY_VARS = 128,  /* VtkWritePrimaryVars            false */
    GBFV_VTK_DOF_INDEX = 256      /* VtkWriteDofIndex               false */
};
#define GBFV_VTK_DEFAULT_FIELDS (GBFV_VTK_PRESSURE | GBFV_VTK_DENSITY | GBFV_VTK_SATURATION | \
                                 GBFV_VTK_RELPERM | GBFV_VTK_POROSITY)
/* the grid's vertices and cells as the VTK file lists them: num_points
 * points (x, y, z), each cell's vertices_per_cell vertex indices in VTK
 * order (4: VTK_QUAD in 2D, 8: VTK_HEXAHEDRON in 3D), cells in natural order */
typedef struct gbfv_vtk_grid {
    int32_t num_points;
    const double* points;          /* [num_points*3]                      */
    int32_t vertices_per_cell;     /* 4 or 8                               */
    const int32_t* cell_vertices;  /* [num_cells*vertices_per_cell]        */
    int32_t num_cells;             /* 0: the context's cells (cell data);
                                      > 0: that many cells of a vertex-centred
                                      grid whose num_points vertices are the
                                      context's degrees of freedom (vertex
                                      data, VcfvBaseOutputModule)           */
} gbfv_vtk_grid;
/* One time step's XML UnstructuredGrid file (.vtu, ASCII as the
 * reference's default VtkOutputFormat, fvbasediscretization.hh:237-238):
 * the selected fields as Float32 cell data (point data on a vertex-centred
 * grid), each value rounded to float as
 * VtkScalarFunction::evaluate does (vtkscalarfunction.hh:76-110), in the
 * modules' order and with their names ("pressure_<phase>", ...,
 * "porosity", "PV_<primary variable>", "DOF index").                     */
int gbfv_write_vtk(gbfv_ctx* ctx, const gbfv_vtk_grid* grid, int32_t fields, const char* path);
/* VtkMultiWriter::fileName_ + suffix (vtkmultiwriter.hh:478-488):
 * <sim_name>-<writer_num as 5 digits>.vtu                                */
int gbfv_vtk_file_name(const char* sim_name, int32_t writer_num, char* buf, size_t cap);
/* the collection file (.pvd) listing the time steps written so far, as
 * startMultiFile_ / the write tasklet / finishMultiFile_ write it
 * (vtkmultiwriter.hh:74-96, 490-518): one DataSet per (time, file name)   */
int gbfv_write_pvd(const char* path, int32_t n, const double* times, const char* const* files);

/* ------------------------------------------------------------------ */
/* Self-test of the device-side wait bound (no counterpart in the
 * reference): one block waits, with the bounded wait of the solver's
 * sweeps, on a barrier phase that nothing completes.  Returns
 * GBFV_ERR_TIMEOUT when the wait gave up as designed (the device stays
 * usable), and the kernel's time in ms.                                   */
int gbfv_selftest_wait_timeout(double* ms);

/* Host-only check of the push sweeps' level-barrier placement (no
 * counterpart in the reference): for a pattern of num_rows rows in level
 * order (lev_ptr[num_levels+1]; col[s*num_rows + p], slots 0..dim-1 the
 * lower neighbours, dim the row itself, dim+1..2dim the upper ones, -1 for
 * none), cluster blocks dealing each level's rows a warp at a time
 * (owner_mode 0) or in contiguous shares (1) and `buffers` dependency
 * buffers per block, barrier_after[l] = 1 where the forward (or backward)
 * sweep needs a cluster barrier after level l.                            */
int gbfv_selftest_level_barriers(int32_t num_rows, int32_t dim, const int32_t* lev_ptr, int32_t num_levels,
                                 const int32_t* col, int32_t cluster, int32_t owner_mode, int32_t buffers,
                                 int32_t forward, int8_t* barrier_after);

/* ------------------------------------------------------------------ */
/* Allocation-free Newton error.  No counterpart in the reference: its
 * NewtonMethod computes the same maximum norm on the host
 * (newtonmethod.hh:572-598, preSolve_).  For callers that hold the
 * residual in their own device memory and may not allocate device memory
 * during a step (a host simulator that owns the whole HBM budget through
 * its own pool allocator): max over cells p with skip[p] == 0 of
 * |residual[p*num_eq + k]|, the value gbfv_newton_error returns.
 *   residual  device pointer, num_cells*num_eq doubles (cell-major)
 *   skip      device pointer to num_cells int32 flags (non-zero: constraint
 *             or auxiliary cell, left out), or NULL for none
 *   num_cells 0 .. GBFV_NOALLOC_MAX_CELLS
 *   num_eq    equations per cell, 1 .. 8 (GBFV_ERR_ARG outside)
 *   stream    cudaStream_t to run on (NULL: legacy default stream); the
 *             call returns after the stream has reached its end
 * Nothing is allocated: the scratch is a fixed static device array of
 * GBFV_NOALLOC_MAX_CELLS/256 partial maxima (512 KiB) plus one result word,
 * and num_cells above GBFV_NOALLOC_MAX_CELLS is rejected with GBFV_ERR_ARG.
 * No scratch word has to start at zero (each call writes every word it
 * reads).  The first call on each device looks up the scratch address
 * (cudaGetSymbolAddress, with that device current) and should come before
 * any stream capture.  That address is kept for the life of the process:
 * after cudaDeviceReset (or anything else that replaces the device's
 * primary context) it is stale, so this entry point must not be called on
 * a device that was reset after its first call there.  Calls that overlap
 * in time share the scratch and race: serialize them.  Returns
 * GBFV_ERR_NONFINITE (error = NaN) when a considered entry is not finite. */
#define GBFV_NOALLOC_MAX_CELLS (1 << 24)
int gbfv_newton_error_noalloc(const double* residual, const int32_t* skip, int32_t num_cells,
                              int32_t num_eq, void* stream, double* error);

#ifdef __cplusplus
}
#endif
#endif /* GBFV_H */
