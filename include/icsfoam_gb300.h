/*
 * icsfoam_gb300.h - C ABI of the GB300 implicit coupled pseudo-time solver.
 *
 * One handle owns one finite-volume case resident on the current CUDA
 * device: mesh addressing and geometry are uploaded once by ics_create(),
 * the conservative state, boundary values, Jacobian and Krylov workspace
 * stay in device memory for the life of the handle.  Host arrays passed in
 * are only read during the call; nothing keeps a pointer to them.
 *
 * Conventions
 *  - Every function returns an ICS_* status; 0 is success.  A failed call
 *    leaves a message retrievable with ics_last_error().  Nothing aborts the
 *    process (the reference raises FatalError instead).
 *  - Cell 5-vectors are stored cell-major [n_cells][5] in the order
 *    (rho, rhoUx, rhoUy, rhoUz, rhoE).  5x5 blocks are row-major with the
 *    same order: block[i][j] = d(equation i)/d(variable j).
 *  - Face arrays list the internal faces first, then the non-empty
 *    boundary faces in patch order, exactly like an OpenFOAM surface field.
 *  - A handle is not thread-safe; several handles may coexist.
 *
 * The oracle library (test infrastructure) exports the same functions with
 * the prefix "icsref_" and the same structs, so one test harness drives both.
 */
#ifndef ICSFOAM_GB300_H
#define ICSFOAM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define ICS_OK             0
#define ICS_ERR_ARG        1  /* invalid argument / size                       */
#define ICS_ERR_CUDA       2  /* CUDA runtime error                            */
#define ICS_ERR_NONFINITE  3  /* NaN/Inf in residual or state                  */
#define ICS_ERR_BREAKDOWN  4  /* zero Krylov norm at the start of a cycle      */
#define ICS_ERR_DIAG       5  /* all-zero diagonal for LU-SGS (lusgs.C:117-121) */
#define ICS_ERR_SCHEME     6  /* unknown scheme/solver name                    */
#define ICS_ERR_STATE      7  /* call made in the wrong order                  */
#define ICS_ERR_NOMEM      8  /* device allocation failed                      */
#define ICS_ERR_TIMEOUT    9  /* bounded device wait gave up                   */

/* ---- selectors (runtime-selection table keys of the reference) ------------ */
/* fvSchemes/convectiveFluxScheme/fluxScheme (newConvectiveFluxScheme.C:50)     */
enum { ICS_FLUX_AUSMPLUSUP = 0, ICS_FLUX_HLLC = 1, ICS_FLUX_ROE = 2 };
/* fvSchemes/interpolationSchemes reconstruct(rho|U|T) (convectiveFluxScheme.C:387-400) */
enum {
  ICS_RECON_UPWIND = 0,              /* first order                                 */
  ICS_RECON_VANLEER = 1,             /* TVD limitedScheme, Gauss linear gradient    */
  ICS_RECON_MINMOD = 2,              /* TVD limitedScheme, Gauss linear gradient    */
  ICS_RECON_MUSCL_VENKATAKRISHNAN = 3, /* linearUpwind + cellLimited<Venkatakrishnan> */
  ICS_RECON_MUSCL_MINMOD = 4         /* linearUpwind + cellLimited<minmod>          */
};
/* ddtSchemes default dualTime rPseudoDeltaT <scheme> (dualTimeDdtScheme.H:109-118) */
enum { ICS_DDT_STEADY = 0, ICS_DDT_EULER = 1, ICS_DDT_BACKWARD = 2 };
/* flowSolver/solver (coupledMatrixSolver.C:41-67): GMRES (gmres.C) or
 * smoothSolverCoupled (smoothSolverCoupled.C:369-515, block-Jacobi sweeps)      */
enum { ICS_SOLVER_GMRES = 0, ICS_SOLVER_SMOOTH = 1 };
/* flowSolver/<solver>/preconditioner (coupledMatrix.H:296-369)                  */
enum { ICS_PC_NONE = 0, ICS_PC_LUSGS = 1, ICS_PC_JACOBI = 2 };
/* precision of the linear solve: FP64 everywhere, or FP32 Jacobian blocks,
 * preconditioner and Krylov basis under an FP64 residual/update            */
enum { ICS_PREC_FP64 = 0, ICS_PREC_MIXED = 1 };

/* boundary patch kinds */
enum {
  ICS_PATCH_EMPTY = 0,
  ICS_PATCH_ZERO_GRADIENT = 1,   /* U, p, T zeroGradient                             */
  ICS_PATCH_SLIP = 2,            /* U slip, p, T zeroGradient                        */
  ICS_PATCH_FIXED = 3,           /* U, p, T fixedValue                               */
  ICS_PATCH_PRESSURE_OUTLET = 4, /* p fixedValue, U, T zeroGradient                  */
  ICS_PATCH_TOTAL_INLET = 5,     /* totalPressure, totalTemperature,
                                    pressureInletOutletVelocity                      */
  ICS_PATCH_ISOTHERMAL_WALL = 6, /* U = 0, T fixed, p zeroGradient                   */
  ICS_PATCH_CYCLIC = 7           /* coupled to a partner patch (OpenFOAM cyclic, parallel
                                    or rotational): face i of the one is face i of the other */
};

typedef struct {
  int32_t kind;     /* ICS_PATCH_*                                         */
  int32_t is_wall;  /* OpenFOAM "wall" patch type (setCoAndDeltaT.H:88-90) */
  double p, T;      /* fixed static pressure / temperature                 */
  double U[3];      /* fixed velocity                                      */
  double p0, T0;    /* total pressure / temperature (ICS_PATCH_TOTAL_INLET) */
  double rotation[9]; /* ICS_PATCH_CYCLIC: row-major R taking the partner side's
                         vectors into this patch's frame (cyclic forwardT)  */
} ics_patch_desc;

/* Mesh in OpenFOAM LDU convention (owner < neighbour, upper-triangular
 * internal faces).  Vectors are [n][3].  Empty patches are not listed.     */
typedef struct {
  int32_t n_cells, n_faces, n_bfaces, n_patches;
  const int32_t* owner;
  const int32_t* neighbour;
  const double* Sf;                   /* [n_faces][3] area vectors          */
  const double* Cf;                   /* [n_faces][3] face centres          */
  const double* weights;              /* [n_faces] linear weights           */
  const double* delta_coeffs;         /* [n_faces]                          */
  const double* nonorth_delta_coeffs; /* [n_faces]                          */
  const double* C;                    /* [n_cells][3] cell centres          */
  const double* V;                    /* [n_cells] volumes                  */
  const int32_t* b_cell;              /* [n_bfaces] adjacent cell           */
  const int32_t* b_patch;             /* [n_bfaces] patch index             */
  const double* b_Sf;                 /* [n_bfaces][3]                      */
  const double* b_Cf;                 /* [n_bfaces][3]                      */
  const double* b_delta_coeffs;       /* [n_bfaces]                         */
  const ics_patch_desc* patches;      /* [n_patches]                        */
  int32_t solution_d[3];              /* +1 solved, -1 empty direction      */
  /* coupled (cyclic) boundary faces, OpenFOAM cyclicFvPatch; all may be NULL
   * when no patch is ICS_PATCH_CYCLIC                                       */
  const int32_t* b_partner;             /* [n_bfaces] the paired face's cell (-1: not cyclic) */
  const double* b_weights;              /* [n_bfaces] coupled linear weights  */
  const double* b_nbr_d;                /* [n_bfaces][3] face centre minus the partner
                                           cell centre seen from this side (Cf - C - delta) */
  const double* b_nonorth_delta_coeffs; /* [n_bfaces]; NULL: b_delta_coeffs  */
} ics_mesh_desc;

/* Dictionary entries of fvSchemes / fvSolution / thermophysicalProperties
 * the hot path reads.  Defaults are those of the reference (ics_default_config). */
typedef struct {
  /* thermo: perfectGas, hConst, sensibleInternalEnergy with Tref = 0      */
  double R, Cp;
  /* transport: const (mu) or sutherland (As, Ts); Prandtl number         */
  double mu, Pr, As, Ts;
  int32_t sutherland;
  int32_t viscous;                 /* add viscous residual and Jacobian   */
  /* convectiveFluxScheme                                                  */
  int32_t flux_scheme;             /* ICS_FLUX_*                          */
  int32_t low_mach_ausm;           /* lowMachAusm (ausmPlusUpFluxScheme.C:61)      */
  double entropy_fix_coeff;        /* entropyFixCoeff (roeFluxScheme.C:255)        */
  int32_t recon_rho, recon_U, recon_T; /* ICS_RECON_* per reconstruct() group      */
  /* ddtSchemes                                                            */
  int32_t ddt_scheme;              /* ICS_DDT_*                           */
  double delta_t;                  /* physical time step                  */
  /* flowSolver                                                            */
  int32_t solver, preconditioner, n_directions, max_iter, min_iter;
  double tolerance, rel_tol;
  int32_t precision;               /* ICS_PREC_*                          */
  /* pseudoTime                                                            */
  int32_t n_pseudo_corr, n_pseudo_corr_min;
  double pseudo_tol, pseudo_tol_rel;
  double pseudo_co_num, pseudo_co_num_min, pseudo_co_num_max;
  double pseudo_co_max_increase, pseudo_co_min_decrease;
  int32_t local_timestepping, local_timestepping_bounding;
  double local_timestepping_lower_bound;
  int32_t reset_pseudo;
  double rho_min, T_min, T_max;
  /* smoothSolverCoupled: Jacobi sweeps per stop test (nSweeps)            */
  int32_t n_sweeps;
  /* viscousFluxScheme: LaxFriedrichJacobian (viscousFluxScheme.C:107).
   * 1 (default): the viscous Jacobian is the scalar laplacian of
   * 0.5 (mu+alphaEff)/rho on every equation.  0: the laplacians of mu and
   * alphaEff acting on the conserved variables through -U/rho, 1/rho,
   * (|U|^2-E)/rho, plus the boundary terms of the physical patches
   * (viscousFluxScheme.C:120-215, 249-267).                               */
  int32_t viscous_lf_jacobian;
  /* gradSchemes cellLimited<limiter> Gauss linear k: the coefficient k in
   * (0, 1] of the cellLimited gradients of linearUpwind reconstruction.
   * k < 1 widens each cell's bounds by (1/k - 1)(max - min) of its
   * neighbourhood before the limiter (OpenFOAM cellLimitedGrad); 1 is the
   * plain limiter.                                                          */
  double limiter_coeff;
} ics_config;

/* residualsIO (residualsIO.H:54-315): L1 residuals normalised per equation. */
typedef struct {
  double init_res[5];   /* rho, rhoUx, rhoUy, rhoUz, rhoE */
  double final_res[5];
  int32_t n_iterations; /* restart cycles */
  int32_t converged;
} ics_solver_perf;

typedef struct {
  ics_solver_perf perf;
  double rho_l2_residual;   /* sqrt(sum((div(phi)*V)^2)), dbnsFoam.C:136-138 */
  double pseudo_co_mean;
  int32_t bounded_cells;    /* cells touched by T/rho bounding           */
  int32_t status;
} ics_iter_stats;

typedef struct ics_handle_s* ics_handle;

/* ---- lifecycle ----------------------------------------------------------- */
/* Defaults of the reference dictionaries (pseudotimeControl.C:49-57,
 * beginTimeStep.H:15-44, initialise.H:39-70, coupledMatrixSolver.C:81-84). */
void ics_default_config(ics_config* cfg);
/* Replaces: fvMesh construction + createFields.H:160-190 (flux scheme and
 * solver objects).  Uploads addressing and geometry once.                   */
int ics_create(const ics_mesh_desc* mesh, const ics_config* cfg, ics_handle* out);
int ics_destroy(ics_handle h);
int ics_set_config(ics_handle h, const ics_config* cfg);
int ics_last_error(ics_handle h, char* buf, int32_t len);

/* ---- state --------------------------------------------------------------- */
/* Initial fields from primitive variables (0/p, 0/U, 0/T); boundary values
 * are evaluated from the patch kinds.  U is [n_cells][3].                   */
int ics_set_primitive(ics_handle h, const double* p, const double* U, const double* T);
/* Overwrite boundary values (p, U[3], T) and the boundary mass flux used by
 * inlet/outlet switching, all [n_bfaces] / [n_bfaces][3].                   */
int ics_set_boundary_state(ics_handle h, const double* p_b, const double* U_b,
                           const double* T_b, const double* phi_b);
int ics_get_boundary_state(ics_handle h, double* p_b, double* U_b, double* T_b, double* phi_b);
/* Any output may be NULL.  W is [n_cells][5].                               */
int ics_get_state(ics_handle h, double* W, double* p, double* U, double* T);
/* Overwrite the conservative state (also the old time levels when
 * set_old != 0) and re-derive primitives without touching boundary values. */
int ics_set_conservative(ics_handle h, const double* W, int32_t set_old);
/* Per-cell pseudo Courant number field (createFields.H:212-235).           */
int ics_set_pseudo_co(ics_handle h, const double* co);
int ics_get_pseudo_co(ics_handle h, double* co, double* rPseudoDeltaT);

/* ---- the hot path, one reference virtual per entry point ---------------- */
/* convectiveFluxScheme::calcFlux(phi, phiUp, phiEp)
 * (convectiveFluxScheme.H:219-224; ausmPlusUpFluxScheme.C:73-299,
 *  hllcFluxScheme.C:70-240, roeFluxScheme.C:276-409).  Outputs are
 * [n_faces+n_bfaces] (phiU: [..][3]); any may be NULL.                      */
int ics_calc_flux(ics_handle h, double* phi, double* phiU, double* phiE);
/* residualsUpdate.H:1-83 then setCoAndDeltaT.H:1-173: matrix source
 * R*V ([n_cells][5]) and the new local rPseudoDeltaT.  Calls calc_flux.     */
int ics_residual(ics_handle h, double* source);
/* convectiveFluxScheme::createConvectiveJacobian(coupledMatrix&, ddtCoeff)
 * (convectiveFluxScheme.C:537-546) + viscousFluxScheme::createViscousJacobian
 * (viscousFluxScheme.C:265-273).  Uses the state of the last ics_residual.  */
int ics_assemble_jacobian(ics_handle h);
/* Export the assembled blocks in LDU form: diag [n_cells][25],
 * lower/upper [n_faces][25] (blockFvMatrix.H:68-222 storage).               */
int ics_get_jacobian(ics_handle h, double* diag, double* lower, double* upper);
/* coupledMatrix::matrixMul (coupledMatrix.C:66-123): y = A x, [n_cells][5]. */
int ics_matrix_mul(ics_handle h, const double* x, double* y);
/* coupledMatrix::preconditioner::precondition (lusgs.C:220-385,
 * Jacobi.C:55-135): r <- P^-1 r in place.                                    */
int ics_precondition(ics_handle h, double* r);
/* coupledMatrix::solveForIncr -> solver::solveDelta (coupledMatrix.C:297-385,
 * gmres.C:772-1107).  Solves for the increment of the last assembly; dW
 * ([n_cells][5]) may be NULL.                                               */
int ics_solve_increment(ics_handle h, ics_solver_perf* perf, double* dW);
/* updateFields.H:1-105 (+ boundLocalTimeStep.H:1-97) with the increment of
 * the last solve.                                                            */
int ics_update_fields(ics_handle h, ics_iter_stats* stats);
/* One pseudo-time iteration: outerLoop.H:1-99 then updateFields.H.          */
int ics_pseudo_iteration(ics_handle h, ics_iter_stats* stats);
/* One pseudo-time iteration on each of n independent handles at once (a
 * batch of small cases): host threads drive the handles, whose kernels
 * overlap on their own streams; each handle keeps its own Krylov space and
 * controls, so every result equals that of ics_pseudo_iteration.  status[i]
 * (optional) receives each handle's status; the return value is the first
 * non-OK one.  The handles must be distinct.  (The reference runs such cases
 * one after another.)                                                        */
int ics_pseudo_iteration_batch(ics_handle* handles, int32_t n, ics_iter_stats* stats, int32_t* status);
/* Independent cases stacked in one handle (the many-small-cases batch as a
 * leading dimension): the handle's mesh is the union of n_cases meshes whose
 * cells case_start[k] .. case_start[k+1]-1 belong to case k (case_start
 * [n_cases+1], increasing, from 0 to n_cells) and no internal face joins two
 * cases.  Every kernel of a pseudo iteration then runs once over all cases,
 * while each case keeps what a handle of its own would have: its GMRES
 * (Hessenberg, Givens rotations, stop test coupledMatrixSolver.C:198-221 and
 * norm factors gmres.C:812-850), its SER pseudo Courant number
 * (setCoAndDeltaT.H:3-37) and its pseudotimeControl (pseudotimeControl.C:
 * 159-241): ics_pseudo_loop reports more work while any case runs, and a case
 * whose loop has completed is frozen (no update) until every case has
 * completed, after which the next call starts the next time step for all.
 * The dot products of case k reduce over segments that depend only on its own
 * cell count, so a case's results do not depend on the other cases in the
 * stack.  Call once, before the first residual.  Not with Harmonic Balance,
 * cyclic patches, the block-Jacobi smoother solver, the passive scalar or
 * checkpoints (ICS_ERR_ARG).
 * (CUDA library.)                                                            */
int ics_set_cases(ics_handle h, int32_t n_cases, const int32_t* case_start);
/* Per case of a stacked handle, each array [n_cases] and optional: the L2 norm
 * of R_rho V of the last residual (dbnsFoam.C:136-138), the GMRES restart
 * cycles of the last linear solve, and 1 while the case is frozen.         */
int ics_case_stats(ics_handle h, double* rho_l2, int32_t* gmres_cycles, int32_t* frozen);
/* Start a physical time step: shift old time levels, beginTimeStep.H:1-45.  */
int ics_begin_time_step(ics_handle h);
/* Harmonic Balance (dbnsFullyImplicitHBFoam outerLoop.H:1-230, HBZone.C:359-519):
 * the mesh given to ics_create holds n_instances stacked copies (instance J
 * owns cells [J*n, (J+1)*n), n = n_cells/n_instances).  D is the row-major
 * n_instances x n_instances spectral operator (HBZone::updateHBOperators).
 * Adds -V sum_K D_JK W_K to each instance's residual source, V D_JJ to the
 * diagonal and V D_JK I couplings to the Jacobian action; norm factors and
 * L1 residuals become per instance (solver_perf reports the maximum over
 * instances) and every instance keeps its own pseudotimeControl state
 * (ics_pseudo_loop answers 1 while any instance is not finished).  Needs
 * steadyState ddt and the GMRES solver; n_instances = 1 switches HB off.
 * Zones and cylindrical momentum sources: ics_set_hb_zone.                */
#define ICS_MAX_INSTANCES 16
int ics_set_hb(ics_handle h, int32_t n_instances, const double* D);
/* The HB zone of an HB handle (HBZone.C:100-165, 359-652): zone[n] (n =
 * n_cells / n_instances, the same cells in every instance; NULL: every cell)
 * marks the cells that carry the spectral source -V sum_K D_JK W_K and the
 * Jacobian's V D_JK couplings; the others carry neither (a cellZone).  With
 * cyl_coords the source combines each instance's momentum in cylindrical
 * components (radial, circumferential, axial about axis through origin, at
 * that instance's cell centre) and turns the sum back into Cartesian
 * components at the cell's own centre (HBZone cylCoords); the Jacobian's
 * couplings stay Cartesian, as the reference's addBlock.                    */
int ics_set_hb_zone(ics_handle h, const int32_t* zone, int32_t cyl_coords, const double axis[3],
                    const double origin[3]);
/* Moving reference frames (MRF zones): replaces the convectiveFluxScheme
 * fields MRFOmega / MRFFaceVelocity (convectiveFluxScheme.H:77-81,192-199)
 * and MRFCoupledZoneList::correctBoundaryVelocity as dbnsFoam sets them up
 * (outerLoop.H:6-21, createFields.H:262-266).  Arrays are in the handle's
 * cell / face numbering:
 *   omega[3*N]         rotation vector of each cell (zero outside zones)
 *   face_velocity[F+B] frame velocity . n of each internal then boundary
 *                      face (MRFZoneList::faceU() & Sf/|Sf|)
 *   boundary_U[3*B]    frame velocity of each boundary face
 *   included[B]        1 where correctBoundaryVelocity assigns boundary_U
 * The face velocity enters every flux scheme (relative normal velocities,
 * pressure work p u_MRF |S|), the wave speed of the local time step and of
 * the LF dissipation, the boundary Jacobian (U_rel . S) and the Jacobian
 * term -div(w, u_MRF |S|); omega adds the source -(omega x rho U) V and its
 * skew block to the diagonal (addMRFSource, convectiveFluxScheme.C:123-139).
 * The boundary velocity is assigned at every ics_begin_time_step and kept by
 * fixed-value patches (fixed, isothermal wall) through every update; with
 * mode ICS_MRF_EVERY_UPDATE (dbnsFullyImplicitHBFoam updateFields.H:88) it
 * is also re-assigned on every included face after each update.
 * omega == NULL switches the zones off.  The passive scalar uses the same
 * face velocity (calculateScalarTransport.H:96-145,217-290).                 */
/* Phase-lag cyclic patches of a Harmonic Balance handle (phaseLagCyclic,
 * src/fields/fvPatchFields/constraint/phaseLagCyclic): mode[n_patches] is 0
 * for a plain patch, 1 for a phase-lag cyclic patch, 2 for one whose velocity
 * is combined in cylindrical components (cylCoords); P[n_patches][n][n] holds,
 * for each phase-lag patch, Re(E^-1 M(IBPA) E) of its HB zone (M = diag(1,
 * e^{i k IBPA}, ..., e^{-i k IBPA}); the neighbour patch uses -IBPA).  Across
 * such a face the neighbour value of instance J of rho, p, the U components,
 * E, H and the sound speed is sum_K P_JK f_K(partner cell of instance K)
 * (phaseLagCyclicFvPatchField::patchNeighbourField); every other field and
 * the Jacobian couplings keep the plain cyclic neighbour of instance J.
 * mode == NULL switches phase lag off.                                      */
int ics_set_phase_lag(ics_handle h, const int32_t* mode, const double* P);
#define ICS_MRF_OUTER_LOOP 0
#define ICS_MRF_EVERY_UPDATE 1
int ics_set_mrf(ics_handle h, const double* omega, const double* face_velocity, const double* boundary_U,
                const int32_t* included, int32_t mode);
/* ---- passive scalar transport (dbnsFoam calculateScalarTransport.H) ----- */
/* Enable the transported scalar s: initial cell values s [n_cells], per
 * patch boundary condition patch_fixed[p] (1 fixedValue with patch_value[p],
 * 0 zeroGradient), diffusivity D (used when the case is viscous: the
 * laplacian(D, s) term and its Jacobian) and the reconstruct(s) scheme
 * (ICS_RECON_*).  rhoS = rho s is formed from the current density.  Not
 * available on Harmonic Balance handles.                                    */
int ics_scalar_enable(ics_handle h, const double* s, const int32_t* patch_fixed, const double* patch_value,
                      double D, int32_t recon_s);
/* n_iterations solves of the scalar equation at the current flow state
 * (dbnsFoam.C:126-133, after the pseudo iterations of a time step): Roe-type
 * upwind flux of rho s with Harten's fix, implicit 1x1-block LDU matrix
 * (convective, dissipation, boundary, viscous and dual-time terms), GMRES
 * with the flow solver's settings, rhoS += increment, s = rhoS / rho.  perf
 * receives the last solve's residuals (index 0).                            */
int ics_scalar_transport(ics_handle h, int32_t n_iterations, ics_solver_perf* perf);
/* Current s and rhoS [n_cells] (either may be NULL).                       */
int ics_get_scalar(ics_handle h, double* s, double* rhoS);

/* ---- failure detection (host-injected) ----------------------------------- */
/* Probe of the bounded device waits: one sync-free forward LU-SGS sweep on the
 * assembled Jacobian with row skip_row left out of the schedule, so its flag
 * is never raised; the rows that depend on it give up after spin_limit polls.
 * Returns ICS_ERR_TIMEOUT when the waits report as designed (ICS_OK when no
 * row depends on skip_row); the context stays usable.                       */
int ics_test_sweep_timeout(ics_handle h, int32_t skip_row, int32_t spin_limit);

/* ---- checkpoint / resume (the reference writes OpenFOAM time directories
 * and a pseudotimeState dictionary, pseudotimeControl.C:59-63,84-89) ------- */
/* Bytes of a checkpoint of this handle.                                    */
int ics_checkpoint_size(ics_handle h, int64_t* bytes);
/* Everything the next pseudo iteration reads -- conservative state, old time
 * levels, primitives, boundary values, pseudo Courant numbers and the last
 * local pseudo time steps, SER and
 * pseudotime-control state, passive scalar -- into a host buffer (raw binary
 * with a header).  A handle created with the same mesh and configuration
 * resumes from it bit for bit.                                              */
int ics_save_checkpoint(ics_handle h, void* buf, int64_t bytes);
/* Restore a checkpoint; ICS_ERR_ARG when it belongs to another mesh size,
 * instance count or scalar-transport setting.                              */
int ics_load_checkpoint(ics_handle h, const void* buf, int64_t bytes);

/* ---- differentiation of the residual (no counterpart in the reference,
 * whose Jacobian is the approximate one of ics_assemble_jacobian) --------- */
/* Jacobian-vector product of the residual source R V (the vector
 * ics_residual returns) with respect to the conservative state, at the
 * current state with the boundary values held fixed: Jv = d(R V)/dW v, by
 * forward-mode dual numbers through the residual kernels (the exact
 * derivative of the discrete residual, branch by branch).  v and Jv are
 * [n_cells][5]; device = 1 when both are device pointers on the handle's
 * device (inputs ready, outputs written before return), 0 for host arrays. */
int ics_jvp(ics_handle h, const double* v, double* Jv, int32_t device);
/* Assemble that exact Jacobian as 5x5 blocks over each cell's stencil (two
 * face hops, plus the other Harmonic Balance instances of the cell) by
 * coloured Jacobian-vector products.  Returns the number of blocks and of
 * colours (products = 5 x colours).  Valid until the state, the boundary
 * values or the configuration change.                                        */
int ics_assemble_exact_jacobian(ics_handle h, int64_t* nnz_blocks, int32_t* n_colours);
/* The assembled exact Jacobian in CSR form (host arrays): row_ptr
 * [n_cells+1], cols [nnz] increasing within a row, blocks [nnz][5][5] with
 * blocks[j][i][k] = d(R V)_i of the row cell / d(W_k) of cols[j].  Any
 * pointer may be NULL.  ICS_ERR_STATE when not assembled at this state.    */
int ics_get_exact_jacobian(ics_handle h, int32_t* row_ptr, int32_t* cols, double* blocks);
/* Vector-Jacobian product JTu = (d(R V)/dW)^T u with the exact Jacobian,
 * assembled first when the state changed.  Pointers as in ics_jvp.         */
int ics_vjp(ics_handle h, const double* u, double* JTu, int32_t device);
/* The same vector-Jacobian product by reverse mode, storing no Jacobian:
 * the face and cell maps of the residual are transposed in reverse order and
 * the fields, Gauss gradients and cellLimited limiters are recomputed from
 * the state in the backward pass (the flux's local partial derivatives by
 * dual numbers through the same flux function).  Equal to ics_vjp up to
 * round-off, and the exact transpose of ics_jvp's map.  Covers the inviscid
 * residual with every reconstruction (upwind, the TVD limitedSchemes,
 * linearUpwind with cellLimited gradients), all three flux schemes, the
 * physical ddt, MRF zones and Harmonic Balance (zones, cylCoords); returns
 * ICS_ERR_ARG for viscous cases and cyclic patches.  Pointers as in ics_jvp. */
int ics_vjp_recompute(ics_handle h, const double* u, double* JTu, int32_t device);
/* ---- Krylov solves with the exact residual derivative (no counterpart in
 * the reference, whose linear solves use the approximate Jacobian) ------- */
typedef struct {
  int32_t n_directions;   /* Krylov dimension (restart length), 1..64            */
  int32_t max_cycles;     /* restart cycles at most                               */
  double rel_tol;         /* stop when ||rhs - A x||_2 <= rel_tol ||rhs||_2        */
  int32_t precision;      /* ICS_PREC_FP64: FP64 Krylov basis; ICS_PREC_MIXED:
                             FP32 basis (operator and preconditioner stay FP64)   */
  int32_t preconditioner; /* ICS_PC_NONE, or ICS_PC_LUSGS: the LU-SGS of the
                             approximate Jacobian of the last ics_assemble_jacobian
                             (transposed for the adjoint system)                  */
  int32_t pseudo_time;    /* 1: add the local pseudo-time diagonal V / dtau of the
                             last ics_residual to the operator (the implicit
                             pseudo-time step), 0: the steady operator           */
} ics_krylov_opts;
typedef struct {
  int32_t iterations;     /* operator applications                                */
  int32_t cycles;         /* restart cycles                                       */
  double rel_residual;    /* final ||rhs - A x||_2 / ||rhs||_2 (recomputed)        */
  int32_t converged;
} ics_krylov_result;
/* The operator of both solves is A = s V / dtau - d(R V)/dW (s = the option
 * pseudo_time): the exact form of the matrix the reference assembles
 * approximately (its Jacobian of -R V plus the pseudo-time diagonal, which
 * ics_solve_increment solves with), so the approximate Jacobian's LU-SGS is a
 * consistent preconditioner.
 * Adjoint system A^T psi = g at the current state, by restarted
 * right-preconditioned GMRES whose operator is ics_vjp_recompute's reverse
 * chain (no Jacobian stored).  g and psi are host [n_cells][5].  Coverage as
 * ics_vjp_recompute; the LU-SGS preconditioner needs no cyclic patches.     */
int ics_adjoint_solve(ics_handle h, const double* g, double* psi, const ics_krylov_opts* opts,
                      ics_krylov_result* result);
/* Tangent (Newton) system A x = b at the current state with the forward-mode
 * product of ics_jvp in the operator: with pseudo_time = 1 and b the residual
 * source R V this is the pseudo-time Newton step of ics_solve_increment with
 * the exact Jacobian (matrix-free Newton-Krylov), preconditioned by the
 * reference's approximate one.                                              */
int ics_tangent_solve(ics_handle h, const double* b, double* x, const ics_krylov_opts* opts,
                      ics_krylov_result* result);
/* Integrated pressure force of one patch along dir: J = sum over its faces of
 * p (S . dir), with p the pressure of each face's cell (the patch's pressure
 * must be zeroGradient: slip, zeroGradient or isothermal wall patches), and,
 * when dJdW is not NULL, dJ/dW [n_cells][5] (host), the right-hand side of
 * the adjoint system of that functional.                                    */
int ics_pressure_force(ics_handle h, int32_t patch, const double dir[3], double* J, double* dJdW);
/* pseudotimeControl::loop() (pseudotimeControl.C:159-241): returns 1 in
 * *more while the pseudo loop should run another iteration.                 */
int ics_pseudo_loop(ics_handle h, int32_t* more);

/* ---- measurement (no counterpart in the reference, which has only Info logs) */
/* kernel classes timed by ics_profile_read                                  */
enum {
  ICS_K_FIELDS = 0, ICS_K_GRAD, ICS_K_FACE, ICS_K_BFACE, ICS_K_CELLRES, ICS_K_JAC_BOUNDARY, ICS_K_JAC_ROWS,
  ICS_K_JACOBI_INV, ICS_K_SPMV, ICS_K_LUSGS_FWD, ICS_K_LUSGS_REV, ICS_K_JACOBI, ICS_K_MGS, ICS_K_VECTOR,
  ICS_K_SCALAR, ICS_K_UPDATE, ICS_K_BC, ICS_K_BOUND, ICS_K_VISC, ICS_K_TANGENT, ICS_K_EXACT, ICS_K_OP0,
  ICS_K_OP1, ICS_K_PASSIVE, ICS_K_ADJOINT, ICS_K_COUNT
};
/* Start (enable=1) or stop (0) recording a CUDA event pair around every
 * kernel launch on the handle's stream; starting clears previous records.  */
int ics_profile(ics_handle h, int32_t enable);
/* Accumulated device time (ms) and launch count of one kernel class.        */
int ics_profile_read(ics_handle h, int32_t kind, double* ms, int64_t* launches);
/* Total kernels launched by the handle since creation.                      */
int ics_launch_count(ics_handle h, int64_t* launches);
/* Device timer on the handle's stream: start records an event, stop records
 * a second one, synchronises and returns the elapsed milliseconds.          */
int ics_timer_start(ics_handle h);
int ics_timer_stop(ics_handle h, double* ms);

/* Launch choices picked by the autotuner (no counterpart in the reference). */
typedef struct {
  int32_t face_block;      /* threads per block of the face-flux kernel (64 / 128)       */
  int32_t grad_block;      /* threads per block of the gradient kernel (64 / 128)        */
  int32_t mgs_blocks;      /* grid of the Gram-Schmidt steps (152 / 304 / 456 / 608)      */
  int32_t fused_operator;  /* 1: fused M^-1 A passes on two-level schedules, 0: SpMV then
                              LU-SGS sweeps                                              */
  int32_t from_cache;      /* 1: taken from an earlier tuning of a case of the same shape */
  int32_t reverse_rows;    /* rows per thread of the reverse LU-SGS level sweep (1 / 2:
                              two rows' slot loads in flight together)                   */
} ics_tuning;
/* Time each candidate launch choice on the handle's current state and
 * assembled Jacobian (CUDA events on its stream) and keep the fastest, for
 * this handle and -- cached per device, mesh shape, precision and scheme --
 * for later handles of the same shape, which take the cached choice without
 * timing.  Needs ics_residual and ics_assemble_jacobian first.  Every choice
 * computes the same result up to the order of floating-point sums.        */
int ics_autotune(ics_handle h, ics_tuning* out);
/* Apply launch choices, e.g. an ics_autotune result saved by the host for a
 * later run of the same case shape (from_cache is ignored).  Values outside
 * the candidate sets above are refused (ICS_ERR_ARG).                        */
int ics_set_tuning(ics_handle h, const ics_tuning* t);

/* FP64 fused multiply-add rate (GFLOP/s, an FMA = 2 flops) of the handle's
 * GPU, measured with CUDA events on the handle's stream by a kernel of
 * independent FMA chains on every SM: the peak against which the FP64-bound
 * residual kernels (face fluxes, gradients) are reported.                   */
int ics_measure_fp64_rate(ics_handle h, double* gflops);

/* ---- allocation-free entry point (no counterpart in the reference) ------ */
/* r = b - A x and the five per-equation L1 sums of r, with A the handle's
 * assembled Jacobian and b its last residual source, for callers that must
 * not allocate device memory while running: real-time drivers that allocate
 * only at start-up (an allocation mid-run can stall on the driver or fail
 * under memory pressure) and hosts that own every device buffer through
 * their own pool.  x, r ([n_cells][5]) and l1 ([5]) are caller-owned DEVICE
 * pointers; nothing is allocated or freed.  The only scratch is a fixed
 * file-scope device array sized for at most 2,097,152 cells: larger handles
 * return ICS_ERR_ARG, and so do Harmonic Balance and cyclic handles (A here
 * has neither coupling).  All calls share that array: calls that overlap on
 * the GPU race; calls on one stream are safe.  The call runs on the handle's
 * stream, with the handle's device made current for its duration, and
 * synchronises that stream before returning, so r and l1 are complete on
 * return; x must already be complete (a caller that wrote it on another
 * stream synchronises that stream first).  The first call on a device looks
 * up the array's address (cudaGetSymbolAddress) with that device current.   */
int ics_linear_residual_noalloc(ics_handle h, const double* x, double* r, double* l1);

#ifdef __cplusplus
}
#endif
#endif /* ICSFOAM_GB300_H */
