/*
 * dgadv.h -- C-ABI of the GB300-native explicit DG advection step.
 *
 * One library (libdgadv.so) holds (a) host helpers that rebuild the reference's static data
 * (grid incidence maps, quadrature rules, basis values) and (b) the device solver for the
 * per-stage operator of FESTUNG's advection problem:
 *     cDot = M^-1 ( L - K_D - K_N + (G1+G2) c - R c )          advection/solveSubStep.m:62-66
 *     c^(i) = w_i c^n + (1-w_i) (c^(i-1) + tau cDot)            advection/solveSubStep.m:83
 * with the vertex-based Taylor slope limiter              advection/solveSubStep.m:69-98.
 *
 * Every entry point returns a status code (DGADV_OK on success); no C++ exception and no
 * longjmp crosses this boundary.  Arrays are column-major (Fortran order) with the shapes the
 * reference keeps them in (K x N for cDisc, K x 3 x R for vNormalOnQuadEdge, ...), so a
 * MEX/oct gateway can pass mxArray data without transposes.  Integer inputs are 0-based int32;
 * integer outputs that the reference stores as "index or 0 for none" keep its values.
 *
 * Threading: calls for one handle must come from one host thread at a time.  Each handle owns
 * one CUDA stream; dgadv_step only enqueues work, dgadv_sync / dgadv_get_state wait for it.
 */
#ifndef DGADV_H
#define DGADV_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------------------- */
enum {
  DGADV_OK = 0,
  DGADV_EINVAL = 1,        /* invalid argument (null pointer, size, option)                */
  DGADV_ECUDA = 2,         /* CUDA runtime error                                           */
  DGADV_ENOMEM = 3,        /* host or device allocation failed                             */
  DGADV_EMESH = 4,         /* inconsistent mesh (non-manifold edge, bad vertex id, ...)     */
  DGADV_ENONFINITE = 5,    /* a kernel found NaN/Inf in the state                          */
  DGADV_ETIMEOUT = 6,      /* a bounded device-side wait gave up; after a wait of the stage
                              kernels (a staging copy, a grid barrier, a tensor-core MMA) the
                              handle's state is undefined and every later step or sweep on it
                              returns DGADV_ETIMEOUT: destroy it and create a new one       */
  DGADV_EUNSUPPORTED = 7,  /* option not supported by this build (e.g. p > 3 on the GPU)  */
  DGADV_EIO = 8,           /* an output file could not be written                          */
  DGADV_ENOCONV = 9        /* an iterative solve stopped before its tolerance               */
};

/* Arithmetic of the stored state and of every kernel: FP64; FP32; or DF32, each real an
 * unevaluated sum of two FP32 numbers (about 48 significant bits) computed on the FP32 units. */
enum { DGADV_FP64 = 0, DGADV_FP32 = 1, DGADV_DF32 = 2 };
enum { DGADV_LIM_LINEAR = 0, DGADV_LIM_HIERARCH_VERT = 1, DGADV_LIM_STRICT = 2 };
enum { DGADV_TIME_CONST = 0, DGADV_TIME_EXP_NEG = 1 };     /* g(t) = 1 or exp(-t) */

/* flags of dgadv_params.flags */
enum {
  DGADV_FLAG_NO_REORDER = 1,   /* keep the caller's element order on the device            */
  DGADV_FLAG_NO_SHIFT = 2,     /* patch min/max without the reference's global shift       */
  DGADV_FLAG_NO_GRAPH = 4,     /* launch stage kernels one by one instead of a CUDA graph  */
  DGADV_FLAG_NO_PDL = 8,       /* no programmatic dependent launch between stage kernels   */
  DGADV_FLAG_FUSE = 16,        /* linear limiter with zero Dirichlet data: apply the solution
                                  limiter inside the next stage's operator kernel            */
  DGADV_FLAG_PERSIST = 32,     /* one cooperative launch per time step with grid barriers
                                  (FP32 / FP64, linear limiter or none, no source terms)     */
  DGADV_FLAG_IMPLICIT = 64     /* the advection_implicit problem: volume integrals and velocity
                                  projections with the rule of order 2p+1; only implicit steps
                                  (dgadv_step_implicit, dgadv_solve_stationary), no limiter     */
};

/* options of dgadv_set_option (launch configuration: graph length and dependent launch leave
 * results bitwise unchanged; the fused pipeline changes them at the roundoff level) */
enum {
  DGADV_OPT_GRAPH_STEPS = 1,   /* time steps per captured CUDA graph, 1..256 (default 12)        */
  DGADV_OPT_FLAGS = 2,         /* the runtime flags NO_GRAPH, NO_PDL, FUSE, PERSIST              */
  DGADV_OPT_PERSIST_BLOCKS = 3, /* blocks per SM of the persistent step (0: all that fit)       */
  DGADV_OPT_ADJ_WARPS = 4,      /* warps per role of the adjoint stage kernel: 1, 2 or 4 (FP32
                                   default 2), or 0: one thread per element (FP64 default);
                                   1, 2 and 4 give the same gradients bit for bit, 0 agrees
                                   with them to roundoff                                      */
  DGADV_OPT_TAYLOR_MASS = 5,    /* time-derivative limiting's Taylor mass correction: 0 reads a
                                   stored per-element block, 1 rebuilds it from the element's B
                                   and a constant table (default: 1 in FP32, 0 otherwise); the
                                   results agree to roundoff                                   */
  DGADV_OPT_VOLUME_MMA = 6,     /* 1: the volume term's two contractions on the tensor cores
                                   (tcgen05, split TF32 with FP32 accumulation; FP32 handles,
                                   p >= 2, time-derivative limiting, no source terms); 0 (the
                                   default): FP32 multiply-adds                                */
  DGADV_OPT_OP_BLOCK = 7,       /* elements per thread block of the stage operator, one thread
                                   per element: 64 or 128 (default); results unchanged        */
  DGADV_OPT_OPERATOR_FP32 = 8,  /* double-float handles: 1 computes the stage operator (volume,
                                   flux, mass) in FP32 arithmetic while the state, the SSP
                                   update and the limiter stay double-float; 0 (default): all
                                   double-float                                              */
  DGADV_OPT_ADJ_STREAMS = 9,    /* streams of a reverse sweep that recomputes: 3 (default) runs
                                   the recomputation of the reversed steps on a second stream,
                                   one reversed step ahead of the reverse stages, and the
                                   advances between checkpoints on a third, with checkpoint
                                   slots renamed so that an advance need not wait for the slot
                                   the schedule reuses; 2: recomputation and advances on one
                                   second stream; 1: one stream.  2 and 3 take one and two more
                                   sets of work states and limiter records (and with 3 the
                                   limiter's key sets), allocated by dgadv_forward_record.
                                   Gradients bitwise unchanged                                 */
  DGADV_OPT_ELEMENT_OPERATOR = 10, /* FP64 and double-float handles without source terms (and,
                                   double-float, without the FP32 operator): 1 (default) keeps the
                                   stage operator's volume term and the element's own outflow
                                   terms as one N x N matrix per element (N^2 reals per element,
                                   rebuilt whenever the velocity changes), which takes the FP64
                                   operator from about 244 to about 100 arithmetic instructions
                                   per element at p = 2; 0: evaluated at the quadrature points.
                                   The results agree to roundoff                              */
  DGADV_OPT_ADJ_GRAPH = 11      /* the reverse sweep captured as one CUDA graph (1) or launched
                                   directly (0); -1 (default): 1 without the limiter, 0 with it.
                                   Gradients bitwise unchanged                                */
};

/* ---- host helpers: static data ------------------------------------------------------- */

/* Output of generateGridData (core/generateGridData.m:130-198).  Allocated by
 * dgadv_grid_build, released by dgadv_grid_free. */
typedef struct dgadv_grid {
  int32_t numT, numV, numE;
  int32_t *V0E;      /* numE x 2   0-based vertex ids (reference V0E - 1)                  */
  int32_t *T0E;      /* numE x 2   1-based element ids, 0 = none (reference T0E)           */
  int32_t *E0T;      /* numT x 3   0-based edge ids (reference E0T - 1)                    */
  int32_t *E0E;      /* numE x 2   1-based local edge index, 0 = none (reference E0E)      */
  double *areaE;     /* numE                                                               */
  double *nuE;       /* numE x 2                                                           */
  double *baryE;     /* numE x 2                                                           */
  double *areaT;     /* numT                                                               */
  double *baryT;     /* numT x 2                                                           */
  double *B;         /* numT x 2 x 2                                                       */
  double *areaE0T;   /* numT x 3                                                           */
  double *nuE0T;     /* numT x 3 x 2                                                       */
  double *coordV0T;  /* numT x 3 x 2                                                       */
  double *detJ0T;    /* numT                                                               */
} dgadv_grid;

/* Replaces generateGridData(coordV, V0T), core/generateGridData.m:130-198 (without the K x K
 * masks markE0TE0T / markV0TV0T, whose content is carried by T0E/E0E). */
int dgadv_grid_build(int32_t numV, const double *coordV, int32_t numT, const int32_t *V0T,
                     dgadv_grid **out);
void dgadv_grid_free(dgadv_grid *grid);

/* Replaces quadRule1D(qOrd) (core/quadRule1D.m:48-95), points on [0,1].  With Q == NULL only
 * *R is written. */
int dgadv_quad_rule_1d(int32_t qOrd, int32_t *R, double *Q, double *W);
/* Replaces quadRule2D(qOrd) (core/quadRule2D.m:64-109; orders >= 7 as core/triquad.m). */
int dgadv_quad_rule_2d(int32_t qOrd, int32_t *R, double *Q1, double *Q2, double *W);
/* Replaces phi(i,X1,X2) / gradPhi(i,m,X1,X2) for i = 1..N (core/phi.m:40-61,
 * core/gradPhi.m:42-87): phi is nPts x N, gradPhi nPts x N x 2 (may be NULL). */
int dgadv_basis_eval(int32_t N, int32_t nPts, const double *X1, const double *X2, double *phi,
                     double *gradPhi);

/* ---- device solver -------------------------------------------------------------------- */

typedef struct dgadv_mesh {
  int32_t numT, numV;
  const double *coordV;        /* numV x 2                                                  */
  const int32_t *V0T;          /* numT x 3, 0-based, counter-clockwise                      */
  const int32_t *idE0T;        /* numT x 3 boundary ids (0 = interior) or NULL: every
                                  boundary edge counts as identified                       */
  const uint8_t *markE0TbdrD;  /* numT x 3 Dirichlet boundary edges or NULL: all boundary   */
  const uint8_t *markE0TbdrN;  /* numT x 3 Neumann boundary edges or NULL: none             */
} dgadv_mesh;

typedef struct dgadv_params {
  int32_t p;             /* polynomial degree 0..3 (the reference allows 0..4)              */
  int32_t ordRK;         /* SSP-RK order 1..3 (core/rungeKuttaExplicit.m:64-78)             */
  int32_t precision;     /* DGADV_FP64, DGADV_FP32 or DGADV_DF32                            */
  int32_t isSlopeLim;    /* vertex-based Taylor limiter on/off                              */
  int32_t typeSlopeLim;  /* DGADV_LIM_*                                                     */
  int32_t device;        /* CUDA device ordinal                                             */
  int32_t flags;         /* DGADV_FLAG_*                                                    */
} dgadv_params;

typedef struct dgadv_handle dgadv_handle;

/* Replaces the device-independent part of advection/preprocessProblem.m:48-112: grid, tables,
 * mass and Taylor data for one mesh; uploads everything once.  On failure *out may still hold a
 * handle (so that dgadv_last_error can explain); release it with dgadv_destroy. */
int dgadv_create(const dgadv_mesh *mesh, const dgadv_params *params, dgadv_handle **out);

/* An ensemble: one handle over the disjoint union of nInst meshes, so that every stage kernel
 * covers all instances in one launch.  Each instance needs a multiple of 128 triangles and
 * keeps its own limiter extremes (the reference's global shift is per problem).  The handle's
 * arrays (cDisc, velocity data, ...) are the instances' arrays stacked in instance order.  The
 * reference runs one problem at a time; this has no counterpart there. */
int dgadv_create_ensemble(const dgadv_mesh *meshes, int32_t nInst, const dgadv_params *params,
                          dgadv_handle **out);

/* Velocity data of advection/preprocessSubStep.m:72-79: u1Disc, u2Disc (K x N, projections of
 * order 2p) and vNormalOnQuadEdge (K x 3 x R, order 2p+1).  Held until replaced. */
int dgadv_set_velocity(dgadv_handle *h, const double *u1Disc, const double *u2Disc,
                       const double *vNormalOnQuadEdge);

/* Right-hand-side data of advection/preprocessSubStep.m:87-98 and the limiter's boundary
 * values (advection/solveSubStep.m:86-88) as separable terms:
 *     sysV(t)  = sum_m g_m(t) rhs_m          rhs_m = L_m - K_D,m - K_N,m      (K x N each)
 *     cDV0T(t) = sum_m g_m(t) cDV0T_m                                         (K x 3 each)
 * g_m = timeFn[m] (DGADV_TIME_*).  nTerms = 0 means zero data (the default).  cDV0T may be
 * NULL (zero boundary values). */
int dgadv_set_source_terms(dgadv_handle *h, int32_t nTerms, const int32_t *timeFn,
                           const double *rhsTerms, const double *cDV0T);

/* cDisc (K x N) in and out (advection/solveStep.m:67-68, advection/postprocessStep.m:58). */
int dgadv_set_state(dgadv_handle *h, const double *cDisc);
int dgadv_get_state(dgadv_handle *h, double *cDisc);

/* applySlopeLimiterDisc on the current state with boundary data at time t
 * (advection/initializeProblem.m:56-67). */
int dgadv_limit_state(dgadv_handle *h, double t);

/* Enqueues time steps nStep0+1 .. nStep0+nSteps (advection/solveStep.m:57-73 with all its
 * sub-steps); step n uses t0 = (n-1)*tau as the reference.  Asynchronous. */
int dgadv_step(dgadv_handle *h, int32_t nSteps, int32_t nStep0, double tau);

/* Waits for enqueued work; reports DGADV_ENONFINITE if a kernel saw NaN/Inf. */
int dgadv_sync(dgadv_handle *h);

/* Runs dgadv_step between two CUDA events recorded on the handle's stream and waits; *ms is
 * the device time of the enqueued steps. */
int dgadv_time_steps(dgadv_handle *h, int32_t nSteps, int32_t nStep0, double tau, double *ms);

/* Runs nSteps with one launch per kernel and CUDA events around every launch; writes the mean
 * device time per launch (ms) and the launch count for each kernel kind:
 * [0] stage operator, [1] time-derivative limiter + SSP, [2] solution limiter, [3] unused. */
int dgadv_profile_kernels(dgadv_handle *h, int32_t nSteps, int32_t nStep0, double tau,
                          double *msPerLaunch, int32_t *launches);

/* Launch configuration of a handle (DGADV_OPT_*), e.g. as chosen by an autotuner.  Changing it
 * drops the handle's captured graphs; the state is kept.  No counterpart in the reference. */
int dgadv_set_option(dgadv_handle *h, int32_t option, int32_t value);
int dgadv_get_option(const dgadv_handle *h, int32_t option, int32_t *value);

/* Failure-detection self-test: a device wait on a flag that nothing sets gives up after
 * `seconds` (at most 2) and the call returns DGADV_ETIMEOUT, as every bounded wait of the stage
 * kernels does; the error is then cleared and the handle stays usable.  No counterpart in the
 * reference. */
int dgadv_selftest_wait(dgadv_handle *h, double seconds);

/* ---- implicit time stepping (advection_implicit) ----------------------------------------
 * Each stage of the diagonally implicit Runge-Kutta method of core/rungeKuttaImplicit.m solves
 * (M + tau a_ii A) x_i = tau a_ii sysV(t_i) + M c^n + sum_j tau a_ij rhs_j
 * (advection_implicit/solveSubStep.m).  The reference uses a sparse direct solver; here the
 * system, multiplied by M^-1, is solved matrix-free by restarted GMRES with a block-Jacobi
 * preconditioner (the inverse of each element's diagonal block), to a relative residual tol. */
typedef struct dgadv_krylov {
  double tol;          /* relative residual of every solve (default 1e-12)                     */
  int32_t maxIter;     /* iterations per solve (default 2000)                                  */
  int32_t restart;     /* Krylov vectors before a restart, 1..256 (default 50)                 */
} dgadv_krylov;

/* Replaces advection_implicit/solveStep.m and its sub-steps: steps nStep0+1 .. nStep0+nSteps
 * of order ordRK (1..4) with step size tau, source terms at the stage times.  kr may be NULL
 * (defaults).  iters receives the GMRES iterations, relres the largest final relative residual
 * (either may be NULL).  DGADV_ENOCONV if a solve stopped at maxIter.  Synchronous. */
int dgadv_step_implicit(dgadv_handle *h, int32_t nSteps, int32_t nStep0, double tau, int32_t ordRK,
                        const dgadv_krylov *kr, int32_t *iters, double *relres);

/* The stationary problem A c = sysV(0) (advection_implicit/solveSubStep.m, isStationary), with
 * the current state as the initial guess; the solution becomes the state. */
int dgadv_solve_stationary(dgadv_handle *h, const dgadv_krylov *kr, int32_t *iters, double *relres);

/* ---- transport of several species (transport/) -----------------------------------------
 * The transport problem without coupling to a flow model: species advected as depth-integrated
 * concentrations c h with the depth-integrated velocity (u h, v h), which the handle holds
 * (dgadv_set_velocity with the projections of u h, v h).  Each species is advected only over
 * its active elements (its mask, recomputed after every step from the limiter's patch extremes,
 * core/computeMask.m 'vertex-based'), and its concentration c = Pi(c h / h) is limited with the
 * handle's linear vertex limiter (zero Dirichlet data).  The handle must be explicit, with the
 * linear limiter and p >= 1, in FP64 or FP32. */

/* Replaces transport/initializeProblem.m: hDisc (K x N) the depth, cH0 (K x N x nSpecies) the
 * projections of c h at t = 0; each species' concentration is formed, limited, and its mask
 * computed (isMask = 0: every element stays active). */
int dgadv_transport_init(dgadv_handle *h, int32_t nSpecies, const double *hDisc, const double *cH0,
                         double maskTol, int32_t isMask);

/* Replaces transport/solveStep.m with its sub-steps and transport/postprocessStep.m: steps
 * nStep0+1 .. nStep0+nSteps of the handle's SSP-RK order. */
int dgadv_transport_step(dgadv_handle *h, int32_t nSteps, int32_t nStep0, double tau);

/* Species s: c h and c (K x N each) and the mask (K, 1 = active); any output may be NULL. */
int dgadv_transport_get(dgadv_handle *h, int32_t species, double *cH, double *conc, uint8_t *mask);

/* ---- set-up on the device ------------------------------------------------------------
 * The reference hands its data to the solver as closures (advection/configureProblem.m:106-133)
 * and evaluates them on the host.  Here the built-in test cases' functions are device
 * functions, selected by kind with their parameters, so the steps either side of the time loop
 * (projections, velocity data, L2 errors) run on the GPU.  An ensemble handle takes one
 * function for every instance (nFn = 1) or one per instance (nFn = number of instances). */
#define DGADV_FN_MAX_PARAMS 64
enum {
  DGADV_FN_CONST = 0,        /* params[0]                                                      */
  DGADV_FN_POLY3 = 1,        /* params . (1, x, y, x^2, xy, y^2, x^3, x^2 y, x y^2, y^3)         */
  DGADV_FN_SOLID_BODY = 2,   /* c0 of 'solid_body': slotted cylinder, cone, hump (:109-113)     */
  DGADV_FN_GAUSS_SLOT = 3,   /* exp(-((x-0.25)^2 + (y-0.5)^2) / 0.01) + the slotted cylinder     */
  DGADV_FN_GAUSS = 4,        /* exp(-((x-p0)^2 + (y-p1)^2) / p2), p2 the squared width          */
  DGADV_FN_TRANSIENT = 5,    /* cCont of 'transient': cos(7x) cos(7y) + exp(-t) (:126)          */
  DGADV_FN_COS7 = 6,         /* cos(7x) cos(7y) ('stationary' of advection_implicit/getTestcase.m) */
  DGADV_VEL_ROTATION = 16,   /* u = (0.5 - y, x - 0.5) ('solid_body', :115-116)                 */
  DGADV_VEL_TRANSIENT = 17,  /* u = (exp((x+y)/2), exp((x-y)/2)) ('transient', :127-128)        */
  DGADV_VEL_STREAM = 18,     /* u = (dpsi/dy, -dpsi/dx), psi = sum_m a_m sin(k_m pi x) sin(l_m pi y),
                                params k[M], l[M], a[M] (nParams = 3M)                          */
  DGADV_VEL_CONST = 19       /* u = (params[0], params[1])                                        */
};
typedef struct dgadv_function {
  int32_t kind;              /* DGADV_FN_* or DGADV_VEL_*                                       */
  int32_t nParams;           /* at most DGADV_FN_MAX_PARAMS                                     */
  const double *params;
} dgadv_function;

/* Replaces projectFuncCont2DataDisc of the initial data (core/projectFuncCont2DataDisc.m:94-102,
 * advection/initializeProblem.m:53): the state becomes the L2 projection of f(t, x) with the
 * 2D rule of order max(qOrd, 1) (at most 20).  Synchronous. */
int dgadv_project_state(dgadv_handle *h, const dgadv_function *f, int32_t nFn, double t,
                        int32_t qOrd);

/* Replaces the host velocity data of dgadv_set_velocity (advection/preprocessSubStep.m:72-79):
 * u1Disc, u2Disc projected with order 2p and the normal velocity at the order-(2p+1) edge
 * points, evaluated on the device.  Synchronous. */
int dgadv_set_velocity_function(dgadv_handle *h, const dgadv_function *u, int32_t nFn);

/* Replaces computeL2Error (core/computeL2Error.m:97-114) for the current state against f(t, x)
 * with the rule of order max(qOrd, 1): err[0], or err[i] for each instance when nFn is the
 * number of instances.  Synchronous. */
int dgadv_l2_error(dgadv_handle *h, const dgadv_function *f, int32_t nFn, double t, int32_t qOrd,
                   double *err);

/* ---- solution output ------------------------------------------------------------------
 * The reference writes u_h at the Lagrange nodes of each triangle (projectDataDisc2DataLagr):
 * numP = 1 value at the centroid (p = 0), 3 at the vertices (p = 1), or 6 at the vertices and
 * edge midpoints (p >= 2), as VTK XML (.vtu) and / or Tecplot ASCII (.plt) files named
 * <fileName>.<tLvl>.vtu / .plt (core/visualizeDataLagr.m:114-291, scalar data); missing
 * directories of fileName are created. */
enum { DGADV_OUT_VTK = 1, DGADV_OUT_TEC = 2 };

/* Replaces core/projectDataDisc2DataLagr.m:43-57 on the current state: dataLagr is K x numP
 * (*numP written if not NULL).  Synchronous. */
int dgadv_get_lagrange(dgadv_handle *h, double *dataLagr, int32_t *numP);

/* Replaces the output of advection/outputStep.m:53-66 (projectDataDisc2DataLagr +
 * visualizeDataLagr): evaluates the nodal values on the device, copies them to a pinned host
 * buffer on the handle's stream and returns; a writer thread of the handle writes the files
 * when the copy has landed, while later steps run.  At most two outputs are in flight (a third
 * call waits for the writer). */
int dgadv_output(dgadv_handle *h, const char *varName, const char *fileName, int32_t tLvl,
                 int32_t fileTypes);

/* Waits until every output file of the handle is written; DGADV_EIO (message in
 * dgadv_last_error) if one could not be.  dgadv_destroy also finishes pending files. */
int dgadv_output_wait(dgadv_handle *h);

/* Host-only writer, core/visualizeDataLagr.m:114-291 for one scalar variable: the mesh
 * in the layout of dgadv_mesh: coordV numV x 2, V0T numT x 3, 0-based; dataLagr numT x numP with
 * numP in {1, 3, 6}. */
int dgadv_write_lagrange(int32_t numT, int32_t numV, const double *coordV, const int32_t *V0T,
                         int32_t numP, const double *dataLagr, const char *varName,
                         const char *fileName, int32_t tLvl, int32_t fileTypes);

/* Number of kernels one time step launches (for launch accounting; for a handle with linked
 * handles, the launches of the linked step). */
int dgadv_kernels_per_step(const dgadv_handle *h, int32_t *count);

/* Linked stepping (the batched launch of an ensemble whose instances differ in degree; no
 * counterpart in the reference, whose problems run one at a time through main.m): links
 * `other` to `h`, after which dgadv_step / dgadv_time_steps on h advance h and every handle
 * linked to it with one launch per stage kernel covering all their elements, on h's stream.
 * Each handle keeps its own state, tables, limiter extremes and RK order (a handle with fewer
 * stages sits out the later stages of a step); results are bitwise those of stepping each
 * handle alone.  Same device and precision (FP64 or FP32), degrees 1..3, the linear limiter or
 * none, no source or boundary terms, the separate-pass pipeline; at most 3 handles linked to
 * one.  A linked handle is not stepped on its own (DGADV_EUNSUPPORTED) until unlinked;
 * dgadv_sync(h) reports the linked handles' non-finite flags too.  other == NULL unlinks every
 * handle linked to h; destroying either handle unlinks it. */
int dgadv_link(dgadv_handle *h, dgadv_handle *other);

const char *dgadv_last_error(const dgadv_handle *h);
const char *dgadv_status_string(int status);
void dgadv_destroy(dgadv_handle *h);

/* ---- discrete adjoint ------------------------------------------------------------------
 * Gradients of a functional J(c(T)) of the final state of an explicit run (unlimited, or with
 * the linear, the hierarchical vertex-based or the strict limiter) with respect to the initial
 * coefficients and to the coefficients theta of a velocity u = sum_m theta_m u_m.  The
 * reference has no adjoint; these follow the torch.autograd.Function contract (forward
 * records, backward maps dJ/dc(T) to the input gradients).  The upwind choice is frozen at the
 * recorded velocity (the flux is piecewise linear in u), and so are the limiters' choices
 * (which vertex bound and which order is active): the gradient is that of the
 * piecewise-smooth map on the recorded piece.
 * Right-hand-side vectors set with dgadv_set_source_terms are treated as independent of theta. */

/* Velocity modes u_m, each given like dgadv_set_velocity: u1Modes, u2Modes K x N x nModes,
 * vNModes K x 3 x R x nModes. */
int dgadv_set_velocity_modes(dgadv_handle *h, int32_t nModes, const double *u1Modes,
                             const double *u2Modes, const double *vNModes);
/* Sets the velocity to sum_m theta[m] u_m (replaces dgadv_set_velocity). */
int dgadv_set_velocity_theta(dgadv_handle *h, const double *theta);
/* Runs nSteps steps from the current state (steps 1..nSteps, t0 = 0) and keeps what
 * dgadv_backward needs: nSnapshots <= 0 keeps every step state and every RK stage state (no
 * recomputation; nSteps x ordRK state-sized buffers); nSnapshots >= nSteps keeps every step
 * state (each reversed step recomputes its stages); otherwise nSnapshots states are placed by
 * binomial checkpointing.  The final state is then the handle's state (dgadv_get_state).
 * DGADV_EUNSUPPORTED with DGADV_FLAG_IMPLICIT or in DF32. */
int dgadv_forward_record(dgadv_handle *h, int32_t nSteps, double tau, int32_t nSnapshots);
/* Reverse sweep of the last recorded run: dJdcT (K x N) in, dJdc0 (K x N, may be NULL) and
 * dJdtheta (nModes, may be NULL) out.  Recomputes what was not stored; the handle's state is
 * the initial state afterwards.  One backward per recorded run. */
int dgadv_backward(dgadv_handle *h, const double *dJdcT, double *dJdc0, double *dJdtheta);
/* The checkpointing schedule as pairs (action, argument): 0 restore slot, 1 advance n steps,
 * 2 store slot, 3 reverse step; *backwardStart = first action of the reverse sweep.  With
 * actions == NULL only *count is written.  Host only. */
int dgadv_checkpoint_schedule(int32_t nSteps, int32_t nSnapshots, int32_t *actions, int32_t *count,
                              int32_t *backwardStart);

/* Largest vertex count dgadv_limit_linear_noalloc accepts (its fixed scratch: 4 MB per GPU). */
#define DGADV_NOALLOC_MAX_VERTICES (1 << 18)

/* One pass of the linear vertex-based slope limiter on device arrays the caller owns, with no
 * device allocation by this call or by the library on its behalf.  This entry point has no
 * counterpart in the reference; it exists for callers that cannot call cudaMalloc, e.g. code
 * whose device memory all comes from another framework's pool (an allocation outside the pool
 * breaks its accounting), code held to a device-memory budget fixed in advance, or code that
 * must not trigger the device-wide synchronisation an allocation can cause.
 *
 * Same result as one solution-limiter pass of a handle created with typeSlopeLim =
 * DGADV_LIM_LINEAR and precision DGADV_FP64 (FP64 arithmetic, the reference's global shift).
 * Device arrays, column-major in element order, 0-based ids:
 *   V0T          numT x 3 int32 vertex ids, each in [0, numV); the kernels check this, and an
 *                element with an id outside that range enters no vertex patch and gets NaN in
 *                every coefficient of cOut (no memory outside the arrays is touched)
 *   markV0TbdrD  numT x 3 uint8, non-zero at Dirichlet vertices (NULL: none)
 *   dataV0T      numT x 3 Dirichlet values at those vertices (NULL: zero)
 *   cIn, cOut    numT x N modal coefficients, N = (p+1)(p+2)/2; cOut may equal cIn
 * p is 1, 2 or 3.  numV above DGADV_NOALLOC_MAX_VERTICES returns DGADV_ENOMEM.  The scratch is
 * a file-scope __device__ array that every GPU loading the library holds until the process
 * exits.  The first call on a device (and the first per degree p) does a synchronous set-up
 * with that device current: it looks up the array's device address and uploads the degree's
 * constant tables; make that first call before any stream capture.  All calls on a device
 * share the one array, which keeps the previous call's contents (each call clears what it
 * needs at its start), so calls whose work overlaps on the GPU (different streams, or
 * different host threads, without ordering between them) race and give wrong results.
 * Enqueued on `stream` (a cudaStream_t, NULL = default stream); asynchronous. */
int dgadv_limit_linear_noalloc(int32_t p, int32_t numT, int32_t numV, const int32_t *V0T,
                               const uint8_t *markV0TbdrD, const double *dataV0T,
                               const double *cIn, double *cOut, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* DGADV_H */
