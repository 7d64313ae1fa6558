/*
 * xg.h -- C ABI of libxg, a single-GPU (sm_103a) implementation of the
 * node-centred edge-based finite-element hot path of Xyst's Inciter:
 *
 *   - RieCG: superedge nodal gradients, MUSCL/Rusanov|HLLC edge and boundary
 *     residual, low-storage 3-stage RK update, nodal BCs, CFL time step;
 *   - KozCG: element Taylor-Galerkin residual with flux-corrected transport;
 *   - ChoCG: projection step of incompressible flow (chorin:: edge passes,
 *     explicit RK momentum prediction, pressure-increment Poisson solve);
 *   - ConjugateGradients: CSR matrix-vector product and preconditioned CG.
 *
 * Every entry point returns an int status (XG_OK on success) and never throws;
 * xg_last_error() returns a message for the last failure on a context.  All
 * arrays are plain host pointers with sizes, laid out exactly like the
 * reference's containers:
 *   - tk::Fields (node-major, src/Base/Data.hpp:419-426): U[i*ncomp + c];
 *   - coordinates as three consecutive arrays x[npoin], y[npoin], z[npoin]
 *     (std::array<std::vector<tk::real>,3> flattened);
 *   - ids as uint64_t (std::size_t on LP64), zero based.
 * One context owns one CUDA stream on one device; a context must be used from
 * one host thread at a time.
 */
#ifndef XG_H
#define XG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct xg_ctx xg_ctx;
typedef struct xg_lpc xg_lpc;  /* learned preconditioner model (xg_lpc_*) */

enum xg_status {
  XG_OK = 0,
  XG_ERR_ARG = 1,      /* invalid argument (sizes, ids out of range, ...) */
  XG_ERR_CUDA = 2,     /* a CUDA runtime call failed */
  XG_ERR_STATE = 3,    /* call out of order (e.g. no operators uploaded) */
  XG_ERR_BLOWUP = 4,   /* dt below machine epsilon (RieCG::advance blowup) */
  XG_ERR_NOTCONV = 5,  /* CG stopped without reaching the tolerance */
  XG_ERR_DEVICE = 6,   /* a kernel reported an error status */
  XG_ERR_HOST = 7      /* host-side failure: out of host memory, threads refused */
};

enum xg_precision {
  XG_FP64 = 0,       /* everything in double precision */
  XG_FP32_FLUX = 1   /* FP32 gradients and fluxes, FP64 state and update */
};

enum xg_flux { XG_RUSANOV = 0, XG_HLLC = 1 };

/* Problems with a manufactured source term in riemann::rhs (riemann::src,
 * src/Physics/Riemann.cpp:880-907, the src functions of
 * src/Physics/Problems.cpp).  The scalar-transport problems (slot_cyl,
 * sheardiff) carry more than five components and are not offered. */
enum xg_source {
  XG_SRC_NONE = 0,
  XG_SRC_TAYLOR_GREEN = 1,
  XG_SRC_VORTICAL_FLOW = 2,
  XG_SRC_NONLINEAR_ENERGY_GROWTH = 3,
  XG_SRC_RAYLEIGH_TAYLOR = 4
};

/* Physics and numerics settings the reference reads from its global config
 * (mat.spec_heat_ratio, flux, stab2, stab2coef, cfl, dt). */
typedef struct xg_riecg_params {
  double gamma;      /* ratio of specific heats */
  int flux;          /* enum xg_flux */
  int stab2;         /* nonzero: artificial viscosity on the edge flux */
  double stab2coef;  /* its coefficient */
  double cfl;        /* CFL number (used when const_dt == 0) */
  double const_dt;   /* constant time step if |const_dt| > eps */
  int precision;     /* enum xg_precision */
} xg_riecg_params;

/* ---- context ------------------------------------------------------------ */
int xg_create(int device, xg_ctx** ctx);
int xg_destroy(xg_ctx* ctx);
const char* xg_last_error(const xg_ctx* ctx);
/* Bytes of device memory the context currently holds. */
int xg_device_bytes(const xg_ctx* ctx, int64_t* bytes);

/* ---- RieCG -------------------------------------------------------------- */

/* Upload the finite-element operators RieCG builds once per mesh
 * (RieCG::feop/streamable/domsuped, src/Inciter/RieCG.cpp:247-736): node
 * coordinates and volumes, the three superedge groups exactly as
 * RieCG::m_dsupedge/m_dsupint (tets: 4 ids + 6x3 integrals; triangles:
 * 3 ids + 3x3; edges: 2 ids + 3), the boundary triangles m_triinpoel and
 * their symmetry flags m_besym.  Counts are in groups.  Replaces the
 * operator arguments of riemann::grad/rhs (src/Physics/Riemann.hpp:17-39).
 * Re-upload after any mesh change. */
int xg_riecg_setup(xg_ctx* ctx, const xg_riecg_params* prm, int64_t npoin,
                   const double* coord, const double* vol,
                   int64_t ntet, const uint64_t* dsupedge0, const double* dsupint0,
                   int64_t ntri, const uint64_t* dsupedge1, const double* dsupint1,
                   int64_t nedge, const uint64_t* dsupedge2, const double* dsupint2,
                   int64_t nbtri, const uint64_t* triinpoel, const uint8_t* besym);

/* Nodal boundary conditions as RieCG::setupBC/streamable store them
 * (src/Inciter/RieCG.cpp:109-245, 527-618), applied by RieCG::BC
 * (RieCG.cpp:764-785) in the order Dirichlet, symmetry, farfield, pressure:
 *   sym:  m_symbcnodes / m_symbcnorms (a node may repeat, once per set);
 *   far:  m_farbcnodes / m_farbcnorms and the farfield state far5 =
 *         {density, u, v, w, pressure};
 *   dir:  node ids, 5 mask ints per node and 5 values per node
 *         (physics::dirbc, src/Physics/BC.cpp:30-71): with a problem set
 *         (xg_riecg_set_source) a component of mask 1 takes the problem's
 *         analytic state at the BC's time (t + dt/3, t + dt/2, t + dt in the
 *         stages, RieCG.cpp:1028; t in xg_riecg_bc); any other nonzero mask
 *         sets the given value;
 *   pre:  m_prebcnodes / m_prebcvals (density, pressure per node).
 * Any count may be zero. */
int xg_riecg_set_bc(xg_ctx* ctx,
                    int64_t nsym, const uint64_t* symnodes, const double* symnorms,
                    int64_t nfar, const uint64_t* farnodes, const double* farnorms,
                    const double* far5,
                    int64_t ndir, const uint64_t* dirnodes, const int32_t* dirmask,
                    const double* dirvals,
                    int64_t npre, const uint64_t* prenodes, const double* prevals);

/* Device-resident state U (npoin x 5, node-major), time t.  U in pinned
 * (page-locked) host memory is read / written by the kernels directly over
 * the host link; other host memory goes through a staging copy. */
int xg_riecg_set_state(xg_ctx* ctx, const double* U, double t);
int xg_riecg_get_state(xg_ctx* ctx, double* U, double* t);

/* Drop-in for riemann::grad (src/Physics/Riemann.cpp:229-367): weak nodal
 * gradients of primitive variables from host U (npoin x 5) into host G
 * (npoin x 15), not divided by the nodal volume. */
int xg_riecg_grad(xg_ctx* ctx, const double* U, double* G);

/* Drop-in for riemann::rhs (src/Physics/Riemann.cpp:909-946): right-hand
 * side R (npoin x 5) from host G (volume-divided, npoin x 15) and U. */
int xg_riecg_rhs(xg_ctx* ctx, const double* G, const double* U, double* R);

/* The manufactured source of riemann::rhs: R -= s(x, t) V per node, with
 * s the problem's source (enum xg_source) and prm its control-file
 * parameters problem_alpha, problem_beta[3], problem_kappa, problem_r0,
 * problem_p0, problem_ce (8 doubles; may be NULL for taylor_green).  The
 * source is evaluated at the context's time: the time given to
 * xg_riecg_set_state, advanced by xg_riecg_run; every stage of a step uses
 * the time at the start of the step, as RieCG::rhs passes it
 * (src/Inciter/RieCG.cpp:948-949).  XG_SRC_NONE switches it off. */
int xg_riecg_set_source(xg_ctx* ctx, int problem, const double* prm);

/* xg_riecg_rhs computed with the edge-coloured scatter instead of owner
 * half-edges with deposits (FP32 mode only): the edges are split into
 * classes with no shared node (greedy colouring, built on the first call),
 * and one launch per class updates both ends of each edge in place.  The
 * same residual (riemann::rhs advdom, src/Physics/Riemann.cpp:652-766, adds
 * -f and +f per edge), summed in another order.  *ncolours (may be NULL)
 * receives the number of classes. */
int xg_riecg_rhs_coloured(xg_ctx* ctx, const double* G, const double* U, double* R,
                          int* ncolours);

/* Apply the boundary conditions to the device state (RieCG::BC). */
int xg_riecg_bc(xg_ctx* ctx);

/* CFL time step of the device state (RieCG::dt, src/Inciter/RieCG.cpp:787-852). */
int xg_riecg_dt(xg_ctx* ctx, double* dt);

/* One RK stage on the device state with a given dt: grad, rhs, update
 * U = Un - rkcoef[stage]*dt*R/V, BCs (RieCG::grad/rhs/solve,
 * src/Inciter/RieCG.cpp:871-1057).  Stage 2 completes the step: the
 * context's time advances by dt. */
int xg_riecg_stage(xg_ctx* ctx, int stage, double dt);

/* Advance nstep full time steps (CFL dt, 3 stages) on the device without
 * host synchronisation.  dts (optional, host, nstep) receives each step's dt;
 * ms (optional) the device time of the run measured with CUDA events on the
 * context stream.  Returns XG_ERR_BLOWUP if a dt fell below eps. */
int xg_riecg_run(xg_ctx* ctx, int64_t nstep, double* dts, float* ms);

/* Per-kernel device time of the last xg_riecg_run with profiling enabled:
 * enable != 0 brackets every launch with CUDA events (slightly slower).
 * names/ms/launches receive up to cap entries; *n the number of kernels. */
int xg_riecg_profile(xg_ctx* ctx, int enable);
int xg_riecg_kernel_times(xg_ctx* ctx, int cap, const char** names, double* ms,
                          int64_t* launches, int* n);

/* Allocation-free CFL time step.  No counterpart in the reference: this is
 * for callers that cannot allocate device memory (their own pool already owns
 * the device's memory, or they run where cudaMalloc is not allowed) and that
 * hold RieCG's state on the device themselves.  U (npoin x 5, node-major)
 * and vol (npoin) are device pointers; dt (host) receives cfl * min over
 * nodes of cbrt(vol)/max(|u|+c, 1e-8) evaluated in FP64 arithmetic, or
 * const_dt when |const_dt| > eps.  That is xg_riecg_dt's result for an FP64
 * context; an XG_FP32_FLUX context's xg_riecg_dt evaluates the same formula
 * in FP32 arithmetic, which can differ in the low bits (about 1e-7
 * relative).  Work is issued on stream (a cudaStream_t, null for the
 * default stream) on the calling thread's current device, then synchronised.
 * The scratch is a fixed 512 KiB device array inside the library, shared by
 * all calls on a device: npoin is limited to 16,777,216 nodes (XG_ERR_ARG
 * beyond), and calls that overlap on the GPU race.  The first call on each
 * device looks the array up (device set-up); make it before any stream
 * capture. */
int xg_riecg_dt_noalloc(const double* U, const double* vol, int64_t npoin, double gamma,
                        double cfl, double const_dt, void* stream, double* dt);

/* ---- KozCG ---------------------------------------------------------------- */

/* KozCG settings (mat.spec_heat_ratio, cfl, dt, fct, fctdif, fctclip, fctsys). */
typedef struct xg_kozcg_params {
  double gamma;
  double cfl;
  double const_dt;
  int fct;       /* nonzero: flux-corrected transport (the reference default) */
  double ctau;   /* fctdif: antidiffusion coefficient */
  int fctclip;   /* nonzero: limits from the low-order solution only */
  int fctsys;    /* bit c set: component c is limited as part of the system */
  int precision; /* enum xg_precision: XG_FP32_FLUX forms the element terms
                    (Galerkin residual, antidiffusive and limited element
                    contributions) in FP32, sums them per node in FP32 and
                    updates the FP64 state in FP64 */
} xg_kozcg_params;

/* Mesh of KozCG: coordinates, nodal volumes and tetrahedra (Discretization
 * Coord()/Vol()/Inpoel()), FP64. */
int xg_kozcg_setup(xg_ctx* ctx, const xg_kozcg_params* prm, int64_t npoin, const double* coord,
                   const double* vol, int64_t nelem, const uint64_t* inpoel);

/* Symmetry (m_symbcnodes / m_symbcnorms) and Dirichlet (nodes, 5 mask ints,
 * 5 values per node) BCs applied by KozCG::BC (src/Inciter/KozCG.cpp:590-611):
 * masks as for xg_riecg_set_bc, the BC's time the end of the step
 * (KozCG.cpp:1167; the context's time in xg_kozcg_bc). */
int xg_kozcg_set_bc(xg_ctx* ctx, int64_t nsym, const uint64_t* symnodes, const double* symnorms,
                    int64_t ndir, const uint64_t* dirnodes, const int32_t* dirmask,
                    const double* dirvals);

int xg_kozcg_set_state(xg_ctx* ctx, const double* U, double t);
int xg_kozcg_get_state(xg_ctx* ctx, double* U, double* t);

/* Drop-in for kozak::rhs (src/Physics/Kozak.cpp:29-180): two-step
 * Taylor-Galerkin residual R (npoin x 5) of host U with time step dt. */
int xg_kozcg_rhs(xg_ctx* ctx, const double* U, double dt, double* R);

/* Apply the BCs to the device state (KozCG::BC). */
int xg_kozcg_bc(xg_ctx* ctx);

/* CFL time step of the device state (KozCG::dt, src/Inciter/KozCG.cpp:613-688). */
int xg_kozcg_dt(xg_ctx* ctx, double* dt);

/* Advance nstep KozCG steps on the device (dt, rhs, FCT aec/alw/lim/solve,
 * BCs; src/Inciter/KozCG.cpp:613-1197); dts and ms as in xg_riecg_run. */
int xg_kozcg_run(xg_ctx* ctx, int64_t nstep, double* dts, float* ms);

/* One KozCG step of the caller's dt (> 0) from the context's time, which
 * then advances by dt: the step Discretization::setdt cuts to end at the
 * final time (src/Inciter/Discretization.cpp:926-939). */
int xg_kozcg_step(xg_ctx* ctx, double dt);

/* The manufactured source of kozak::rhs (src/Physics/Kozak.cpp:125-132,
 * 161-170): dt/8 of each node's source at the step's start time in the
 * element's half step, and J/24 of the source at its centroid half a step
 * later in each node's residual; problem and prm as for
 * xg_riecg_set_source.  The time is the context's: set by
 * xg_kozcg_set_state, advanced by xg_kozcg_run and xg_kozcg_step;
 * xg_kozcg_rhs evaluates the sources at it.  XG_SRC_NONE switches it off. */
int xg_kozcg_set_source(xg_ctx* ctx, int problem, const double* prm);

/* ---- ChoCG ---------------------------------------------------------------- */

enum xg_chorin_flux { XG_DAMP2 = 0, XG_DAMP4 = 1 };

/* ChoCG settings the reference reads from its global config
 * (mat_dyn_viscosity, cfl, dt, flux, stab, stab2, stab2coef, rk and the
 * pressure{iter, tol, pc} block), plus the pressure-solve variants of this
 * library: ppc 2 is the factored preconditioner of xg_cg_set_factor, pmixed
 * the mixed-precision solve of xg_cg_solve_mixed. */
typedef struct xg_chocg_params {
  double mu;          /* dynamic viscosity */
  double cfl;         /* CFL number (used when const_dt == 0) */
  double const_dt;    /* constant time step if |const_dt| > eps */
  int flux;           /* enum xg_chorin_flux (the reference needs damp2 or damp4) */
  int stab;           /* nonzero: advective stabilisation |vnL + vnR|/2 */
  int stab2;          /* nonzero: artificial viscosity stab2coef*max(|vnL|,|vnR|) */
  double stab2coef;
  int rk;             /* explicit Runge-Kutta stages, 1..4 */
  int ppc;            /* pressure preconditioner: 0 none, 1 jacobi, 2 factor */
  double ptol;        /* pressure solve: relative residual tolerance */
  int64_t pmaxit;     /* pressure solve: iteration limit */
  int pmixed;         /* nonzero: mixed-precision refinement (xg_cg_solve_mixed) */
  double pinner_tol;  /* its inner residual reduction per replacement */
  int pguard;         /* FP64 breakdown guard, as xg_cg_set_guard (0: the reference's) */
} xg_chocg_params;

/* Upload the operators ChoCG builds once per mesh (ChoCG::feop/streamable/
 * domsuped, src/Inciter/ChoCG.cpp:277-813): coordinates, nodal volumes, the
 * three superedge groups as ChoCG::m_dsupedge/m_dsupint with five integrals
 * per edge (tets: 4 ids + 6x5; triangles: 3 ids + 3x5; edges: 2 ids + 5) and
 * the boundary triangles m_triinpoel.  The pressure matrix of ChoCG::prelhs
 * goes to xg_cg_setup on the same context (as the reference inserts it into
 * its ConjugateGradients array); xg_chocg_init and xg_chocg_run solve on it. */
int xg_chocg_setup(xg_ctx* ctx, const xg_chocg_params* prm, int64_t npoin, const double* coord,
                   const double* vol, int64_t ntet, const uint64_t* dsupedge0,
                   const double* dsupint0, int64_t ntri, const uint64_t* dsupedge1,
                   const double* dsupint1, int64_t nedge, const uint64_t* dsupedge2,
                   const double* dsupint2, int64_t nbtri, const uint64_t* triinpoel);

/* The theta-implicit momentum prediction of ChoCG (theta > 0; 0 switches
 * back to the explicit one): the last Runge-Kutta stage solves
 * A du = R with A = -(M / dt + theta mu K), M the consistent mass and K the
 * stiffness matrix of the tetrahedra (ChoCG::lhs, src/Inciter/ChoCG.cpp:
 * 1433-1477), the velocity Dirichlet components and noslip nodes as zero
 * rows, warm-started from the previous increment, at most mom_iter
 * iterations to mom_tol with mom_pc (0 none, 1 jacobi), and sets
 * u = un + du (ChoCG::solve/msolve/msolved, ChoCG.cpp:1529-1645).  inpoel:
 * the tetrahedra, 4 node ids each.  The control file's theta, and the
 * momentum solver's iter, tol and pc. */
int xg_chocg_set_theta(xg_ctx* ctx, double theta, int64_t ntet, const uint64_t* inpoel,
                       int mom_pc, int64_t mom_iter, double mom_tol);
/* Iterations of the last momentum solve (negative: stopped short of mom_tol). */
int xg_chocg_momentum_its(xg_ctx* ctx, int64_t* it);

/* Boundary conditions as ChoCG::setupDirBC/streamable store them and
 * ChoCG::BC applies them (src/Inciter/ChoCG.cpp:207-275, 1333-1354):
 *   velocity Dirichlet: nodes, 3 mask ints per node (nonzero: set) and 3
 *     values per node (time independent);
 *   symmetry: m_symbcnodes / m_symbcnorms (a node may repeat);
 *   noslip: m_noslipbcnodes;
 *   pressure Dirichlet (pressure.bc_dir and the hydrostat node): nodes and
 *     the values of the initial solves; the time-increment solves use 0
 *     (ChoCG::pinit, src/Inciter/ChoCG.cpp:1025-1125). */
int xg_chocg_set_bc(xg_ctx* ctx, int64_t ndir, const uint64_t* dirnodes, const int32_t* dirmask,
                    const double* dirvals, int64_t nsym, const uint64_t* symnodes,
                    const double* symnorms, int64_t nnoslip, const uint64_t* noslipnodes,
                    int64_t npdir, const uint64_t* pdirnodes, const double* pdirvals);

/* Device state: velocity u (npoin x 3, node-major), pressure p (npoin; null
 * keeps zero on set), time t. */
int xg_chocg_set_state(xg_ctx* ctx, const double* u, const double* p, double t);
int xg_chocg_get_state(xg_ctx* ctx, double* u, double* p, double* t);

/* ChoCG's start-up sequence on the device state (ChoCG::merge -> div ->
 * pinit -> psolve -> sgrad -> psolved, twice, then pgrad;
 * src/Inciter/ChoCG.cpp:739-764, 868-1281): BCs, projection of the initial
 * velocity onto divergence-free fields, the initial pressure from the
 * momentum-flux divergence and its gradient.  *it receives the iterations of
 * the last pressure solve (negated when that solve stopped short of its
 * tolerance; the reference carries on in that case, and so does this). */
int xg_chocg_init(xg_ctx* ctx, int64_t* it);

/* Advance nstep time steps (ChoCG::dt/advance/rhs/solve/pred/corr/div/pinit/
 * psolve/sgrad/psolved/pgrad, src/Inciter/ChoCG.cpp:1356-1695, 868-1281) on
 * the device: explicit RK momentum prediction, pressure-increment Poisson
 * solve, projection.  dts and its (optional, host, nstep) receive each step's
 * dt and pressure-solve iterations (negated for a solve that stopped short
 * of its tolerance at the iteration limit or the (p,q) breakdown guard, after
 * which the step completes as in the reference), ms (optional) the device
 * time.  Returns XG_ERR_BLOWUP if dt fell below eps. */
int xg_chocg_run(xg_ctx* ctx, int64_t nstep, double* dts, int64_t* its, float* ms);

/* Diagnostics fields of the device state (NodeDiagnostics::precompute,
 * src/Inciter/NodeDiagnostics.cpp:148-246): what 0 = u at the start of the
 * last step (npoin x 3), 1 = pressure gradient (npoin x 3), 2 = velocity
 * gradient (npoin x 9), 3 = last Poisson right-hand side (npoin), 4 = last
 * pressure increment (npoin). */
int xg_chocg_fields(xg_ctx* ctx, int what, double* out);

/* Drop-ins for the chorin:: passes (src/Physics/Chorin.hpp:19-70) on host
 * arrays with the operators of xg_chocg_setup; outputs are the raw weak
 * sums (not divided by the nodal volume), like the reference functions:
 *   div: D (npoin) of U (npoin x 3) with pressure P and its gradient G
 *        (npoin x 3), stabilised when stab (Chorin.cpp:85-209);
 *   grad: G (npoin x 3) of the scalar S (Chorin.cpp:336-449);
 *   vgrad: G (npoin x 9) of U (npoin x 3) (Chorin.cpp:211-334);
 *   flux: F (npoin x 3) of U with velocity gradients G (npoin x 9)
 *         (Chorin.cpp:509-638);
 *   rhs: R (npoin x 3) of P, U and G (npoin x 9) (Chorin.cpp:1010-1044). */
int xg_chorin_div(xg_ctx* ctx, const double* U, const double* P, const double* G, double dt,
                  int stab, double* D);
int xg_chorin_grad(xg_ctx* ctx, const double* S, double* G);
int xg_chorin_vgrad(xg_ctx* ctx, const double* U, double* G);
int xg_chorin_flux(xg_ctx* ctx, const double* U, const double* G, double* F);
int xg_chorin_rhs(xg_ctx* ctx, const double* P, const double* U, const double* G, double* R);

/* ---- ConjugateGradients ---------------------------------------------------- */

/* Upload a scalar sparse matrix in the layout of tk::CSR with one degree of
 * freedom per node (src/LinearSolver/CSR.hpp:98-103): row pointers ia[nrow+1],
 * column ids ja[nnz], values a[nnz], rows sorted by column, every row holding
 * its diagonal.  base is 1 for the reference's one-based ia/ja, 0 for
 * zero-based arrays.  The matrix is kept unmodified on the device; Dirichlet
 * elimination works on a copy at every xg_cg_init(apply != 0). */
int xg_cg_setup(xg_ctx* ctx, int64_t nrow, const uint64_t* ia, const uint64_t* ja,
                const double* a, int base);

/* Drop-in for tk::CSR::mult (src/LinearSolver/CSR.cpp:154-172): y = A x. */
int xg_cg_mult(xg_ctx* ctx, const double* x, double* y);

/* ConjugateGradients::init (src/LinearSolver/ConjugateGradients.cpp:335-427):
 * x (nrow, optional: null keeps the previous solution as the initial guess),
 * b (nrow, optional: null keeps the previous rhs), neubc (optional Neumann
 * contributions added to b), Dirichlet nodes and values applied symmetrically
 * when apply != 0 (as ConjugateGradients::apply/r), pc 0 = "none",
 * 1 = "jacobi".  Computes the initial residual, ||b|| and (r,z) (setup/initres). */
int xg_cg_init(xg_ctx* ctx, const double* x, const double* b, const double* neubc,
               int64_t ndir, const uint64_t* dirnodes, const double* dirvals, int apply,
               int pc);

/* ConjugateGradients::solve (ConjugateGradients.cpp:558-823): PCG until
 * ||r|| < tol * ||b|| (||b|| floored at 1e-14 -> 1), maxit iterations or a
 * (p,q) = 0 breakdown, at least one iteration.  Reports the iteration count,
 * the final ||r||, ||b|| and whether it converged (ConjugateGradients::it(),
 * converged()).  The solution stays on the device (xg_cg_solution). */
int xg_cg_solve(xg_ctx* ctx, int64_t maxit, double tol, int64_t* it, double* normr,
                double* normb, int* converged);

/* Mixed-precision variant of xg_cg_solve: iterative refinement with the FP64
 * residual r = b - A x and FP32 inner PCG solves of A e = r (FP32 matrix and
 * vectors, FP64 dot products) to inner_tol * ||r||, x += e, until
 * ||r|| < tol * ||b|| or maxit refinements.  Reports refinement steps, total
 * inner iterations, final FP64 ||r|| and ||b||. */
int xg_cg_solve_mixed(xg_ctx* ctx, int64_t maxit, double tol, double inner_tol,
                      int64_t inner_maxit, int64_t* outer, int64_t* inner, double* normr,
                      double* normb, int* converged);

/* Factored approximate-inverse preconditioner (pc = 2 in xg_cg_init; no
 * counterpart in the reference, whose preconditioners are "none" and
 * "jacobi"): M^-1 = -S (I+N)(I+N)^T S on the non-Dirichlet rows, identity on
 * Dirichlet rows, S = diag(1/sqrt|a_ii|), N strictly lower on A's sparsity.
 * With model == null, N = scale * e with e_ij = a_ij s_i s_j (scale 0 is
 * Jacobi); otherwise the model's network emits N.  The factor is built at
 * xg_cg_init(pc = 2) after the Dirichlet elimination and kept while later
 * inits use the same Dirichlet node set and no xg_cg_set_factor intervenes
 * (call it again after changing the model's parameters). */
int xg_cg_set_factor(xg_ctx* ctx, xg_lpc* model, double scale);

/* Breakdown guard of the FP64 solver (no counterpart in the reference):
 * guard 0 (the default) ends a solve when |(p,q)| < DBL_EPSILON, the
 * reference's absolute test (ConjugateGradients.cpp:681-690), which stops
 * well-posed solves early when the right-hand side is small (a pressure
 * increment on a fine mesh); guard 1 stops only on underflow (|(p,q)| <
 * DBL_MIN), as the mixed-precision solver does, so the relative tolerance is
 * what ends the solve.  Applies from the next xg_cg_init. */
int xg_cg_set_guard(xg_ctx* ctx, int guard);

/* z = M^-1 r with the preconditioner of the last xg_cg_init (host vectors). */
int xg_cg_precondition(xg_ctx* ctx, const double* r, double* z);

/* ConjugateGradients::solution(): copy the device solution to x (nrow). */
int xg_cg_solution(xg_ctx* ctx, double* x);

/* ---- learned preconditioner (no counterpart in the reference) ----------
 * A message-passing network on the matrix graph (3 layers, hidden width 64)
 * that emits the factor N of xg_cg_set_factor.  The model lives on the
 * device of the context it is created with; precision 0 runs its dense
 * layers in FP32, 1 as BF16 tensor-core GEMMs with FP32 accumulation.
 * Parameters are one flat FP32 vector of xg_lpc_nparams() values in the
 * order W0 (4x64) b0 W1 (128x64) b1 W2 b2 W3 b3 Wo (64x128) c c2 d w ob. */
int64_t xg_lpc_nparams(void);
int xg_lpc_create(xg_ctx* ctx, int precision, xg_lpc** model);
int xg_lpc_destroy(xg_lpc* model);
int xg_lpc_set_params(xg_lpc* model, const float* theta); /* also resets Adam */
int xg_lpc_get_params(xg_lpc* model, float* theta);
int xg_lpc_zero_grads(xg_lpc* model);
int xg_lpc_get_grads(xg_lpc* model, float* grad);
/* Adds d loss / d theta for the matrix of the CG system of `system`
 * (after xg_cg_init, Dirichlet rows eliminated) to the model's gradient.
 * loss = (tr(L^T A^ L) - n) / n with A^ = -S A S and L = I + N: Kaporin's
 * trace functional of the factorised approximate inverse (no solve needed).
 * Calls on one model must not overlap. */
int xg_lpc_grad(xg_lpc* model, xg_ctx* system, double* loss);
const char* xg_lpc_last_error(xg_lpc* model);
/* One Adam step on the accumulated gradient. */
int xg_lpc_adam(xg_lpc* model, double lr, double beta1, double beta2, double eps);

/* ---- host operator setup (the caller side of xg_riecg_setup) ------------- */

/* Locality renumbering of mesh nodes (reverse Cuthill-McKee over points
 * surrounding points; plays the role of the constructor reordering in
 * RieCG::RieCG, src/Inciter/RieCG.cpp:82-100).  new_of_old[npoin]. */
int xg_mesh_rcm(int64_t npoin, int64_t nelem, const uint64_t* inpoel, uint64_t* new_of_old);

/* Nodal volumes (Discretization::vol, src/Inciter/Discretization.cpp:619-660).
 * Fails with XG_ERR_ARG on a non-positive element Jacobian. */
int xg_mesh_vol(int64_t npoin, const double* coord, int64_t nelem, const uint64_t* inpoel,
                double* vol);

/* Domain edge integrals (RieCG::domint, src/Inciter/RieCG.cpp:339-382; with
 * ncoef == 5 also ChoCG's two extra coefficients, src/Inciter/ChoCG.cpp:
 * 398-445).  Each edge is oriented from the smaller to the larger gid (gid may
 * be null: identity) and reported with local ids.  Call with cap = 0 to get
 * *nedge, then again with arrays of that size (edges 2 per edge, dint ncoef
 * per edge), sorted by (gid, gid). */
int xg_mesh_edges(int64_t npoin, const double* coord, int64_t nelem, const uint64_t* inpoel,
                  const uint64_t* gid, int ncoef, int64_t cap, int64_t* nedge,
                  uint64_t* edges, double* dint);

/* Inverse-distance weighted boundary point normals of one side set
 * (RieCG::bndint + bnorm, src/Inciter/RieCG.cpp:281-337, 483-525) for the
 * given nodes, which must lie on faces of the set. */
int xg_mesh_bnorm(int64_t npoin, const double* coord, int64_t nface, const uint64_t* faces,
                  int64_t nnode, const uint64_t* nodes, double* norms);

/* Pressure-Poisson matrix of ChoCG::prelhs (src/Inciter/ChoCG.cpp:146-188):
 * A(a,b) -= grad_a.grad_b / (6J) over tets, on the points-surrounding-points
 * sparsity plus the diagonal, zero-based, rows sorted by column.  Call with
 * cap = 0 to get *nnz, then with ia[npoin+1], ja[nnz], a[nnz]. */
int xg_mesh_pressure_matrix(int64_t npoin, const double* coord, int64_t nelem,
                            const uint64_t* inpoel, int64_t cap, int64_t* nnz, uint64_t* ia,
                            uint64_t* ja, double* a);

#ifdef __cplusplus
}
#endif

#endif /* XG_H */
