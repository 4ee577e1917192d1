/*
 * atm_gb300.h -- C ABI of the GB300 IMEX-DG dynamical-core hot path.
 *
 * The entry points replace the matrix-free operator and the stage solvers of
 * GiuseppeOrlando878776/Atmospheric_Flows (a deal.II code).  Each block below
 * names the reference interface it stands in for (file:line in that project).
 * All arithmetic is FP64 unless an entry point says otherwise.
 *
 * Conventions
 *   - Every call returns an int status (ATM_OK = 0); no C++ exception crosses
 *     the ABI.  atm_last_error() gives a message for the last failure.
 *   - dim = 2, degree k in 1..5, quadrature QGauss(2k+1) for every integral.
 *   - Field vectors are cell-contiguous: scalar fields [cell][node], velocity
 *     [cell][component][node], node = iz*(k+1)+ix on Gauss-Lobatto points
 *     (the layout of FE_DGQ / FESystem(FE_DGQ,dim) blocks).
 *   - Operator entry points (atm_vmult*, atm_set_*_fixed, atm_solve*) take
 *     DEVICE pointers and run asynchronously on the context's stream; the
 *     destination is overwritten (deal.II loop(..., zero_dst=true)).
 *   - The solver-level entry points (atm_solver_*) take HOST pointers.
 *   - A handle is not thread-safe; several handles may be used from one
 *     host thread.
 */
#ifndef ATM_GB300_H
#define ATM_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

enum atm_status {
  ATM_OK = 0,
  ATM_BAD_ARG = 1,
  ATM_NOT_CONVERGED = 2,
  ATM_NONFINITE = 3,
  ATM_OOM = 4,
  ATM_TIMEOUT = 5,
  ATM_CUDA_ERROR = 6,
  ATM_NOT_READY = 7
};

typedef struct atm_ctx *atm_handle;

/* Message of the last failing call on this thread (never NULL). */
const char *atm_last_error(void);
/* Library version string. */
const char *atm_version(void);

/* ---------------------------------------------------------------------------
 * Context = EULEROperator + its MatrixFree storage.
 * Replaces: MatrixFree::reinit / EULEROperator::initialize
 *   (Atmospheric_Flow.cc:325-348,435), the mesh/dof set-up
 *   (Atmospheric_Flow.cc:279-409) re-uploaded as plain tables.
 *   mapping_nodes : [n_cells][(m+1)^2][2] host, Gauss-Lobatto points of a
 *                   degree-m tensor Lagrange mapping (MappingQ(m)), x fastest
 *   inner_faces   : [n_inner][5] host: cell+, face+, cell-, face-, o
 *                   (local faces 0:x=0 1:x=1 2:z=0 3:z=1; face+ and face- opposite).
 *                   o = 0: conforming face.  o = 1, 2: hanging face of a 2:1
 *                   adaptive mesh -- cell+ is the fine cell and its face is
 *                   subface o-1 (the half at the lower face parameter for o = 1)
 *                   of face- of the coarse cell cell-; both subfaces must be
 *                   listed.  As deal.II, the fine side is the interior side.
 *                   Replaces the hanging-face handling of MatrixFree on
 *                   p4est meshes (Atmospheric_Flow.cc:279-283).
 *   bdry_faces    : [n_bdry][3] host: cell, face, boundary id (all walls)
 * ------------------------------------------------------------------------- */
int atm_ctx_create(int dim, int degree, int n_cells, int mapping_degree,
                   const double *mapping_nodes, int n_inner, const int *inner_faces,
                   int n_bdry, const int *bdry_faces, atm_handle *out);
int atm_ctx_destroy(atm_handle h);
/* Validate mesh tables on the host without a device (the checks
 * atm_ctx_create makes): index ranges, opposite face pairs, every cell face
 * listed once (a coarse hanging face twice, by its two subfaces), positive
 * Jacobians.  On success *n_hanging (if given) is the number of hanging faces.
 * Error messages as atm_ctx_create.  No reference counterpart (deal.II
 * asserts on its own triangulation). */
int atm_check_mesh(int degree, int n_cells, int mapping_degree, const double *mapping_nodes,
                   int n_inner, const int *inner_faces, int n_bdry, const int *bdry_faces,
                   int *n_hanging);
/* Re-upload geometry and connectivity after mesh adaptation (same sizes).
 * Drops the multigrid levels: add them again for the new mesh.  Replaces the
 * MatrixFree::reinit that follows a refinement (Atmospheric_Flow.cc:283,
 * 325-348). */
int atm_upload_mesh(atm_handle h, int mapping_degree, const double *mapping_nodes,
                    int n_inner, const int *inner_faces, int n_bdry,
                    const int *bdry_faces);
/* cudaStream_t as void*; NULL = the legacy default stream.  Streams, device
 * memory queries and the FMA probe below have no reference counterpart
 * (deal.II runs on the host). */
int atm_set_stream(atm_handle h, void *stream);
int atm_synchronize(atm_handle h);
/* A non-blocking CUDA stream (as void*) for one member of an ensemble, so
 * that members driven from different host threads overlap on the device
 * (no reference counterpart: the reference runs one member per MPI job). */
int atm_stream_create(void **out);
int atm_stream_destroy(void *stream);
/* cudaMemGetInfo of the current device, for admission against a budget. */
int atm_device_memory(double *free_bytes, double *total_bytes);
/* Sizes: scalar field length n_cells*(k+1)^2; velocity twice that (the
 * DoFHandler sizes written at Atmospheric_Flow.cc:250-252). */
long atm_n_scalar(atm_handle h);

/* Instrumentation (replaces deal.II TimerOutput, Atmospheric_Flow.cc:176-178,
 * 249).  atm_kernel_launches counts every kernel launch of the library in
 * this process.  With timing enabled, each operator launch is bracketed by
 * CUDA events on the context's stream; atm_timing_read synchronises and
 * returns, per family 0..11 = rhs_rho, rhs_vel, rhs_pres, B, C/D, mass,
 * diagonal, block inverse, block apply, multigrid level Schur apply (B+C/D
 * pair, any level), whole V-cycle (nested: contains the level applies),
 * p_fix preparation for C/D (values at quadrature points, face traces):
 * total ms, launches, algorithmic HBM
 * bytes (fields read + written, 8 B per node value) and FP64 flops of the
 * sum-factorisation contractions; then resets them.  Any output may be NULL. */
long atm_kernel_launches(void);
/* FP64 and FP32 FMA throughput of the current device in GFLOP/s (independent
 * FMA chains, 8 blocks per SM); the compute-roofline denominators. */
int atm_probe_fma_peak(double *fp64_gflops, double *fp32_gflops);
int atm_timing_enable(atm_handle h, int on);
int atm_timing_read(atm_handle h, double *ms, long *launches, double *bytes, double *flops,
                    int n);

/* ---------------------------------------------------------------------------
 * Setters.  Replace EULEROperator::set_dt / set_Mach / set_Froude /
 * set_HYPERBOLIC_stage / set_NS_stage (euler_operator.h:34-43,245-303).
 * ------------------------------------------------------------------------- */
int atm_set_dt(atm_handle h, double dt);
int atm_set_mach(atm_handle h, double mach);
int atm_set_froude(atm_handle h, double froude);
int atm_set_hyperbolic_stage(atm_handle h, int stage); /* 1..3 */
int atm_set_ns_stage(atm_handle h, int stage);         /* 1..6 */

/* Frozen fields (device pointers, copied).  Replace set_rho_for_fixed /
 * set_pres_fixed / set_u_fixed (euler_operator.h:45-52,306-339).
 * set_rho_for_fixed also rebuilds the exact cell-wise inverse of
 * A = (rho_fix-weighted velocity mass) used by the Schur apply and solves. */
int atm_set_rho_for_fixed(atm_handle h, const double *rho);
int atm_set_pres_fixed(atm_handle h, const double *pres);
int atm_set_u_fixed(atm_handle h, const double *u);

/* ---------------------------------------------------------------------------
 * Explicit stage right-hand sides (device pointers).  Replace
 *   vmult_rhs_rho_update      euler_operator.h:54-55,697-712
 *   vmult_rhs_velocity_fixed  euler_operator.h:60-61,2310-2325
 *   vmult_rhs_pressure        euler_operator.h:57-58,1366-1381
 * src is the positional source list of the reference call sites
 * (Atmospheric_Flow.cc:439-449,555-568,696-698,796-799); nsrc must be
 *   rho: 2 / 4 / 6, velocity: 4 / 7 / 9, pressure: 5 / 8 / 11
 * for IMEX stage 1 / 2 / 3.
 * ------------------------------------------------------------------------- */
int atm_vmult_rhs_rho_update(atm_handle h, double *dst, const double *const *src, int nsrc);
int atm_vmult_rhs_velocity_fixed(atm_handle h, double *dst, const double *const *src,
                                 int nsrc);
int atm_vmult_rhs_pressure(atm_handle h, double *dst, const double *const *src, int nsrc);

/* B: pressure -> velocity space.  Replaces vmult_pressure
 * (euler_operator.h:63,1512-1617,2422-2435). */
int atm_vmult_pressure(atm_handle h, double *dst, const double *src);
/* C: velocity -> pressure space, with pres_fixed.  Replaces vmult_enthalpy
 * (euler_operator.h:65,1413-1507,2440-2453). */
int atm_vmult_enthalpy(atm_handle h, double *dst, const double *src);
/* Base::vmult -> apply_add for the current NS stage
 * (euler_operator.h:93,2366-2417): NS 1/4 rho mass, NS 2 Schur
 * S p = D p - C A^{-1} B p (A^{-1} exact per cell), NS 3/5 A, NS 6 D. */
int atm_vmult(atm_handle h, double *dst, const double *src);
/* compute_diagonal + get_matrix_diagonal_inverse (euler_operator.h:67,
 * 2458-2626): writes the inverse diagonal for the current NS stage
 * (NS 2 uses the diagonal of D only, as the reference does). */
int atm_diagonal_inverse(atm_handle h, double *dst);

/* Schur apply S p = D p - C A^{-1} B p (same result as atm_vmult in NS
 * stage 2) that allocates nothing: the intermediate A^{-1} B p is kept in a
 * static 8 MiB device array owned by the library.  For callers that must not
 * have the library allocate device memory at call time (a host that owns all
 * HBM through its own pool or budget; loops that cannot afford the device-wide
 * synchronisation of cudaMalloc/cudaFree).  No counterpart in the reference.
 * Limits: 2*n_scalar <= 1048576 doubles, else ATM_BAD_ARG; all calls on a
 * device share the array, so calls that overlap on the GPU race; the first
 * call with a handle looks the array's address up in the handle's CUDA
 * context (kept in the handle, so it stays right across contexts and device
 * resets) and should come before any stream capture; kernel timing must be
 * off.  Device pointers, context's stream. */
int atm_schur_vmult_static_scratch(atm_handle h, double *dst, const double *src);

/* Solve op x = b for the current NS stage.  Replaces the stage solvers'
 * SolverCG+PreconditionMG (mass systems, solved here exactly with the
 * cell-wise inverse) and SolverGMRES+PreconditionJacobi (NS 2)
 * (Atmospheric_Flow.cc:452-536,642,656-672,701-780,801-870).  x holds the
 * initial guess.  tol is absolute on the (Jacobi-preconditioned) residual;
 * iters/res may be NULL.  Returns ATM_NOT_CONVERGED on maxit. */
int atm_solve(atm_handle h, double *x, const double *b, double tol, int maxit,
              int *iters, double *res);

/* ---------------------------------------------------------------------------
 * Mixed-precision Schur solve: FP64 flexible GMRES right-preconditioned by an
 * FP32 geometric-multigrid V-cycle with Chebyshev smoothing (the reference's
 * smoother recipe, Atmospheric_Flow.cc:489-502, applied to the Schur system,
 * which the reference solves with GMRES + Jacobi, Atmospheric_Flow.cc:656-672).
 * Levels are added fine to coarse.  Level 0 is the context's mesh.  Each call
 * adds the next coarser mesh, whose cells are unions of 2x2 cells of the
 * previous level: children[n_cells][4] lists, for each coarse cell, the
 * previous-level cells at positions (x-,z-), (x+,z-), (x-,z+), (x+,z+).
 * Mesh tables as in atm_ctx_create. */
int atm_mg_add_level(atm_handle h, int n_cells, int mapping_degree, const double *mapping_nodes,
                     int n_inner, const int *inner_faces, int n_bdry, const int *bdry_faces,
                     const int *children);
/* Chebyshev degree (4; the reference's 3 needs more FGMRES iterations),
 * smoothing range (15), power iterations for the largest eigenvalue (10),
 * degree of the coarsest-level Chebyshev (6).  Replaces the smoother_data
 * set-up of Atmospheric_Flow.cc:477-498,594-615. */
int atm_mg_set_smoother(atm_handle h, int degree, double smoothing_range, int eig_iterations,
                        int coarse_degree);
/* One V-cycle: dst ~= S^{-1} src (FP64 device vectors); precision 1 runs the
 * V-cycle in FP32, 2 in FP64.  Replaces PreconditionMG::vmult
 * (Atmospheric_Flow.cc:518-522, 635-642), here on the Schur operator. */
int atm_mg_vcycle(atm_handle h, int precision, double *dst, const double *src);
/* Replay the V-cycle as a captured CUDA graph (1, default) or launch its
 * kernels one by one (0).  Same kernels, same arguments, same results; the
 * graph is re-captured when the stage coefficient, dt, Ma or the smoother's
 * eigenvalue estimates change.  No reference counterpart (deal.II's
 * PreconditionMG::vmult, Atmospheric_Flow.cc:517-536, runs on the host). */
int atm_mg_set_graphs(atm_handle h, int on);
/* out[0] = V-cycles run, out[1] = of those, replays of a captured graph.
 * No reference counterpart. */
int atm_mg_stats(atm_handle h, long *out);

/* Tile-shape autotuner of the face kernels (the explicit right-hand sides, B
 * and C/D, on every level): cells per block among 64/(2k+1), 128/(2k+1) and
 * 256/(2k+1), timed on the first launch of each (kernel, degree, mode, mesh
 * size class) on meshes of 2048 cells or more.  On by default; results do not
 * depend on it.  No reference counterpart (deal.II's MatrixFree fixes its
 * cell batch size at compile time, Atmospheric_Flow.cc:337-344). */
int atm_set_autotune(atm_handle h, int on);
/* The choices made so far in this process: up to max_entries rows of 8 ints
 * (device, family 0 rhs_rho / 1 rhs_vel / 2 rhs_pres / 3 B / 4 C/D, degree,
 * mode or stage, hanging faces, bytes per value, log2 of the cell count,
 * cells per block).  Returns the number of entries (may exceed max_entries). */
int atm_autotune_table(int *out, int max_entries);
/* FGMRES(16) + V-cycle on S x = b (NS 2 operator state); tol absolute on the
 * unpreconditioned residual; precision as for atm_mg_vcycle.  Replaces the
 * Schur GMRES of Atmospheric_Flow.cc:657-672 with a multigrid-preconditioned
 * flexible GMRES. */
int atm_solve_fgmres(atm_handle h, int precision, double *x, const double *b, double tol,
                     int maxit, int *iters, double *res);
/* S is not linear (the upwind lambda of C depends on A^{-1}B p,
 * euler_operator.h:1497-1498), so a Krylov solve that stops on its
 * linearised residual estimate returns an answer that depends on the Krylov
 * algorithm.  With this option on, GMRES and FGMRES only stop on the
 * recomputed true residual b - S(x).  Off (default) = deal.II SolverGMRES. */
int atm_set_true_residual_check(atm_handle h, int on);

/* ---------------------------------------------------------------------------
 * Time loop.  Replaces EulerSolver (Atmospheric_Flow.cc:57-272,1100-1257):
 * the 3-stage IMEX step with the Picard loop (<= 100 iterations, 1e-10
 * relative L-infinity stop), stage combination and an optional Rayleigh
 * sponge on u (applied after stage 3).  The solver state lives in the
 * context (one solver per context); set/get use HOST pointers unless the
 * name ends in _device.
 *   precision: 0 = FP64 GMRES + Jacobi on diag(D) (the reference solver),
 *              1 = FP64 flexible GMRES + FP32 multigrid V-cycle,
 *              2 = FP64 flexible GMRES + FP64 multigrid V-cycle.
 * ------------------------------------------------------------------------- */
int atm_solver_init(atm_handle h, double dt, double mach, double froude, double eps,
                    int max_its, int precision);
int atm_solver_set_state(atm_handle h, const double *rho, const double *u,
                         const double *p);
int atm_solver_get_state(atm_handle h, double *rho, double *u, double *p);
/* device-pointer variants (length n_scalar / 2*n_scalar / n_scalar) */
int atm_solver_set_state_device(atm_handle h, const double *rho, const double *u,
                                const double *p);
int atm_solver_get_state_device(atm_handle h, double *rho, double *u, double *p);
/* Rayleigh sponge: after each step relax u toward (ubg_x, ubg_z) with rate
 * alpha_nodes (1/s per node; NULL switches it off).  Not in the reference: it
 * is the flow-over-hill absorbing layer, applied where the reference's step
 * ends (Atmospheric_Flow.cc:1220-1222). */
int atm_solver_set_sponge(atm_handle h, const double *alpha_nodes, double ubg_x,
                          double ubg_z);
/* Per-node target velocity of the sponge ([cell][2][node], host, 2*n_scalar
 * values) instead of the constant (ubg_x, ubg_z); NULL returns to the
 * constant.  Lets one context hold several flow-over-hill members with
 * different background winds (batched serving).  No reference counterpart. */
int atm_solver_set_sponge_target(atm_handle h, const double *u_target);
/* Restore the simulated time and step count (checkpoint restart).  No
 * reference counterpart (the reference writes VTU output only,
 * Atmospheric_Flow.cc:885-918). */
int atm_solver_set_clock(atm_handle h, double time, long steps);
/* Advance n_steps IMEX steps.  A Schur solve that reaches max_its ends the
 * call with ATM_NOT_CONVERGED, as the reference's SolverControl throws and
 * main returns 1 (Atmospheric_Flow.cc:1289-1311); a non-finite residual or
 * Picard update ends it with ATM_NONFINITE.  The failed step is abandoned:
 * the state, time and step count stay those of the last completed step (the
 * state is written only in the final stage, which has no Krylov solve). */
int atm_solver_run(atm_handle h, int n_steps);
/* on = 1: a Schur solve that reaches max_its is counted (stats[5]) and the
 * step carries on with the unconverged iterate; on = 0 (default): it fails
 * as atm_solver_run says.  No reference counterpart (deal.II always throws). */
int atm_solver_set_continue_on_not_converged(atm_handle h, int on);
/* ---------------------------------------------------------------------------
 * Several independent members in one context (ensemble serving).  No
 * reference counterpart: the reference runs one member per process
 * (Atmospheric_Flow.cc:1265-1313).  The context's cells are n_members
 * contiguous ranges cell_offsets[m] .. cell_offsets[m+1] (n_members + 1
 * entries, from 0 to n_cells) that share no faces, and member m advances with
 * its own time step member_dt[m] (the context's dt only sets the units).
 * Every Schur solve and Picard loop is then member-wise: inner products,
 * Krylov stops and Picard stops are each member's own, so a member's result
 * does not depend on the others in the context.  A member whose solve fails
 * (non-converged, or a non-finite state or residual) is frozen at a uniform
 * rest state and reported by atm_member_stats; the others carry on and
 * atm_solver_run returns ATM_OK.  Multigrid levels must keep members apart
 * (each coarse cell's children in one member).  n_members = 0 returns to a
 * single member.  Call after atm_solver_init. */
int atm_set_members(atm_handle h, int n_members, const int *cell_offsets,
                    const double *member_dt);
/* out[5 m + 0..4] for each member m: status (ATM_OK or its failure), Picard
 * iterations, Krylov iterations, step of its failure (-1: none), its dt. */
int atm_member_stats(atm_handle h, int n, double *out);
/* stats[0..8] as doubles: steps, Picard iterations (total), Krylov
 * iterations (total), last Picard count stage 1, stage 2, Krylov solves that
 * hit max_its, simulated time, current dt, V-cycles (total). */
int atm_solver_stats(atm_handle h, double *stats);
/* Diagnostics of Atmospheric_Flow.cc:991-1087 at the Gauss-Lobatto nodes:
 * out[0..3] = min rho, max |rho|, max sqrt(gamma p/rho), max |u|. */
int atm_solver_diagnostics(atm_handle h, double *out);

/* ---------------------------------------------------------------------------
 * The reference's own 3D case: FE_DGQ(1) hexahedra on a spherical shell with
 * radial gravity -e_r a^2/r^2 / Fr^2 (EulerSolver<3>, Atmospheric_Flow.cc:
 * 279-286, 1277; euler_operator.h:790-811 for the gravity terms).  Same
 * operators, stages and time loop as the 2D entry points above, dim = 3.
 *   mapping_nodes : [n_cells][27][3] host, degree-2 mapping (MappingQ(2),
 *                   equation_data.h:43) at the points {0, 1/2, 1}^3, first
 *                   reference coordinate fastest; right-handed cells
 *   inner_faces   : [n_inner][4] host: cell+, face+, cell-, face- (local faces
 *                   0/1: xi1 = 0/1, 2/3: xi2, 4/5: xi3)
 *   face_perm     : [n_inner][9] host: the 3x3 Gauss points of face+ (lower
 *                   tangential coordinate fastest) are, in order, the points
 *                   face_perm[q] of face- (rotated or flipped neighbours)
 *   bdry_faces    : [n_bdry][3] host: cell, face, id (walls)
 * Fields: scalars [cell][8], velocity [cell][3][8] on the cell vertices.
 * ------------------------------------------------------------------------- */
typedef struct atm3_ctx *atm3_handle;
int atm3_ctx_create(int n_cells, const double *mapping_nodes, int n_inner,
                    const int *inner_faces, const int *face_perm, int n_bdry,
                    const int *bdry_faces, atm3_handle *out);
int atm3_ctx_destroy(atm3_handle h);
/* set_dt / set_Mach / set_Froude, set_HYPERBOLIC_stage / set_NS_stage
 * (euler_operator.h:34-43). */
int atm3_set_params(atm3_handle h, double dt, double mach, double froude);
int atm3_set_stage(atm3_handle h, int hyperbolic_stage, int ns_stage);
/* set_rho_for_fixed / set_pres_fixed / set_u_fixed (euler_operator.h:45-52),
 * device pointers, NULL leaves a field unchanged; rho rebuilds A^{-1}. */
int atm3_set_frozen(atm3_handle h, const double *rho, const double *pres, const double *u);
/* which 0/1/2: vmult_rhs_rho_update / vmult_rhs_velocity_fixed /
 * vmult_rhs_pressure (euler_operator.h:54-61), positional sources as the 2D
 * entry points; device pointers, dst overwritten. */
int atm3_rhs(atm3_handle h, int which, double *dst, const double *const *src, int nsrc);
/* which 0: vmult_pressure (B), 1: vmult_enthalpy (C), 2: Base::vmult of the
 * current NS stage (euler_operator.h:63-65, 93, 2366-2417). */
int atm3_apply(atm3_handle h, int which, double *dst, const double *src);
/* EulerSolver (Atmospheric_Flow.cc:430-871, 1100-1257) with GMRES + Jacobi for
 * the Schur system.  scaled_tol = 0 stops as the reference, eps |rhs| on the
 * Jacobi-scaled residual; on the shell diag(D)^{-1} ~ 1/|cell| is tiny and
 * that rule stops before the first iteration, so scaled_tol = 1 compares with
 * eps |diag(D)^{-1} rhs| instead.  State with HOST pointers. */
int atm3_solver_init(atm3_handle h, double eps, int max_its, int scaled_tol,
                     int true_residual_check);
int atm3_solver_set_state(atm3_handle h, const double *rho, const double *u, const double *p);
int atm3_solver_get_state(atm3_handle h, double *rho, double *u, double *p);
int atm3_solver_run(atm3_handle h, int n_steps);
/* out[0..3]: steps, Picard iterations, Krylov iterations, solves that hit max_its. */
int atm3_solver_stats(atm3_handle h, double *out);

#ifdef __cplusplus
}
#endif
#endif /* ATM_GB300_H */
