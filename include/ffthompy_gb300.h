/*
 * ffthompy_gb300 -- C ABI of the GB300 Fourier-Galerkin homogenisation library.
 *
 * One plan = one solve grid (2D or 3D), one physics (scalar conductivity or
 * small-strain elasticity in Mandel notation), a batch of nloads macroscopic
 * load cases solved together, and one working precision.  All field pointers
 * are DEVICE pointers of the plan's element type (double for FHP_F64, float
 * for FHP_F32) with layout [load][component][n0][n1][n2] in C order, unless a
 * function says "host".  `stream` is a cudaStream_t (NULL = legacy default
 * stream).  The solvers (fhp_cg_solve, fhp_cg_solve_many, the other solvers,
 * fhp_homogenize_host) asked for the legacy default stream run on a stream of
 * the plan instead, ordered after the caller's earlier work and before its
 * later work by events, so that their iterations replay as CUDA graphs (the
 * legacy stream cannot be captured).  Every function returns an FHP_* status
 * code; no function aborts or traps.  Plans are not re-entrant: one thread
 * and one stream per plan.
 *
 * The reference (vondrejc/FFTHomPy, pure Python/NumPy) has no C interface;
 * each entry point below names the Python call it replaces.  The ctypes
 * binding that the Python host layer uses is ffthompy_gb300/_lib.py.
 */
#ifndef FFTHOMPY_GB300_H
#define FFTHOMPY_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fhp_plan_s* fhp_plan;

enum fhp_status {
  FHP_OK = 0,
  FHP_NONCONVERGED = 1, /* maxiter reached with norm_res > tol (per load) */
  FHP_BREAKDOWN = 2,    /* <P, AP> <= 0 */
  FHP_NONFINITE = 3,    /* NaN/Inf in a reduction */
  FHP_TIMEOUT = 4,
  FHP_BAD_ARG = 5,
  FHP_OOM = 6,
  FHP_CUDA = 7
};

/* FHP_MIXED: fields and the outer residual in FP64, inner CG with FP32
   fields / FFTs and FP64 reductions (iterative refinement). */
enum fhp_precision { FHP_F64 = 0, FHP_F32 = 1, FHP_MIXED = 2 };
enum fhp_physics { FHP_SCALAR = 0, FHP_ELASTICITY = 1 };
/* coefficient storage per voxel: a*I, packed upper triangle, full dv x dv */
enum fhp_coef_kind { FHP_COEF_ISO = 1, FHP_COEF_SYM = 2, FHP_COEF_FULL = 3 };
/* Green projection: 1 = G1 (compatible fields, primal), 2 = G2 (dual) */

/* ABI version (major*100 + minor). */
int fhp_version(void);
const char* fhp_status_string(int status);
/* Message of the last failure in this process (empty string if none). */
const char* fhp_last_error(void);

/*
 * Create a plan.  n[dim]: solve grid.  n_band[dim]: grid N whose band
 * |k_i| <= (Nodd_i-1)/2 carries the Green projection (n_band = n for GaNi,
 * n_band = N with n = 2N-1 for Ga).  g_scale multiplies the projection
 * (prod(2N-1)/prod(N) for Ga, 1 for GaNi).
 * Replaces: ffthompy/projections.py:9-112 (scalar), :114-267 (elasticity),
 * Tensor.enlarge for Ga (ffthompy/tensors/objects.py:428-467) and the DFT /
 * Operator objects of ffthompy/applications.py:24-37,106-122.
 */
int fhp_plan_create(fhp_plan* out, int dim, const int* n, const int* n_band, const double* Y,
                    int physics, int nloads, double g_scale, int precision);
/*
 * A plan of ncells cells of the same grid (1..65535), solved together: every
 * pass launches once for all cells.  Device fields are [cell][load][component]
 * [grid], the coefficient of fhp_set_coefficient is [cell][c][grid], and the
 * per-load arrays of fhp_cg_solve / fhp_cg_solve_many / fhp_homogenize_host
 * and the A_H of fhp_energy_matrix hold every cell, cell-major
 * (ncells * nloads entries, ncells * nloads * nloads for A_H).  Each load of
 * each cell keeps its own CG state and stops on its own test; passes skip the
 * cells whose loads have all stopped.  The potential formulation, the other
 * solvers, fhp_energy_gradient and fhp_fourier_interp take single-cell plans.
 * Replaces: the per-cell loop over applications.scalar
 * (ffthompy/applications.py:24-82) for an ensemble of cells of one size.
 */
int fhp_plan_create_cells(fhp_plan* out, int dim, const int* n, const int* n_band,
                          const double* Y, int physics, int nloads, double g_scale,
                          int precision, int ncells);
/* Cells of a plan (1 unless created by fhp_plan_create_cells; 0 for NULL). */
int fhp_plan_cells(fhp_plan plan);
/*
 * Band-representation plan for Galerkin with exact integration (Ga): the CG
 * fields live on the solve grid n (they are trigonometric polynomials of the
 * band |k_i| <= (Nodd_i-1)/2, so nothing is lost), the coefficient is given on
 * an integration grid n_int >= 2n-1 (any such grid integrates exactly; a
 * smooth size avoids prime-length FFTs) and g_scale is the reference's Ga
 * scale prod(2n-1)/prod(n).  The operator equals the reference's FiGFA on the
 * (2n-1)-grid restricted to band-limited fields, and inner products agree by
 * Parseval.  Replaces: applications.scalar / elasticity with solve kind 'Ga'
 * (ffthompy/applications.py:28-31,111-116) including the Ga bound energy.
 */
int fhp_plan_create_band(fhp_plan* out, int dim, const int* n, const int* n_int,
                         const double* Y, int physics, int nloads, double g_scale,
                         int precision);
/*
 * Band plans: how CG stores its iterates.  spectral = 1 (default): as half
 * spectra of the solve grid, so an iteration runs the operator from the pad
 * to the integration grid to the band projection with no transform on the
 * solve grid; spectral = 0: as real fields of the solve grid, with forward
 * and inverse transforms of the solve grid in every iteration.  The same CG
 * recursion on the same operator (inner products by Parseval), so iterates
 * and stopping tests agree up to roundoff.  Other plans ignore the setting.
 * No counterpart in the reference (its CG iterates are real fields,
 * ffthompy/general/solver.py:80-139).
 */
int fhp_plan_set_band_cg(fhp_plan plan, int spectral);
/*
 * Band plans: kernel of the integration pass (inverse transform of the last
 * axis, coefficient, forward transform).  kind = 1 (default): lines held in
 * registers, one warp per line, where that kernel applies (FP32 fields, an
 * isotropic coefficient, a 512-point integration line with the band within a
 * quarter of it), with TMA row loads on an mbarrier when the band fills the
 * quarter (a 255-point solve line); kind = 2: the same register lines with
 * per-lane cp.async loads; kind = 0: the shared-memory line cores, for every
 * plan.
 * All compute the same transforms.  No counterpart in the reference (its
 * transforms are numpy.fft.rfftn / irfftn, ffthompy/tensors/fft.py:39-43).
 */
int fhp_plan_set_integration_kernel(fhp_plan plan, int kind);
/*
 * Autotuner: times candidate launch shapes of the plan's operator on the
 * plan's own buffers (three applications each, CUDA events) and keeps the
 * fastest.  Band plans: the integration kernel (register lines at 1 or 2 CTAs
 * per SM, or the shared-memory cores) and the column-tile target of the axis
 * passes; other plans: rows per CTA of the last-axis passes and the column
 * tile of the projection pass.  Choices are cached per plan geometry,
 * precision, coefficient kind and device for the life of the process, so a
 * second plan of the same shape is tuned without timing.  The coefficient
 * must be set.  chosen[3] (host, may be NULL) receives the choice, and
 * ms_per_apply (may be NULL) the time of one application.  Synchronises
 * `stream`.  No counterpart in the reference.
 */
int fhp_plan_autotune(fhp_plan plan, int* chosen, float* ms_per_apply, void* stream);
int fhp_plan_destroy(fhp_plan plan);
/* FHP_MIXED plans: inner relative tolerance floor eta (default 1e-4) and the
   maximum number of refinement steps (default 30). */
int fhp_plan_set_refinement(fhp_plan plan, double eta, int max_outer);
/* voxels = prod(n); components = dv per load; elem_bytes = 8 or 4. */
int fhp_plan_query(fhp_plan plan, long long* voxels, int* components, int* loads,
                   int* elem_bytes);

/*
 * Coefficient A on the solve grid, float64 values [c][n0][n1][n2] with
 * c = 1 (ISO), dv(dv+1)/2 (SYM, packed upper triangle) or dv*dv (FULL);
 * values on host (on_device = 0) or device.  Converted to the plan precision.
 * Replaces: the Tensor produced by Material.get_A_GaNi / get_A_Ga
 * (ffthompy/materials.py:54-123) as the A factor of FiGFA.
 */
int fhp_set_coefficient(fhp_plan plan, int kind, const double* values, int on_device,
                        void* stream);

/*
 * y = iF( G . F( A . x ) ) for every load (x, y device, all loads).
 * Replaces: Operator(name='FiGFA', mat=[[GN, A]]).__call__
 * (ffthompy/applications.py:58, ffthompy/tensors/operators.py:136-144).
 */
int fhp_apply(fhp_plan plan, int proj, const void* x, void* y, void* stream);

/*
 * b_l = FiGFA(-E_l), E_l the constant unit field of load l.
 * Replaces: B = Afun(-EN) (ffthompy/applications.py:64-69,150-155).
 */
int fhp_rhs_macro(fhp_plan plan, int proj, void* b, void* stream);

/*
 * Conjugate gradients on all loads at once, each load with its own scalars
 * and stopping test sqrt(<R,R>) <= tol, <u,v> = sum(u*v)/prod(n).
 * x0 may be NULL (zero start).  kit[loads], norm_res[loads], status[loads]
 * (host) receive the per-load results (status FHP_OK, FHP_NONCONVERGED,
 * FHP_BREAKDOWN or FHP_NONFINITE per load; the call itself returns FHP_OK
 * unless an argument, memory or CUDA error occurred); res_log (host, may be
 * NULL) receives log_rows x loads residual norms (row k = iteration k).
 * FHP_MIXED plans run iterative refinement: FP64 residuals, FP32 inner CG.
 * Replaces: linear_solver(..., solver='CG') / CG
 * (ffthompy/general/solver.py:8-60, 80-139).
 */
int fhp_cg_solve(fhp_plan plan, int proj, const void* b, const void* x0, double tol,
                 int maxiter, void* x, int* kit, double* norm_res, int* status,
                 double* res_log, int log_rows, void* stream);

/*
 * CG on several plans at once: an ensemble of independent cells (grids may
 * differ), each solving its own loads from its own right-hand sides b[i] into
 * x[i] from a zero start, with its own scalars and stopping tests, exactly as
 * fhp_cg_solve would.  The plans advance together: every iteration of all of
 * them is one CUDA graph (the plans' kernels forked over a pool of streams),
 * and the host checks one combined done flag.  kit, norm_res and status
 * (host, may be NULL) receive the per-load results concatenated over the
 * plans in order.  The plans must all be FHP_MIXED (refinement, each outer
 * step's FP32 solves advanced together) or all not, and no plan may appear
 * twice.  Replaces: one applications.scalar / elasticity run per cell
 * (ffthompy/applications.py:11-90, 93-176), i.e. linear_solver(..., 'CG')
 * called once per cell and load (ffthompy/general/solver.py:80-139).
 */
int fhp_cg_solve_many(int count, const fhp_plan* plans, int proj, const void* const* b,
                      double tol, int maxiter, void* const* x, int* kit, double* norm_res,
                      int* status, void* stream);

/*
 * The reference's other linear solvers over the fused operator, all loads at
 * once with per-load scalars and stopping tests kept on the device (one
 * CUDA-graph replay per iteration, the host reads only an all-done flag):
 * fhp_richardson_solve: x += omega (b - A x) while the norm of the residual
 *   of the previous iterate exceeds tol (norm_res starts at 1e15).
 *   Replaces: richardson / 'iterative' (ffthompy/general/solver.py:63-77).
 * fhp_chebyshev_solve: the two-term Chebyshev iteration for eigenvalues in
 *   [eig_min, eig_max]; norm_res relative to the first residual (r0 / |b| at
 *   the start).  Replaces: cheby2TERM (solver.py:206-285).
 * fhp_bicg_solve: biconjugate gradients with the operator as its own
 *   transpose, shadow residual and directions updated with it, stopping test
 *   sqrt(<R, Rs>) <= tol.  Replaces: BiCG (solver.py:142-204; see the
 *   package's general/solver.py for the scalar product it uses).
 * x0 may be NULL (zero start); kit, norm_res, status as fhp_cg_solve.
 * FHP_MIXED plans run these in FP64.
 */
int fhp_richardson_solve(fhp_plan plan, int proj, const void* b, const void* x0, double omega,
                         double tol, int maxiter, void* x, int* kit, double* norm_res,
                         int* status, void* stream);
int fhp_chebyshev_solve(fhp_plan plan, int proj, const void* b, const void* x0, double eig_min,
                        double eig_max, double tol, int maxiter, void* x, int* kit,
                        double* norm_res, int* status, void* stream);
int fhp_bicg_solve(fhp_plan plan, int proj, const void* b, const void* x0, double tol,
                   int maxiter, void* x, int* kit, double* norm_res, int* status, void* stream);

/*
 * AH[i*loads + j] = <A u_i, u_j>, u_i = X_i + E_i if add_macro else X_i
 * (AH on host, float64, accumulated in FP64).
 * Replaces: assembly_matrix (ffthompy/postprocess.py:53-70) with
 * add_macro2minimizer (ffthompy/postprocess.py:73-86).
 */
int fhp_energy_matrix(fhp_plan plan, const void* X, int add_macro, double* AH, void* stream);

/*
 * Coefficient gradient of a weighted energy matrix, for adjoint / sensitivity
 * use: grad[c][v] = sum_ij W[i*loads + j] dA_H[i][j] / dA_c(v), where A_c(v)
 * are the stored coefficient components of the plan's kind at voxel v
 * (ISO: a(v); SYM: packed upper triangle; FULL: dv*dv) and A_H is as in
 * fhp_energy_matrix.  At the CG solution the fields are stationary, so no
 * adjoint solve is needed.  W on host (loads*loads), X and grad device
 * (grad float64, components x voxels of the solve grid).  Plans with the
 * coefficient on a band integration grid return FHP_BAD_ARG.
 * No counterpart in the reference (it has no derivatives); the derivative of
 * assembly_matrix (ffthompy/postprocess.py:53-70) at the solution.
 */
int fhp_energy_gradient(fhp_plan plan, const void* X, int add_macro, const double* W,
                        double* grad, void* stream);

/*
 * Trigonometric interpolation of the fields of plan src onto the grid of
 * plan dst (same field count and precision; dst grid >= src grid).
 * Replaces: Tensor.project / Tensor.enlarge (ffthompy/tensors/objects.py:
 * 428-467, 488-511) as used by assembly_matrix for the Ga bounds.
 */
int fhp_fourier_interp(fhp_plan src, fhp_plan dst, const void* x_src, void* x_dst,
                       void* stream);

/*
 * End to end with HOST buffers: upload the coefficient, build the right-hand
 * sides, solve all loads by CG, assemble A_H (with the macroscopic field
 * added) and copy AH / kit / norm_res (and the solution if x_host != NULL)
 * back.  Replaces: the per-primal/dual body of applications.scalar /
 * applications.elasticity with postprocess kind equal to the solve kind
 * (ffthompy/applications.py:39-90, 124-176).
 */
int fhp_homogenize_host(fhp_plan plan, int proj, int coef_kind, const double* coef_host,
                        double tol, int maxiter, double* AH_host, int* kit_host,
                        double* norm_res_host, void* x_host, void* stream);
/*
 * fhp_homogenize_host for `count` coefficients of the same plan in turn
 * (coef_host[k] host arrays; pinned memory lets the uploads overlap): the
 * upload of coefficient k + 1 runs on a second stream of the plan while
 * problem k is solved.  AH_host holds count x (cells x L x L) values, kit_host
 * and norm_res_host count x (cells x L).  Replaces: the reference's loop of
 * applications.scalar / elasticity runs over several materials of one grid
 * (ffthompy/applications.py:11-176).
 */
int fhp_homogenize_host_many(fhp_plan plan, int proj, int coef_kind, int count,
                             const double* const* coef_host, double tol, int maxiter,
                             double* AH_host, int* kit_host, double* norm_res_host,
                             void* stream);

/*
 * Potential formulation with the 1/|xi| preconditioner (scalar physics; plans
 * created by fhp_plan_create, not the band variant).  The unknown is a scalar
 * potential per load in the 'r' Fourier form of the plan's band grid N
 * (n_band): unnormalised half spectra [load][N0][N1][N2/2+1] of complex
 * values (interleaved re/im) of the plan's element type, device pointers.
 * The solve grid n is N (GaNi) or any larger grid with N odd (Ga: 2N-1), on
 * which the coefficient lives.  P = 1/|2 pi xi| (1 at the mean).
 *
 * fhp_potential_rhs: bh_l = P div(decrease_N F(A E_l)), E_l = unit vector l.
 *   Replaces: P*B of homog_GaNi_full_potential / homog_Ga_full_potential
 *   (ffthompy/tensorsLowRank/homogenisation.py:58-65, 95-101, 296-300).
 * fhp_potential_apply: yh = P (-div) decrease_N F(A iF(enlarge_n(grad(P xh)))).
 *   Replaces: PDFAFGPfun (homogenisation.py:50-65, 88-101).
 * fhp_potential_cg: CG from x0 = 0 on the preconditioned system with the
 *   'r' Fourier inner product (ffthompy/tensors/objects.py:618-631); per-load
 *   kit / norm_res / status and a residual log (log_rows x loads, host) as
 *   fhp_cg_solve.  xh receives iPU; the potential is Fu = P iPU.
 *   Replaces: linear_solver(solver='CG', Afun=PDFAFGPfun, B=PB, x0=0)
 *   (homogenisation.py:66-69, 104-106; ffthompy/general/solver.py:80-139).
 * fhp_potential_field: X = iF(enlarge_n(grad(P xh))) as plan fields
 *   [load][dim][n...]; A_H then follows from fhp_energy_matrix(add_macro=1).
 *   Replaces: X = iF2(grad(Fu).project(Nbar)) / iF(grad(Fu)) and
 *   AH = A(X+E)*(X+E) (homogenisation.py:74-79, 114-125).
 */
int fhp_potential_rhs(fhp_plan plan, void* bh, void* stream);
int fhp_potential_apply(fhp_plan plan, const void* xh, void* yh, void* stream);
int fhp_potential_cg(fhp_plan plan, const void* bh, double tol, int maxiter, void* xh, int* kit,
                     double* norm_res, int* status, double* res_log, int log_rows,
                     void* stream);
int fhp_potential_field(fhp_plan plan, const void* xh, void* X, void* stream);

/*
 * Plain FFT plan of ncomp real fields on grid n (no physics): used for
 * coefficient assembly.  Fields are [ncomp][n0][n1][n2].
 */
int fhp_fft_plan_create(fhp_plan* out, int dim, const int* n, int ncomp, int precision);

/*
 * Exact-integration coefficient of a voxel image on the 2N-1 grid:
 * out = real( iDFT( W . H ) ) with H the DFT of the image on grid P read
 * through the per-axis source index tables src_index (host, concatenated per
 * axis, sum(n_out) ints; the reference's periodic tiling + central crop) and
 * W the separable cell-shape weights (host, concatenated per axis, doubles).
 * image (device, plan_img grid, origin 0) and out (device, plan_out grid,
 * origin 0) hold ncomp fields each.
 * Replaces: Material.get_A_Ga grid-based branch (ffthompy/materials.py:77-110).
 */
int fhp_ga_grid_coefficient(fhp_plan plan_img, fhp_plan plan_out, const void* image,
                            const int* src_index, const double* weights, void* out,
                            void* stream);

/*
 * Characteristic function of a ball inclusion for the exact-integration (Ga)
 * coefficient: out = real(iDFT(X)) * prod(n), origin 0, with
 * X = W(|xi|) prod_a phase_a, W = r^2 J1(2 pi r |xi|) / (r |xi|) / volume
 * (pi r^2 / volume at xi = 0; J1 is CUDA's j1).  plan: an FP64
 * fhp_fft_plan_create plan of one component on a grid odd on every axis.
 * Host tables per axis, concatenated, indexed by the centred position i of
 * the axis (i - n_a/2 the frequency): sq (sum n doubles) = xi_a^2 and phase
 * (2 sum n doubles, interleaved re/im) = the phase the caller pairs with that
 * position.  The real part is formed as the inverse c2r transform of the
 * Hermitian part (X(k) + conj X(-k)) / 2, so a phase table that is not
 * conjugate-symmetric is handled as the reference's .real handles it.
 * out: float64 device array on the plan's grid.  Synchronises `stream`.
 * Replaces, for balls: get_weights_circ (ffthompy/materials.py:392-425), the
 * phase of get_shift_inclusion (materials.py:317-330) and the centred inverse
 * DFT of Material.get_shape_functions (materials.py:125-169).
 */
int fhp_ball_characteristic(fhp_plan plan, double r, double volume, const double* sq,
                            const double* phase, void* out, void* stream);

/*
 * Nodal indicator of a ball summed over its 3^dim periodic images (the
 * topology of Material.get_A_GaNi): out[x] = number of images im in
 * {-1,0,1}^dim with sqrt(sum_a ((x_a - x0_a) - Y_a im_a)^2) < radius, each
 * difference, square and sum rounded as NumPy evaluates them (bit-identical).
 * axes: host, concatenated per-axis node coordinates (sum n doubles); x0, Y:
 * host, dim doubles; out: float64 device array [n0]..[n_{dim-1}].  dim 2 or 3.
 * Replaces: the ball branch of Material.get_topologies
 * (ffthompy/materials.py:212-301).
 */
int fhp_ball_topology(int dim, const int* n, const double* axes, const double* x0,
                      const double* Y, double radius, double* out, void* stream);

/*
 * Characteristic function of a separable inclusion (a box or a bilinear
 * pyramid): out[x] = prod_a re_a[x_a] when im is NULL, else the real part of
 * prod_a (re_a + i im_a)[x_a] - the per-axis factors of its GaNi topology
 * (sums over the periodic images) or of its Ga spectrum transformed per axis.
 * re, im: host, concatenated per axis (sum n doubles each); out: float64
 * device array [n0]..[n_{dim-1}].  Products are formed left to right and the
 * complex ones as NumPy forms them (bit-identical to its outer products).
 * dim 2 or 3.  Replaces, for boxes and pyramids: the topologies of
 * Material.get_topologies (ffthompy/materials.py:212-301) and the centred
 * inverse DFT of Material.get_shape_functions (materials.py:125-169).
 */
int fhp_separable_char(int dim, const int* n, const double* re, const double* im, double* out,
                       void* stream);

/*
 * out[k][i] += v[k] * c[i] for k < nv, i < M: one inclusion's value matrix
 * (nv = d_v^2 host doubles) times its characteristic function c (device,
 * M doubles) added to the coefficient field out (device, [nv][M]), product and
 * sum rounded as NumPy rounds val += np.multiply.outer(v, c) (bit-identical).
 * c and out must not overlap.  1 <= nv <= 36.
 * Replaces: the sum over inclusions of Material.get_A_Ga, order None
 * (ffthompy/materials.py:66-75).
 */
int fhp_outer_accumulate(int nv, const double* v, const double* c, double* out, long long M,
                         void* stream);

/*
 * Per-voxel inverse of a field of d x d matrices (the dual coefficient):
 * Ainv(x) = A(x)^-1 by Gauss-Jordan elimination without pivoting, in the
 * reference's order, each product and difference rounded separately as NumPy
 * evaluates them: bit-identical to the reference for finite input, and a zero
 * pivot gives the reference's Inf / NaN.  A and Ainv are float64 device arrays
 * [d][d][n0]...[n_{dim-1}] (C order) that must not overlap; shift = 1 writes the
 * result ifftshift-ed over the grid axes (Ainv at j from A at (j + n/2) mod n,
 * a centred origin moved to 0).  1 <= dim <= 3, 1 <= d <= 6, n[i] <= 65535.
 * Written on `stream`; the call does not synchronise.
 * Replaces: get_inverse (ffthompy/trigpol.py:120-159) behind Tensor.inv
 * (ffthompy/tensors/objects.py:247-251), and with shift = 1 the inverse plus
 * origin shift of Material.get_A_GaNi(primaldual='dual')
 * (ffthompy/materials.py:115-123).
 */
int fhp_coefficient_inverse(int dim, const int* n, int d, const double* A, double* Ainv,
                            int shift, void* stream);

/*
 * Per-kernel timing with CUDA events recorded on the launch stream around each
 * operator / CG pass (enable resets the counters).  fhp_profile_read returns
 * up to max_kinds entries: names (64 chars each), launches, total ms and the
 * algorithmic bytes per launch (each input read once, each output written
 * once); *nkinds receives the number of kinds recorded.
 */
int fhp_profile_enable(fhp_plan plan, int enable);
int fhp_profile_read(fhp_plan plan, int max_kinds, char* names, long long* launches,
                     double* total_ms, double* bytes_per_launch, int* nkinds);

/* Number of kernel launches issued by this plan since creation. */
long long fhp_plan_launches(fhp_plan plan);

/*
 * A_H[i*loads + j] = <A u_i, u_j> as fhp_energy_matrix computes it, for fields
 * and a coefficient on one grid, without a plan and without allocating
 * anything: one kernel launch whose block partial sums go to a fixed scratch
 * array inside the library (36,896 doubles, 288.25 KiB per device).
 * For callers that must not allocate while they run: code whose device memory
 * is all owned by another allocator (a framework's caching allocator, or a pool
 * reserved up front to the limit of HBM), where a cudaMalloc from inside a
 * library fails or stalls the device, and loops that must not wait on the host.
 * X [loads][dv][n...] and A [c][n...] (c as for fhp_set_coefficient) are
 * float64 device arrays; AH is a float64 device array of loads*loads, written
 * on `stream`; the call does not synchronise.
 * Limits: loads <= 6 and dv <= 6 (the scratch holds 6 x 6 accumulators for at
 * most 1024 blocks); larger sizes return FHP_BAD_ARG.
 * Every call on a device uses the same scratch: calls that overlap in time on
 * one device (several streams or host threads) race, so serialise them.
 * Every call looks up the scratch's device address (no allocation); the first
 * call on each device also loads the kernels: make that call before any stream
 * capture.
 * No counterpart in the reference: its assembly_matrix
 * (ffthompy/postprocess.py:53-70) is the same sum, with no allocation contract.
 */
int fhp_energy_matrix_noalloc(int dim, const int* n, int dv, int loads, int kind,
                              const double* A, const double* X, int add_macro, double* AH,
                              void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FFTHOMPY_GB300_H */
