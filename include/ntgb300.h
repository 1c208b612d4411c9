/*
 * ntgb300.h - C ABI of the GB300-native spectral-element Helmholtz/Poisson
 * hot path (ax_helm, gather-scatter, Jacobi-PCG, residual projection,
 * mixed-precision CG and GMRES, overlapping Schwarz, learned initial guess,
 * RAMP/Brinkman coefficient kernels and the masked vector kernels of
 * neko-top) and of the steps either side of it: the derivative operators,
 * the Pn/Pn residuals, the adjoint and linearised advection terms (with and
 * without dealiasing), the minimum-dissipation forcing, the MMA optimiser
 * and Nek5000 field files.
 *
 * Conventions (the same as the reference's own C ABI in
 * sources/neko_ext/math/bcknd/device/cuda/math_ext.cu:41-108 and its
 * Fortran bind(c) blocks in sources/neko_ext/math/bcknd/device_math_ext.f90:43-103):
 *   - plain C types only; field arrays are DEVICE pointers (Neko's x_d),
 *     laid out as x(lx,ly,lz,nelv) with i fastest;
 *   - real = double unless a function says float;
 *   - every function returns an int status (NTG_OK = 0) instead of
 *     aborting; the reference's cuda_* masked kernels keep their void
 *     signature and report through ntg_last_error();
 *   - masks are index lists with an explicit base (Neko masks are 1-based);
 *   - a plan owns every buffer it allocates and frees it in *_destroy;
 *     caller pointers are never freed by the library;
 *   - all kernels of a plan run on the plan's stream (default: the legacy
 *     default stream); calls on one plan are not re-entrant.
 */
#ifndef NTGB300_H
#define NTGB300_H

#include <stdint.h>

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif
#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
enum {
  NTG_OK = 0,
  NTG_ERR_INVALID = 1,     /* bad argument or handle */
  NTG_ERR_CUDA = 2,        /* a CUDA call failed */
  NTG_ERR_ALLOC = 3,       /* device allocation failed */
  NTG_ERR_UNSUPPORTED = 4, /* polynomial order not compiled in */
  NTG_MAXITER = 10,        /* solve stopped at max_iter before the tolerance */
  NTG_BREAKDOWN = 11,      /* p.Ap <= 0 (operator not SPD) */
  NTG_NONFINITE = 12,      /* NaN/Inf met in a residual or a dot product */
  NTG_GUESS_REJECTED = 13  /* learned guess worse than the fallback; fallback used */
};

/* gather-scatter operations (Neko GS_OP_ADD/MUL/MIN/MAX) */
enum { NTG_GS_ADD = 1, NTG_GS_MUL = 2, NTG_GS_MIN = 3, NTG_GS_MAX = 4 };

/* precision selector for operator applications */
enum { NTG_FP64 = 0, NTG_FP32 = 1 };

/* Krylov solver types */
enum {
  NTG_KSP_CG = 0,        /* Jacobi-PCG, FP64 throughout (the plain drop-in) */
  NTG_KSP_FCG_MIXED = 1, /* FP64 flexible CG whose preconditioner is an FP32
                            Jacobi-PCG inner solve (FP32 Ax, FP32 Jacobi, FP32
                            geometric factors); FP64 residuals and dots */
  NTG_KSP_CG_MIXED = 2,  /* Jacobi-PCG iterated in FP32 with FP64 reliable
                            updates: the FP32 correction is folded into the
                            FP64 solution and the residual recomputed in FP64
                            (FP64 operator) whenever the FP32 residual fell by
                            delta (ntg_ksp_set_inner's first argument, default
                            0.1); convergence is confirmed on the FP64 residual */
  NTG_KSP_GMRES = 3,      /* restarted flexible GMRES(m), FP64 (Neko's 'gmres';
                            Jacobi or the Schwarz preconditioner) */
  NTG_KSP_GMRES_MIXED = 4 /* FP32 flexible GMRES(m) cycles inside FP64
                            iterative refinement: each cycle starts from the
                            FP64 residual and reduces it by delta
                            (ntg_ksp_set_inner's first argument, default 1e-4)
                            or m steps; x accumulates in FP64 */
};

typedef struct ntg_plan ntg_plan; /* mesh + coef_t + gs_t + Jacobi state */
typedef struct ntg_ksp ntg_ksp;   /* Krylov solver workspace */
typedef struct ntg_proj ntg_proj; /* residual projection space */
typedef struct ntg_guess ntg_guess; /* learned initial-guess network */
typedef struct ntg_schwarz ntg_schwarz; /* overlapping Schwarz preconditioner */
typedef struct ntg_dealias ntg_dealias; /* GL over-integration space of a plan */
typedef struct ntg_mma ntg_mma;         /* MMA optimiser state */

/* ksp_monitor_t of the reference (iter, res_start, res_final;
   sources/mapping_functions/PDE_filter_mapping.f90:265-272), plus the
   status, the outer/inner split of the mixed solver and device time. */
typedef struct ntg_monitor {
  int iter;          /* outer iterations (CG: all iterations) */
  int inner_iter;    /* total inner FP32 iterations (mixed solver) */
  double res_start;  /* ||r0|| (mult-weighted, i.e. over unique nodes) */
  double res_final;  /* ||r|| at exit, recomputed in FP64 */
  double rhs_norm;   /* ||f|| */
  int status;        /* NTG_OK, NTG_MAXITER, NTG_BREAKDOWN, NTG_NONFINITE */
  int fp64_ax;       /* FP64 operator applications performed */
  int guess_rejected; /* 1 if the guess guard replaced the guess by zero */
} ntg_monitor;

/* ---------------------------------------------------------------------- */
/* library                                                                */
/* ---------------------------------------------------------------------- */
const char* ntg_version(void);
/* message of the last error on this host thread ("" if none) */
const char* ntg_last_error(void);
/* compiled polynomial orders: writes up to cap values of lx, returns count */
int ntg_supported_lx(int* lx, int cap);
/* kernels the library has launched in this process (all entry points) */
unsigned long long ntg_launch_count(void);
/* per-kernel device timers (CUDA events around each launch, on the
   launching stream).  Ids: 0 FP64 Ax, 1 FP32 Ax, 2 FP64 gs, 3 FP32 gs, 4/5
   CG update FP64/FP32, 6/7 CG direction FP64/FP32, 8 the whole FP32
   preconditioner application, 9 Schwarz FDM local solves, 10 Schwarz
   coarse solve, 11 Schwarz prolongation (pull).  Off by default. */
int ntg_timer_enable(int on);
int ntg_timer_read(int id, double* total_ms, long long* count);
int ntg_timer_reset(void);
/* Neko's profiler_start_region(name, colour) / profiler_end_region as NVTX
   ranges (the reference's regions: sources/adjoint/adjoint_pnpn.f90:715,
   733,746,783; sources/mapping_functions/PDE_filter_mapping.f90:254,341).
   colour <= 0: no colour.  Regions nest; end closes the innermost. */
int ntg_profiler_start_region(const char* name, int colour);
int ntg_profiler_end_region(void);

/* ---------------------------------------------------------------------- */
/* mesh / coef_t / gs_t plan                                               */
/* Replaces: coef_t init + gs_t init (Neko; called at                      */
/* sources/adjoint/adjoint_scheme.f90:341-343) and dofmap_t's global ids.  */
/* ---------------------------------------------------------------------- */
/* Build a plan from node coordinates x_d,y_d,z_d (device, n = nelv*lx^3
   doubles each) and global node ids glb_d (device, n int64; equal ids are
   the same mesh node).  Computes G11..G33, B, mult and the gs maps on the
   device. */
int ntg_plan_create(ntg_plan** plan, int64_t nelv, int lx, const double* x_d, const double* y_d,
                    const double* z_d, const int64_t* glb_d);
int ntg_plan_destroy(ntg_plan* plan);
/* stream: a cudaStream_t cast to void* (NULL = legacy default stream) */
int ntg_plan_set_stream(ntg_plan* plan, void* stream);
/* sizes: n local DOFs, nu unique nodes, nshared segments with > 1 copy */
int ntg_plan_info(const ntg_plan* plan, int64_t* nelv, int* lx, int64_t* n, int64_t* nu, int64_t* nshared);
/* copy the geometric factors / mass / multiplicity into caller device
   arrays (any pointer may be NULL) */
int ntg_coef_get(const ntg_plan* plan, double* g11_d, double* g12_d, double* g13_d, double* g22_d,
                 double* g23_d, double* g33_d, double* B_d, double* mult_d);
/* Helmholtz coefficients (coef%h1, coef%h2, coef%ifh2).  h1_d == NULL ->
   constant h1c; h2_d == NULL with ifh2 -> constant h2c; ifh2 == 0 -> no
   mass term.  Values are copied (FP64 and FP32); h2*B is precombined. */
int ntg_coef_set(ntg_plan* plan, const double* h1_d, double h1c, const double* h2_d, double h2c, int ifh2);
/* Dirichlet mask (bc_list): index list mask_d (device int32, nmask
   entries) in base `base` (1 for Neko masks).  nmask == 0 clears it. */
int ntg_plan_set_mask(ntg_plan* plan, const int32_t* mask_d, int64_t nmask, int base);
/* FP32 Ax path: 1 (default) = bulk-copy pipelined kernel for lx = 8, 0 =
   the generic kernel (both give the same results within FP32 rounding) */
int ntg_plan_set_ax_path(ntg_plan* plan, int use_tma);
/* gather-scatter kernel: 1 (default) = groups split by multiplicity with
   vector index loads, 0 = one thread per group (bit-identical results) */
int ntg_plan_set_gs_path(ntg_plan* plan, int by_class);
/* *flag = 1 if a bounded device wait of one of the plan's kernels ran out
   since the last call (that launch's output is invalid) */
int ntg_plan_check_error(ntg_plan* plan, int* flag);
/* gs maps: perm (n int32: local indices sorted by global id, stable) and
   offs (nu+1 int64 segment offsets), device arrays */
int ntg_gs_export(const ntg_plan* plan, int32_t* perm_d, int64_t* offs_d);

/* ---------------------------------------------------------------------- */
/* synthetic mesh generator (replaces Neko's genmeshbox for the tests and  */
/* benchmark; examples/rugby_ball/prepare.sh uses genmeshbox)             */
/* ---------------------------------------------------------------------- */
/* Box of ex*ey*ez hexes on [lo,hi]^3 with GLL nodes of order lx-1 and a
   seeded sinusoidal deformation of amplitude amp*h per axis. Writes
   coordinates and global ids (device arrays of n entries). */
int ntg_mesh_box(int ex, int ey, int ez, int lx, const double* lo3, const double* hi3, double amp,
                 uint64_t seed, double* x_d, double* y_d, double* z_d, int64_t* glb_d, void* stream);
/* 1-based local indices of the x = hi face (nmask = ex*ey*ez/ex * lx^2
   entries when mask_d != NULL).  Returns the count in *nmask. */
int ntg_mask_face_xmax(int ex, int ey, int ez, int lx, int32_t* mask_d, int64_t* nmask, void* stream);
/* seeded synthetic fields (SplitMix64 keyed by (seed, stream_id, global id)):
   uniform in [lo, hi) per global node */
int ntg_field_uniform(const int64_t* gid_d, int64_t n, uint64_t seed, uint64_t stream_id, double lo, double hi,
                      double* f_d, void* stream);
/* sum of nmodes Fourier modes cos(2 pi k.X + phi) with amplitudes
   U[-1,1]/|k|^2, k in [1,kmax]^3, X the coordinates normalised by the box */
int ntg_field_fourier(const double* x_d, const double* y_d, const double* z_d, int64_t n, const double* lo3,
                      const double* hi3, int nmodes, int kmax, uint64_t seed, double* f_d, void* stream);
/* the same modes with explicit parameters (host arrays: k 3*nmodes ints,
   amplitudes, phases), for right-hand-side sequences */
int ntg_field_modes(const double* x_d, const double* y_d, const double* z_d, int64_t n, const double* lo3,
                    const double* hi3, int nmodes, const int* k, const double* amp, const double* ph, double* f_d,
                    void* stream);
/* clip(sum of nblobs Gaussians of the given width, 0, 1), centres U(box) */
int ntg_field_blobs(const double* x_d, const double* y_d, const double* z_d, int64_t n, const double* lo3,
                    const double* hi3, uint64_t seed, int nblobs, double width, double* f_d, void* stream);
/* weak right-hand side b = mask(gs(B f)) */
int ntg_rhs_assemble(ntg_plan* plan, const double* f_d, double* b_d);

/* ---------------------------------------------------------------------- */
/* ax_t (ax_helm): w = h1 (D^T G D) u + h2 B u, element-local.            */
/* Replaces: ax_helm_factory(Ax, full_formulation=.false.)%compute (Neko; */
/* sources/mapping_functions/PDE_filter_mapping.f90:177,256,               */
/* sources/adjoint/adjoint_pnpn.f90:207,217).                              */
/* ---------------------------------------------------------------------- */
int ntg_ax_helm(ntg_plan* plan, double* w_d, const double* u_d);
int ntg_ax_helm_f32(ntg_plan* plan, float* w_d, const float* u_d);

/* ---------------------------------------------------------------------- */
/* gs_t%op(u, n, op) (Neko; sources/adjoint/adjoint_pnpn.f90:725,755-757, */
/* sources/mapping_functions/PDE_filter_mapping.f90:249)                  */
/* ---------------------------------------------------------------------- */
int ntg_gs_op(ntg_plan* plan, double* u_d, int op);
int ntg_gs_op_f32(ntg_plan* plan, float* u_d, int op);

/* bc_list_apply_scalar(bclst, x, n): zero the masked entries
   (sources/adjoint/adjoint_pnpn.f90:726) */
int ntg_bc_apply_scalar(ntg_plan* plan, double* x_d);
/* the same for an FP32 field */
int ntg_bc_apply_scalar_f32(ntg_plan* plan, float* x_d);

/* ---------------------------------------------------------------------- */
/* pc_t (Jacobi): update() builds 1/gs(diag A) in FP64 and FP32;          */
/* solve(z, r) applies it.  (sources/adjoint/adjoint_pnpn.f90:732,781,     */
/* sources/mapping_functions/PDE_filter_mapping.f90:262,365-400)          */
/* ---------------------------------------------------------------------- */
int ntg_pc_jacobi_update(ntg_plan* plan);
int ntg_pc_jacobi_solve(ntg_plan* plan, double* z_d, const double* r_d);
/* copy the FP64 inverse diagonal into dinv_d */
int ntg_pc_jacobi_get(const ntg_plan* plan, double* dinv_d);

/* ---------------------------------------------------------------------- */
/* Meshes from Neko's binary .nmsh files (the reference's cases load their  */
/* meshes as "mesh_file": "*.nmsh", e.g. examples/brinkman_term/            */
/* brinkman_term.case:4).  Host buffers; vertices in tensor corner order    */
/* (v = i + 2j + 4k; the file stores each layer cyclically); zones as      */
/* stored, 9 int32 each (e, f, p_e, p_f, pt_ids[4], type; f 1-based: r-,   */
/* r+, s-, s+, t-, t+; labeled zones, type 7, carry the label in p_f);     */
/* curves as stored (element, 12 x 5 float64, 12 int32 types).  nv = 8 for */
/* gdim 3, 4 for gdim 2.                                                     */
/* ---------------------------------------------------------------------- */
int ntg_nmsh_info(const char* path, int32_t* nelv, int32_t* gdim, int32_t* nzones, int32_t* ncurves);
/* el_idx: nelv; v_idx: nelv x nv; xyz: nelv x nv x 3; zones: nzones x 9;  */
/* curve_el: ncurves; curve_data: ncurves x 60; curve_type: ncurves x 12   */
int ntg_nmsh_read(const char* path, int32_t* el_idx, int32_t* v_idx, double* xyz, int32_t* zones,
                  int32_t* curve_el, double* curve_data, int32_t* curve_type);
int ntg_nmsh_write(const char* path, int32_t nelv, int32_t gdim, const int32_t* el_idx, const int32_t* v_idx,
                   const double* xyz, int32_t nzones, const int32_t* zones, int32_t ncurves,
                   const int32_t* curve_el, const double* curve_data, const int32_t* curve_type);
/* GLL node coordinates (x fastest per element) of straight-sided hexahedra */
/* from their tensor-ordered vertices (xyz_d: device, nelv x 8 x 3)         */
int ntg_nodes_from_vertices(int64_t nelv, int lx, const double* xyz_d, double* x_d, double* y_d, double* z_d,
                            void* stream);

/* ---------------------------------------------------------------------- */
/* Overlapping additive Schwarz preconditioner in FP32 (fast-diagonalisation */
/* local solves on each element extended by one node layer), the one-level */
/* part of the Schwarz-multigrid pressure preconditioner ('hsmg') the      */
/* reference's cases select (examples/rugby_ball/rugby_ball.case:46-52).   */
/* lx in {4, 6, 8}.  ntg_schwarz_create: structured boxes, ex*ey*ez       */
/* elements numbered x fastest (as built by ntg_mesh_box).                  */
/* ntg_schwarz_create_general: any conforming hexahedral mesh (read from   */
/* .nmsh, neighbours in any orientation): each element is extended across  */
/* its six faces only (the face neighbours' nodes one step in, found       */
/* through the plan's global node ids; edge and corner positions excluded, */
/* as Neko's Schwarz smoother does on general meshes), and the coarse      */
/* level is the Galerkin Q1 operator P^T A P on the element vertices,      */
/* inverted densely (at most 8192 active vertices).  Every other call      */
/* below takes either kind; the tensor-core FDM path is box-only.          */
/* ---------------------------------------------------------------------- */
int ntg_schwarz_create(ntg_plan* plan, int ex, int ey, int ez, const double* x_d, const double* y_d,
                       const double* z_d, ntg_schwarz** sw);
int ntg_schwarz_create_general(ntg_plan* plan, const double* x_d, const double* y_d, const double* z_d,
                               ntg_schwarz** sw);
/* The general form's face-neighbour table, on the host (no device needed): */
/* gid_h the global node id of every local node (nelv * lx^3); ghost_h      */
/* (nelv * 6 * lx^2) receives, per element face (r-, r+, s-, s+, t-, t+) and */
/* face node (tangential indices, lower axis fastest), the 0-based local    */
/* index one step inside the face neighbour, -1 on the boundary.            */
int ntg_schwarz_ghost_table(int64_t nelv, int lx, const int64_t* gid_h, int32_t* ghost_h);
/* refresh the element means of h1 / h2 after ntg_coef_set (and, with the  */
/* coarse level on, its Dirichlet faces from the plan's mask and h1/h2)    */
int ntg_schwarz_update(ntg_schwarz* sw);
/* Coarse level on/off: adds P A_c^-1 P^T r, A_c the separable Q1 operator */
/* on the (ex+1)(ey+1)(ez+1) element vertices (fast diagonalisation),     */
/* P trilinear interpolation to the GLL nodes -- the coarse-grid part of   */
/* the Schwarz-multigrid preconditioner, here solved directly.  A face     */
/* whose nodes are all masked is Dirichlet on the coarse grid.             */
int ntg_schwarz_set_coarse(ntg_schwarz* sw, int enable);
/* Additive diagonal term for a mass term varying inside elements (Brinkman */
/* penalisation): z += w D^-1 r with D the assembled diagonal and w the     */
/* node's mass fraction (h2 B) / D in [0, 1].                               */
int ntg_schwarz_set_mass_term(ntg_schwarz* sw, int enable);
/* FDM local solves: 0 (default) = FP32 cores with even-odd 1D transforms  */
/* (the reference eigenvectors are symmetric / antisymmetric about the     */
/* extended interval's centre: half the FMAs); 2 = FP32 cores, full 1D     */
/* products; 1 = lx = 8 only, the in-plane transforms on the tcgen05       */
/* tensor cores (one shared 100 x 100 plane operator in BF16, data split   */
/* into two BF16 terms, FP32 accumulation; the third direction in FP32).   */
/* All three are symmetric preconditioners.                                */
int ntg_schwarz_set_fdm_path(ntg_schwarz* sw, int path);
int ntg_schwarz_destroy(ntg_schwarz* sw);
/* z = M r (FP32; assembled and masked) */
int ntg_schwarz_apply(ntg_schwarz* sw, float* z_d, const float* r_d);

/* ---------------------------------------------------------------------- */
/* ksp_t: krylov_solver_factory(ksp, n, type, max_iter, abstol) / solve /  */
/* krylov_solver_destroy (sources/adjoint/adjoint_scheme.f90:1046-1055,    */
/* sources/mapping_functions/PDE_filter_mapping.f90:180-181,197,255-257). */
/* Stopping test: ||r|| <= max(abstol, rtol*||f||), norms weighted by     */
/* mult (unique-node Euclidean norm of the assembled residual).           */
/* ---------------------------------------------------------------------- */
int ntg_ksp_create(ntg_plan* plan, int type, int max_iter, double rtol, double abstol, ntg_ksp** ksp);
int ntg_ksp_destroy(ntg_ksp* ksp);
/* mixed solver: inner relative tolerance and inner iteration cap */
int ntg_ksp_set_inner(ntg_ksp* ksp, double inner_rtol, int inner_max_iter);
/* use the Schwarz preconditioner (NULL: back to Jacobi) in the FP32
   iteration of an NTG_KSP_CG_MIXED solver */
int ntg_ksp_set_schwarz(ntg_ksp* ksp, ntg_schwarz* sw);
/* change the stopping tolerances of an existing solver */
int ntg_ksp_set_tol(ntg_ksp* ksp, double rtol, double abstol);
/* guess guard (default off): when the initial guess's residual exceeds the
   right-hand side's norm, restart from a zero guess and report
   NTG_GUESS_REJECTED in ntg_monitor.guess_rejected */
/* cg_mixed with a structured-box Schwarz preconditioner: gather-scatter,  */
/* mask and vector update of each iteration in one kernel (1, default) or */
/* as three launches (0); the same sums in the same order either way.     */
int ntg_ksp_set_fused_update(ntg_ksp* ksp, int on);
int ntg_ksp_set_guess_guard(ntg_ksp* ksp, int on);
/* how many iterations run between host convergence checks (default 16) */
int ntg_ksp_set_check_every(ntg_ksp* ksp, int every);
/* GMRES restart length m in [1, 31] (default 30) */
int ntg_ksp_set_restart(ntg_ksp* ksp, int m);
/* x_d: initial guess in, solution out.  f_d: assembled, masked RHS. */
int ntg_ksp_solve(ntg_ksp* ksp, double* x_d, const double* f_d, ntg_monitor* mon);
/* solve_coupled for three components with one operator
   (sources/adjoint/adjoint_pnpn.f90:784-786) */
int ntg_ksp_solve_coupled(ntg_ksp* ksp, double* x_d, double* y_d, double* z_d, const double* fx_d,
                          const double* fy_d, const double* fz_d, ntg_monitor* mon3);

/* ---------------------------------------------------------------------- */
/* projection_t (Fischer residual projection): init(n, L) / pre_solving / */
/* post_solving / free (sources/adjoint/adjoint_pnpn.f90:365-374,729-741) */
/* ---------------------------------------------------------------------- */
int ntg_proj_create(ntg_plan* plan, int L, ntg_proj** proj);
int ntg_proj_destroy(ntg_proj* proj);
/* b_d (assembled, masked) is replaced by b - A xbar; xbar is kept */
int ntg_proj_pre_solving(ntg_proj* proj, double* b_d);
/* pre_solving plus one extra direction g_d for this solve only (a learned
   guess): g is A-orthogonalised against the basis and the Galerkin
   component of b along it joins xbar, so the projected guess is never worse
   in the A-norm than plain projection.  One FP64 operator application.
   *used = 0 when g adds no new direction. */
int ntg_proj_pre_solving_with(ntg_proj* proj, double* b_d, const double* g_d, int* used);
/* x_d: the correction solved for on entry, the full solution on exit;
   one FP64 operator application updates the basis */
int ntg_proj_post_solving(ntg_proj* proj, double* x_d);
int ntg_proj_size(const ntg_proj* proj);
/* post_solving for a solution x_d of the full right-hand side found
   elsewhere (another solver, a restart): the basis takes x - xbar as
   post_solving(x - xbar) would; x_d is not modified.  Follows
   ntg_proj_pre_solving (not pre_solving_with). */
int ntg_proj_post_solving_full(ntg_proj* proj, const double* x_d);
/* checkpoint access: dir = 0 stores the basis size in *m and copies the m
   basis vectors and their A-images to xs_d / axs_d (device, m*n doubles
   each; either may be null); dir = 1 loads *m (<= L) of them back. */
int ntg_proj_state(ntg_proj* proj, int* m, double* xs_d, double* axs_d, int dir);

/* ---------------------------------------------------------------------- */
/* learned initial guess (new; the reference has no learned part).  A      */
/* per-element MLP, (history + 1) * lx^3 -> 64 -> 64 -> lx^3 (lx = 8):     */
/* inputs the last `history` solutions and the right-hand side on the      */
/* element's nodes, output a nodal correction of the newest solution (the  */
/* output layer starts at zero, so an untrained net returns the newest     */
/* solution), averaged over shared nodes and masked.  BF16 weights,        */
/* tcgen05 tensor-core GEMMs with FP32 accumulation in tensor memory,      */
/* trained online with Adam on the solver's own solutions (relative energy */
/* + L2 loss of the assembled guess).  Inserted where the reference sets   */
/* the initial guess: projection pre_solving                               */
/* (sources/adjoint/adjoint_pnpn.f90:729) and the filter's guess copy      */
/* (sources/mapping_functions/PDE_filter_mapping.f90:246,332).             */
/* ---------------------------------------------------------------------- */
int ntg_guess_create(ntg_plan* plan, int history, int hidden, uint64_t seed, ntg_guess** guess);
int ntg_guess_destroy(ntg_guess* guess);
int ntg_guess_set_lr(ntg_guess* guess, double lr);
/* guess for the rhs b_d from the stored solution history; *ready = 0 (and
   x_d untouched) until `history` solutions have been observed.  The guess
   is continuous (mult-averaged over shared nodes) and zero on the mask. */
int ntg_guess_predict(ntg_guess* guess, const double* b_d, double* x_d, int* ready);
/* record the solution x_d of rhs b_d: with train_steps > 0 (and a full
   history) first take that many Adam steps on (history, b) -> x, then push
   x into the history.  *loss = the last training loss (-1 if none). */
int ntg_guess_observe(ntg_guess* guess, const double* b_d, const double* x_d, int train_steps, double* loss);
int ntg_guess_reset_history(ntg_guess* guess);
/* checkpoint of the network state: a device FP32 buffer of
   ntg_guess_state_len floats (weights, Adam moments, solution history),
   ints[4] = {Adam step, history head, history count, 0} and hrms[8] (the
   history's RMS scales); dir = 0 stores, dir = 1 loads.  A restored network
   continues bit for bit. */
int64_t ntg_guess_state_len(const ntg_guess* g);
int ntg_guess_state(ntg_guess* g, float* buf_d, long long* ints, double* hrms, int dir);
/* online-training loss: 1 (default) = relative element-energy error
   (e, A_e e)/(x, A_e x) plus relative L2 error (CG pays for energy-norm
   error, so a guess trained in L2 alone carries nodal noise); 0 = MSE */
int ntg_guess_set_loss(ntg_guess* guess, int energy);
/* parameters as one flat FP32 array [W1 | b1 | W2 | b2 | W3 | b3] (W row
   major, [in x out]); set != 0 writes them */
int64_t ntg_guess_num_params(const ntg_guess* guess);
int ntg_guess_params(ntg_guess* guess, float* params_d, int set);
/* raw access for gradient checks: X_d rows are BF16 bit patterns */
int ntg_guess_forward_raw(ntg_guess* guess, const uint16_t* X_d, int64_t E, float* Y_d);
int ntg_guess_grad_raw(ntg_guess* guess, const uint16_t* X_d, const float* T_d, int64_t E, float* grad_d,
                       double* loss);
int ntg_guess_train_raw(ntg_guess* guess, const uint16_t* X_d, const float* T_d, int64_t E, double* loss);

/* BF16 GEMM on the tcgen05 tensor cores (the learned guess's GEMM):
   C = A B^T with A [M x K] (row stride lda) and B [N x K] (row stride
   ldb), BF16, K contiguous, every row 16-byte aligned (lda, ldb multiples
   of 8); C FP32 [M x ldc].  Accumulation in FP32 (tensor memory).  err_d:
   device int set to 1 if a bounded wait of the kernel ran out (null: a
   library-owned flag).  Asynchronous on `stream`. */
int ntg_gemm_bf16(const uint16_t* A_d, int64_t lda, const uint16_t* B_d, int64_t ldb, float* C_d, int64_t ldc,
                  int64_t M, int64_t N, int64_t K, int* err_d, void* stream);

/* ---------------------------------------------------------------------- */
/* dot products (FP64 accumulation, deterministic order)                   */
/* ---------------------------------------------------------------------- */
/* glsc3(a, b, c) = sum a*b*c over n entries */
int ntg_glsc3(ntg_plan* plan, const double* a_d, const double* b_d, const double* c_d, int64_t n, double* out);

/* ---------------------------------------------------------------------- */
/* coefficient path                                                        */
/* ---------------------------------------------------------------------- */
/* RAMP mapping (sources/mapping_functions/RAMP_mapping.f90:182-267) */
int ntg_ramp_forward(double* xout_d, const double* xin_d, int64_t n, double fmin, double fmax, double q,
                     int convex_up, void* stream);
int ntg_ramp_backward(double* dF_din_d, const double* dF_dout_d, const double* xin_d, int64_t n, double fmin,
                      double fmax, double q, int convex_up, void* stream);
/* simple_brinkman_source_term compute: f_c -= u_c * chi
   (sources/source_terms/simple_brinkman_source_term.f90:139-153);
   mask_d == NULL -> all n entries, else the masked entries (base `base`) */
int ntg_brinkman_compute(double* fx_d, double* fy_d, double* fz_d, const double* u_d, const double* v_d,
                         const double* w_d, const double* chi_d, int64_t n, const int32_t* mask_d,
                         int64_t nmask, int base, void* stream);
/* permeability kappa(phi), negated (sources/topology_optimization/design.f90:316-348) */
int ntg_permeability(double* kappa_d, const double* phi_d, int64_t n, double perm0, double perm1,
                     double penalty, void* stream);
/* minimum-dissipation sensitivity -u.u_adj (+ K|u|^2), FP64
   (sources/objectives/minimum_dissipation_objective_function.f90:260-301) */
int ntg_sens_min_dissipation(double* s_d, const double* u_d, const double* v_d, const double* w_d,
                             const double* ua_d, const double* va_d, const double* wa_d, int64_t n,
                             int if_lube, double K_scale, void* stream);
/* PDE filter (r^2 K + B) X_out = B X_in, all-Neumann, guess = X_in
   (sources/mapping_functions/PDE_filter_mapping.f90:212-278 forward,
   :298-363 backward).  Overwrites the plan's h1/h2. */
int ntg_filter_apply(ntg_plan* plan, ntg_ksp* ksp, double* X_out_d, const double* X_in_d, double r,
                     ntg_monitor* mon);

/* ---------------------------------------------------------------------- */
/* derivative operators and the adjoint-equation terms (FP64, on the plan's */
/* stream).  The operators are Neko's (operators.f90: opgrad, dudxyz, cdtp, */
/* conv1, curl) as the reference calls them; ntg_metrics_set must come     */
/* first (it derives the cofactors drdx..dtdz, 1/jac and 1/gs(B) from the   */
/* coordinates, as coef_t's generate_dxyz does).                            */
/* ---------------------------------------------------------------------- */
int ntg_metrics_set(ntg_plan* plan, const double* x_d, const double* y_d, const double* z_d);
/* du = du/dx_dir, strong (dir 0..2) */
int ntg_dudxyz(ntg_plan* plan, double* du_d, const double* u_d, int dir);
/* (ux, uy, uz) = B grad u (weak gradient); adv_adjoint_no_dealias.f90:165-167 */
int ntg_opgrad(ntg_plan* plan, double* ux_d, double* uy_d, double* uz_d, const double* u_d);
/* dtx = transpose of opgrad's `dir` component applied to x;
   adv_adjoint_no_dealias.f90:297-299 */
int ntg_cdtp(ntg_plan* plan, double* dtx_d, const double* x_d, int dir);
/* du = vx du/dx + vy du/dy + vz du/dz (strong); adv_adjoint_no_dealias.f90:383 */
int ntg_conv1(ntg_plan* plan, double* du_d, const double* u_d, const double* vx_d, const double* vy_d,
              const double* vz_d);
/* w = Binv gs(B curl u); adjoint_minimum_dissipation_source_term.f90:231 */
int ntg_curl(ntg_plan* plan, double* w1_d, double* w2_d, double* w3_d, const double* u1_d, const double* u2_d,
             const double* u3_d);
/* adjoint advection without dealiasing, f_i -= sum_j u_j opgrad_i(Ub_j) +
   sum_d cdtp_d(u_i Ub_d) (adv_adjoint_no_dealias.f90:118-255 and 266-302, device
   branch); (vx, vy, vz) the adjoint velocity, (vxb, vyb, vzb) the primal one */
int ntg_adjoint_advection_no_dealias(ntg_plan* plan, double* fx_d, double* fy_d, double* fz_d,
                                     const double* vx_d, const double* vy_d, const double* vz_d,
                                     const double* vxb_d, const double* vyb_d, const double* vzb_d);
/* linearised advection without dealiasing, f_i -= B conv1(u_i; Ub) +
   B conv1(Ub_i; u) (adv_adjoint_no_dealias.f90:365-427 linear_advection_no_dealias) */
int ntg_linear_advection_no_dealias(ntg_plan* plan, double* fx_d, double* fy_d, double* fz_d,
                                    const double* vx_d, const double* vy_d, const double* vz_d,
                                    const double* vxb_d, const double* vyb_d, const double* vzb_d);
/* minimum-dissipation adjoint forcing f += scale curl(curl(u)), kept on the
   zone's nodes only when nzone > 0 (zone_d: nzone unique indices, base
   `base`) (adjoint_minimum_dissipation_source_term.f90:175-249).  Uses the
   plan's derivative scratch (6 n doubles, allocated on first use). */
int ntg_adjoint_min_dissipation(ntg_plan* plan, double* fx_d, double* fy_d, double* fz_d, const double* u_d,
                                const double* v_d, const double* w_d, double scale, const int32_t* zone_d,
                                int64_t nzone, int base);

/* Dealiased advection (sources/adjoint/adv_adjoint_dealias.f90).  create
   replaces init_dealias (:137-224): lxd Gauss-Legendre points per direction
   (lxd <= 0: 3 lx / 2, advection_adjoint_fctry.f90:66-90), the GLL -> GL
   interpolation J and the metric cofactors interpolated to GL (9 x nelv
   lxd^3 doubles).  Needs ntg_metrics_set first; compiled (lx, lxd) pairs:
   (4,6) (5,7) (6,9) (7,10) (8,12).  The handle borrows the plan. */
int ntg_dealias_create(ntg_dealias** d, ntg_plan* plan, int lxd);
int ntg_dealias_destroy(ntg_dealias* d);
int ntg_dealias_info(const ntg_dealias* d, int* lxd, int64_t* ngl);
/* interp_t%map: to_gl != 0: out (GL, nelv lxd^3) = J in (GLL);
   to_gl == 0: out (GLL) = J^T in (GL) */
int ntg_dealias_map(ntg_dealias* d, double* out_d, const double* in_d, int to_gl);
/* f_i -= J^T [ sum_j u_j opgrad_i(Ub_j) + sum_d cdtp_d(u_i Ub_d) ]_GL
   (compute_adjoint_advection_dealias, :235-462) */
int ntg_adjoint_advection_dealias(ntg_dealias* d, double* fx_d, double* fy_d, double* fz_d, const double* vx_d,
                                  const double* vy_d, const double* vz_d, const double* vxb_d, const double* vyb_d,
                                  const double* vzb_d);
/* f_i -= J^T [ u . opgrad(Ub_i) + Ub . opgrad(u_i) ]_GL
   (compute_linear_advection_dealias, :470-600) */
int ntg_linear_advection_dealias(ntg_dealias* d, double* fx_d, double* fy_d, double* fz_d, const double* vx_d,
                                 const double* vy_d, const double* vz_d, const double* vxb_d, const double* vyb_d,
                                 const double* vzb_d);

/* Pn/Pn splitting residuals (FP64), replacing prs_res%compute and
   vel_res%compute (sources/adjoint/adjoint_pnpn.f90:716-723, :747-753).
   mu/rho: fields (mu_d, rho_d) or, when the pointer is NULL, the constants
   mu_c, rho_c; bd = the first BDF coefficient, dt the step.  Results are
   neither gs-assembled nor masked (the caller does both next, as the
   reference does).  The plan's h1/h2 are left untouched.

   p_res = -A(h1 = 1/rho) p + sum_d cdtp_d(ta_d)
           - (bd/dt) sum_c u_c s_c over the velocity-surface entries
           - sum_c ta_c s'_c over the symmetry-surface entries,
   ta_d = Binv gs(f_d / rho - (mu/rho) B curl(curl(u_e))_d).
   Surface lists: prs_idx/sym_idx (n entries, unique, base `base`) with
   s = 3 x n doubles (all x, then all y, then all z): the outward normal
   times the facet area at each entry.  Uses the plan's derivative
   scratch. */
int ntg_pnpn_prs_res(ntg_plan* plan, double* p_res_d, const double* p_d, const double* u_d, const double* v_d,
                     const double* w_d, const double* ue_d, const double* ve_d, const double* we_d,
                     const double* fx_d, const double* fy_d, const double* fz_d, const double* mu_d, double mu_c,
                     const double* rho_d, double rho_c, double bd, double dt, const int32_t* prs_idx_d,
                     const double* prs_s_d, int64_t nprs, const int32_t* sym_idx_d, const double* sym_s_d,
                     int64_t nsym, int base);
/* u_res_c = f_c - (mu K + rho (bd/dt) B) u_c - opgrad_c(p), one fused pass */
int ntg_pnpn_vel_res(ntg_plan* plan, double* u_res_d, double* v_res_d, double* w_res_d, const double* u_d,
                     const double* v_d, const double* w_d, const double* p_d, const double* fx_d, const double* fy_d,
                     const double* fz_d, const double* mu_d, double mu_c, const double* rho_d, double rho_c,
                     double bd, double dt);

/* ---------------------------------------------------------------------- */
/* MMA optimiser on the GPU (FP64), replacing mma_t (sources/mma/mma.f90,  */
/* sources/mma/bcknd/cpu/mma_cpu.f90): Svanberg's method of moving         */
/* asymptotes with the primal-dual interior-point subproblem solver.       */
/* ---------------------------------------------------------------------- */
/* mma_t%init (mma.f90:186-295).  n design variables (x_d, xmin_d, xmax_d:
   device), m in [1, 4] constraints with a, c, d host arrays of m; max_iter
   <= 0, epsimin <= 0, asy* <= 0 take the reference's defaults (100,
   1e-9 sqrt(m + n), 0.5, 1.2, 0.7).  Kernels run on `stream`. */
int ntg_mma_create(ntg_mma** mma, int64_t n, int m, const double* x_d, double a0, const double* a, const double* c,
                   const double* d, const double* xmin_d, const double* xmax_d, int max_iter, double epsimin,
                   double asyinit, double asyincr, double asydecr, void* stream);
int ntg_mma_destroy(ntg_mma* mma);
/* mma_t%update (mma.f90:297-324): x_d (device, n) is replaced by the new
   design; df0dx_d device n; fval host m; dfdx_d device, the reference's
   dfdx(m, n) layout (entry (i, j) at i + m j).  Synchronises the stream. */
int ntg_mma_update(ntg_mma* mma, int iter, double* x_d, const double* df0dx_d, const double* fval,
                   const double* dfdx_d);
/* mma_t%KKT (mma.f90:355-393): max and 2-norm of the KKT residual at x */
int ntg_mma_kkt(ntg_mma* mma, const double* x_d, const double* df0dx_d, const double* fval, const double* dfdx_d,
                double* residumax, double* residunorm);
/* counts[3] (may be NULL): interior-point Newton steps, line-search trials
   and epsilon levels taken so far; the last KKT max and norm */
int ntg_mma_info(const ntg_mma* mma, long long* counts, double* residumax, double* residunorm);

/* ---------------------------------------------------------------------- */
/* field files (Nek5000 binary "#std" format, as Neko's fld_file_t writes  */
/* them for fld_file_output_t; sources/topology_optimization/             */
/* topopt_design.f90:283-286).  Host code; on_device = 1: the field        */
/* pointers are device arrays, 0: host arrays.                             */
/* ---------------------------------------------------------------------- */
/* Write one file: header (wdsize 4 = float32 data, 8 = float64), element
   numbers glb_el (host, 1-based; NULL = 1..nelv), then the fields given (a
   NULL pointer leaves a field out; x, y, z and u, v, w come as triples;
   nscal scalar fields s[0..nscal)) and the per-element min/max block. */
int ntg_fld_write(const char* path, int lx, int64_t nelv, const int64_t* glb_el, double time, int tstep, int wdsize,
                  int on_device, const double* x, const double* y, const double* z, const double* u,
                  const double* v, const double* w, const double* p, const double* t, const double* const* s,
                  int nscal);
/* the "<name>.nek5000" index: filetemplate <name>%01d.f%05d, first step, count */
int ntg_fld_write_index(const char* path, const char* name, int first, int count);
/* header of a field file; rdcode receives the field codes (e.g. "XUPTS02") */
int ntg_fld_info(const char* path, int* lx, int64_t* nelv, int* wdsize, double* time, int* tstep, char* rdcode,
                 int cap);
/* read the fields the file holds into the non-NULL arrays (n = nelv lx^3
   each, element order as stored; element numbers to glb_el if given) */
int ntg_fld_read(const char* path, int on_device, int64_t* glb_el, double* x, double* y, double* z, double* u,
                 double* v, double* w, double* p, double* t, double* const* s, int nscal);

/* ---------------------------------------------------------------------- */
/* masked vector kernels of neko-top, same names and signatures as the     */
/* reference's extern "C" wrappers (math_ext.cu:49-108): device arrays by  */
/* value, sizes and scalars by pointer, 1-based masks, real = double.      */
/* They run on the stream set with ntg_set_glb_queue (default stream 0).  */
/* ---------------------------------------------------------------------- */
void cuda_cadd_mask(void* a, double* c, int* size, int* mask, int* mask_size);
void cuda_invcol1_mask(void* a, int* size, int* mask, int* mask_size);
void cuda_col2_mask(void* a, void* b, int* size, int* mask, int* mask_size);
void cuda_col3_mask(void* a, void* b, void* c, int* size, int* mask, int* mask_size);
void cuda_sub3_mask(void* a, void* b, void* c, int* size, int* mask, int* mask_size);
/* cmult_mask and glsc2_mask exist on the CPU only in the reference
   (math_ext.f90:40-52,99-116); these are their device versions. */
void cuda_cmult_mask(void* a, double* c, int* size, int* mask, int* mask_size);
double cuda_glsc2_mask(void* a, void* b, int* size, int* mask, int* mask_size);
/* the stream the cuda_* kernels use (Neko's glb_cmd_queue) */
void ntg_set_glb_queue(void* stream);

/* Masked dot product sum_{i in mask} a[mask[i]-1] * b[mask[i]-1] that
   allocates nothing.  No counterpart in the reference: it is the variant of
   cuda_glsc2_mask for callers that cannot allocate device memory (device
   memory owned by another allocator or exhausted, or no allocation-driven
   synchronisation allowed mid-solve).  Its scratch is a fixed static device
   array held by every GPU that loads the library until process exit; masks
   longer than 16,777,216 entries are rejected with NTG_ERR_INVALID.  The
   result goes to out_d (device, one double) on `stream`.  The first call on
   each device looks up the scratch address and should come before any
   stream capture.  Calls share the array: calls that overlap on the GPU
   race; order them on one stream. */
int ntg_glsc2_mask_noalloc(const double* a_d, const double* b_d, const int* mask_d, int mask_size,
                           double* out_d, void* stream);

#ifdef __cplusplus
}
#endif
#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#endif /* NTGB300_H */
