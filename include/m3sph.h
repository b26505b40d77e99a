/*
 * m3sph.h - C ABI of the GB300 library for M3TET_SPH's time-step hot path.
 *
 * Plain pointers and sizes only. Array layouts are the reference's MATLAB column-major ones:
 * EL2NOD is 10 x nel uint32 (1-based, element-major: the 10 nodes of element e are contiguous),
 * GCOORD / GCOORD_SPH are 3 x nnod double, velocity vectors are dof-interleaved
 * (dof 3*(node-1)+{1,2,3}, nod2dof.m). Every entry point returns an int status (M3SPH_OK = 0)
 * and never throws; m3sph_last_error() describes the last failure of the calling thread.
 * Host arrays are borrowed for the duration of a call; results go into caller-provided buffers.
 * Handles own their device memory and one CUDA stream; calls on one handle are not reentrant.
 */
#ifndef M3SPH_H
#define M3SPH_H
#include <stdint.h>
#include <stddef.h>

#if defined(__GNUC__)
#define M3SPH_API __attribute__((visibility("default")))
#else
#define M3SPH_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

enum {
  M3SPH_OK = 0,
  M3SPH_ERR_BAD_INPUT = 1,
  M3SPH_ERR_CUDA = 2,
  M3SPH_ERR_NAN = 3,            /* NaN in a right-hand side or solution */
  M3SPH_ERR_NOT_CONVERGED = 4,  /* iteration limit reached above tolerance */
  M3SPH_ERR_NEGATIVE_JACOBIAN = 5,
  M3SPH_ERR_POINT_NOT_FOUND = 6,
  M3SPH_ERR_NO_DEVICE = 7
};

/* element classes (tetmesh_p1_to_p2_sph.m:183-189) */
enum { M3SPH_OUT_CONE_NO_CROSS_2PI = 0, M3SPH_OUT_CONE_CROSS_2PI = 1,
       M3SPH_IN_CONE_NO_ISO = 2, M3SPH_IN_CONE_ISO = 3 };

/* One multigrid level of the reference MESH struct (init_mesh_curved_p.m:182-217).
 * Level 0 is the finest (MESH.EL2NOD{1}); level nmg-1 the coarsest. The nodes of a coarse
 * level are the first nnod nodes of the next finer level, and the children of coarse element
 * e (1-based) are fine elements 8(e-1)+1 .. 8e (tetmesh_p2_to_p1.m). */
typedef struct m3sph_level {
  int32_t nel;                  /* number of P2 tetrahedra */
  int32_t nnod;                 /* number of P2 nodes */
  int32_t nvnod;                /* number of vertex (pressure) nodes */
  const uint32_t *EL2NOD;       /* 10 x nel, 1-based */
  const uint8_t *isplit;        /* nel, split (1..3) that made the next finer level; NULL on level 0 */
  /* geometry: required on level 0 only (NULL elsewhere) */
  const double *GCOORD;         /* 3 x nnod Cartesian */
  const double *GCOORD_SPH;     /* 3 x nnod (theta, phi, r) */
  const uint8_t *elclass;       /* nel, M3SPH_* element class */
  int32_t niso;                 /* number of in-cone isoparametric elements */
  const uint32_t *els_iso;      /* niso, 1-based element ids */
  const double *cubic_sph_rot;  /* niso x 3 x 20 (theta,phi,r) of the 20 cubic nodes, X-90 frame */
} m3sph_level;

typedef struct m3sph_mesh m3sph_mesh;   /* opaque: device-resident MESH + MG hierarchy */

/* Semi-Lagrangian options (OPTS_SLM, default_numerics_M3TET.m:141-158). */
typedef struct m3sph_slm_opts {
  int32_t method_BT;      /* 1: PC2 predictor-corrector (the reference default); 2: RK4 over 3
                             substeps (the reference's RK4 is an error stub, advect3d_slm_p_sph.m:103) */
  int32_t method_interp;  /* 0: 'quadratic' (interp3d_tet), 1: 'cubic' (interp3d_cubic_p) */
  int32_t monotonic;      /* clamp to the element's nodal min/max */
  int32_t method_wght;    /* cubic gradient weights: 0 'ones', 1 'dist' */
  double r_cmb, r_surf;   /* MESH.r_cmb, MESH.r_surf */
} m3sph_slm_opts;

/* Point-location counters: points placed by the walk, points that several elements contain
 * (within 1e-10 in barycentric coordinates) resolved by the tie rule, points in frame gaps placed
 * with a grown tolerance, brute-force placements, lost points, and the ties that the reference
 * rejects with error('no good') (tsearch2_sph.m:387-392: cross-frame, no isoparametric element, not
 * at a shared vertex), which are resolved by the largest id. */
typedef struct m3sph_locate_info {
  int32_t npt, nwalk, nties, ngap, nbrute, nlost, nambig;
} m3sph_locate_info;

/* Physical parameters used by the element operator (PHYSICS, NUMSCALE fields). */
typedef struct m3sph_physics {
  double g;          /* PHYSICS.g (e.g. -9.81) */
  double Bscale;     /* NUMSCALE.Bscale */
  double Dens0;      /* NUMSCALE.Dens0 */
  double minVisc;    /* PHYSICS.minVisc (<=0: no clamp) */
  double maxVisc;    /* PHYSICS.maxVisc (<=0: no clamp) */
} m3sph_physics;

/* Solver options (flow3d_patera_mg_sph_p.m:70-129, mgpcg_solver_p.m:620-724). */
typedef struct m3sph_opts {
  double rtol_Pat;      /* 1e-4 in the reference */
  double rtol_U;        /* 5e-3 */
  int32_t itmax_Pat;    /* 120 */
  int32_t itmin_Pat;    /* 3 */
  int32_t itmax_U;      /* 20 */
  int32_t precision;    /* 0: plain FP64 everywhere; 1: FP32 V-cycle inside FP64 outer CG */
  int32_t smoother;     /* 0: weighted Jacobi; 1: learned element smoother on the 2 finest levels */
  double target_rel_residual; /* >0: keep iterating Patera until the coupled FP64 residual is below */
} m3sph_opts;

typedef struct m3sph_info {
  int32_t itPat;            /* Patera iterations */
  int32_t nitU;             /* velocity MG-PCG iterations (initial + restarts + final) */
  int32_t nitZ;             /* MG-PCG iterations inside Patera */
  int32_t nvcycle;          /* V-cycles applied */
  double norm_rP;           /* final pressure residual (normdf) */
  double rel_residual;      /* coupled FP64 relative residual on free dofs, pressure mean removed */
  double t_setup_ms;        /* element matrices, Galerkin, coarse factorisation */
  double t_iter_ms;         /* Patera + MG-PCG iterations */
  int32_t smoother_fallbacks; /* times the learned smoother was replaced by Jacobi */
  int32_t status;
} m3sph_info;

M3SPH_API const char *m3sph_last_error(void);
M3SPH_API int m3sph_device_count(int *count);

/* Build the device-resident mesh + MG hierarchy (init_mesh_curved_p / create_multigrid_meshes_3d_sph
 * outputs). Computes per-node rotations (make_rotation_matrix.m), element colours, and the
 * intermesh transfer operators (intermesh_transfer_matrix.m:1-62). */
M3SPH_API int m3sph_mesh_create(int32_t nmg, const m3sph_level *levels, int32_t device, m3sph_mesh **out);
M3SPH_API int m3sph_mesh_destroy(m3sph_mesh *mesh);
/* number of element colours of level `img` (0-based) */
M3SPH_API int m3sph_mesh_ncolors(const m3sph_mesh *mesh, int32_t img, int32_t *ncolors);

/* Set the velocity boundary conditions in the rotated (theta,phi,r) frame (UBC.ifix/vfix,
 * 1-based dof ids as in bc_sph.m) and the nodal viscosity / density (VAR.Visc, VAR.Dens,
 * nnod each; only vertex values are used, calc_element_visc.m:5-7). Recomputes the element
 * operator (assembly_stokes_sph_3d_double_jacobian.m), the Galerkin coarse operators
 * (restrict_stiffmat.m) and the coarse factorisation (cholesky_factorization.m). */
M3SPH_API int m3sph_stokes_setup(m3sph_mesh *mesh, const double *Visc, const double *Dens, const int32_t *ifix,
                       const double *vfix, int32_t nfix, const m3sph_physics *phys, int32_t precision);
/* Replaces the UBC that update_vel_bc (update_vel_bc.m:84-150) hands to the next flow3d_patera_sph
 * call in a GPlates-driven loop: new prescribed values vfix on the fixed dofs ifix (1-based, any
 * order) of the last m3sph_stokes_setup. The dof set must equal the set-up's (M3SPH_ERR_BAD_INPUT
 * otherwise: a new set needs m3sph_stokes_setup). The next operator rebuild (m3sph_time_step,
 * m3sph_stokes_step_device, or m3sph_stokes_solve, which rebuilds when values changed) uses them. */
M3SPH_API int m3sph_stokes_set_vel_bc(m3sph_mesh *mesh, const int32_t *ifix, const double *vfix, int32_t nfix);

/* Replaces flow3d_patera_mg_sph_p (flow3d_patera_mg_sph_p.m:1-780): Patera pressure CG around
 * MG-PCG. P (nvnod) is the initial pressure on input and the solution on output; U_xyz (3*nnod,
 * dof-interleaved Cartesian) receives the velocity. */
M3SPH_API int m3sph_stokes_solve(m3sph_mesh *mesh, double *U_xyz, double *P, const m3sph_opts *opts,
                       m3sph_info *info);

/* One device-resident hot-path step: rebuild the operator from the resident Visc/Dens/BCs of the
 * last m3sph_stokes_setup (assembly + restrict_stiffmat + coarse factorisation) and run the
 * Patera solve from P = 0; U and P stay on the device (read them with m3sph_solution). No
 * counterpart call in the reference: flow3d_patera_mg_sph_p always starts from host arrays. */
M3SPH_API int m3sph_stokes_step_device(m3sph_mesh *mesh, const m3sph_opts *opts, m3sph_info *info);
/* Copy the device-resident solution of the last solve: U_xyz (3*nnod) and P (nvnod). */
M3SPH_API int m3sph_solution(m3sph_mesh *mesh, double *U_xyz, double *P);
/* Replaces calculate_dt (calculate_dt.m:40-52) on the device-resident velocity of the last solve
 * (the VAR.Ux/Uy/Uz that flow3d_patera_sph returns): a device max-reduction of |Ux|, |Uy|, |Uz|,
 * then dt_adv = dt_adv_limit * min(Lx/max|Ux|, Ly/max|Uy|, Lz/max|Uz|) with MESH.Lx/Ly/Lz the extents
 * of the finest mesh (init_mesh_curved_p.m:264-272), dt = min(dtmax, dt_adv); a zero velocity gives
 * dt = dtmax and dt_adv = 0. dt_adv may be NULL. */
M3SPH_API int m3sph_calculate_dt(m3sph_mesh *mesh, double dt_adv_limit, double dtmax, double *dt, double *dt_adv);
/* The CUDA stream (cudaStream_t) the handle launches its kernels on. */
M3SPH_API int m3sph_stream(m3sph_mesh *mesh, void **stream);

/* Rock properties of rock_prop (rock_prop.m:5-66). A cut-off that is NaN is not applied. */
typedef struct m3sph_rock_params {
  double Visc0;      /* PHYSICS.Visc: reference viscosity */
  double Dens0;      /* PHYSICS.Dens: reference density */
  double T_ref;      /* PHYSICS.T_ref (degC) */
  double alpha;      /* PHYSICS.alpha: thermal expansivity */
  double Ea;         /* PHYSICS.Ea (J/mol; 0: no Arrhenius factor; 0 < Ea < 1000 is rejected as kJ/mol) */
  double Va;         /* PHYSICS.Va (m^3/mol; 0: no pressure factor) */
  double g;          /* PHYSICS.g */
  double L0;         /* NUMSCALE.L0: metres per mesh length unit */
  double a_UM2LM;    /* PHYSICS.a_UM2LM: cap of the pressure factor (<= 0: none) */
  double minDens, maxDens, minVisc, maxVisc;
} m3sph_rock_params;

/* Replaces rock_prop (rock_prop.m:5-66): nodal Visc and Dens (nnod each) from T (nnod):
 * Dens = Dens0 (1 - alpha (T - T_ref)); Arrhenius factor exp(Ea/(R T0) (T0/T - 1)) in Kelvin,
 * clamped to [1e-8, 1e8]; pressure factor exp(|g Dens0 L0 depth| Va / (R T0)) with depth below the
 * outermost node; Visc = Visc0 times the smaller of (Arrhenius x pressure, Arrhenius x a_UM2LM). */
M3SPH_API int m3sph_rock_prop(m3sph_mesh *mesh, const m3sph_rock_params *p, const double *T, double *Visc,
                              double *Dens);

/* Thermal diffusion of diffusion3d_p (diffusion3d_p.m:1-121) with the reference's default element
 * options (default_numerics_M3TET.m:94-121): linear elements on the 8-child split of every P2
 * tetrahedron (tetmesh_p2_to_p1), double-Jacobian integrals with 4 points per element
 * (assembly_diffusion_3d_double_jacobian.m), lumped capacity, theta scheme, the temperature of
 * nodes ifix (1-based, TBC.ifix) prescribed to vfix, Jacobi-preconditioned CG (pcg_solver_p.m). */
typedef struct m3sph_diffusion_opts {
  double kappa;       /* PHYSICS.kappa (0: diffusion is skipped) */
  double theta;       /* OPTS_D.theta: 1 implicit Euler (the default), 0.5 Crank-Nicolson */
  double tol;         /* OPTS_D.tol, relative to the initial residual (<= 0: 1e-8) */
  int32_t itmax;      /* OPTS_D.itmax (<= 0: 500) */
  double theta_cone;  /* MESH.theta_cone in degrees for the split elements' classes (<= 0: 45) */
} m3sph_diffusion_opts;
M3SPH_API int m3sph_diffusion_setup(m3sph_mesh *mesh, const m3sph_diffusion_opts *opts, const int32_t *ifix,
                                    const double *vfix, int32_t nfix);
/* Replaces diffusion3d_p(T,kappa,MESH,COMM,SETTINGS,TBC,dt): T (nnod) diffused over dt in place;
 * *nit receives the CG iterations (may be NULL). */
M3SPH_API int m3sph_diffusion3d(m3sph_mesh *mesh, double *T, double dt, int32_t *nit);

/* One time step of the reference's loop (M3TET_SPH_SOUTH_ATLANTIC_PLUME.m:213-296) on device-
 * resident fields: rock_prop (optional) -> flow3d_patera_sph (operator rebuild from the resident
 * viscosity/density and the boundary conditions of the last m3sph_stokes_setup, Patera solve
 * warm-started from the previous step's pressure) -> calculate_dt -> thermal_advdiff_3d_p of the
 * resident temperature: optional diffusion half step, advect3d_slm_p_sph in the new velocity (search
 * guesses carried between steps as WS_SLM), optional diffusion half step.
 * No counterpart call in the reference, whose loop calls the functions one by one from MATLAB. */
typedef struct m3sph_step_opts {
  m3sph_opts stokes;          /* solver options (precision must match the set-up's) */
  m3sph_slm_opts slm;         /* advection options */
  int32_t rock_prop;          /* 1: Visc, Dens from the resident T by rock_prop before the solve */
  m3sph_rock_params rock;
  double dt_adv_limit;        /* SETTINGS.dt_adv_limit (calculate_dt.m) */
  double dtmax;               /* SETTINGS.dtmax */
  int32_t diffusion;          /* 1: diffusion half steps of dt/2 before and after the advection
                                 (thermal_advdiff_3d_p.m:13-18,46-51) with m3sph_diffusion_setup's state */
} m3sph_step_opts;

typedef struct m3sph_step_info {
  m3sph_info stokes;          /* the Patera solve of this step */
  m3sph_locate_info locate;   /* point location of the advection */
  double dt, dt_adv;          /* calculate_dt outputs */
  double time;                /* model time after the step */
  double t_rock_ms, t_stokes_ms, t_dt_ms, t_advect_ms, t_total_ms;
  int32_t status;
  double t_diffusion_ms;      /* both diffusion half steps (inside t_advect_ms) */
  int32_t diffusion_its;      /* CG iterations of both half steps */
} m3sph_step_info;

/* Upload the temperature T (nnod) that the time steps advect (and restart the step counter, the
 * model time and the advection search guesses); read it back. */
M3SPH_API int m3sph_set_temperature(m3sph_mesh *mesh, const double *T, double time);
M3SPH_API int m3sph_get_temperature(m3sph_mesh *mesh, double *T);
M3SPH_API int m3sph_time_step(m3sph_mesh *mesh, const m3sph_step_opts *opts, m3sph_step_info *info);
/* The resident nodal viscosity and density (VAR.Visc, VAR.Dens: nnod each; either may be NULL), for
 * output and restart files (write_output_file.m, write_restart_file.m). */
M3SPH_API int m3sph_get_properties(m3sph_mesh *mesh, double *Visc, double *Dens);
/* Resume from a restart file: the pressure (nvnod) the next solve or time step starts from. */
M3SPH_API int m3sph_set_pressure(m3sph_mesh *mesh, const double *P);

/* Learned element smoother (no counterpart in the reference: M3TET_SPH smooths with weighted
 * Jacobi only). A 52-128-30 MLP (BF16 tensor cores, FP32 accumulation) replaces Jacobi sweeps on
 * the two finest levels when m3sph_opts.smoother = 1 and trained weights are loaded; the outer
 * FP64 CG falls back to Jacobi when its contraction factor exceeds 0.95.
 * Parameters are a flat FP32 vector of m3sph_ml_nparam() values: W1 [128][64] (input columns
 * >= 52 are zero), b1 [128], W2 [32][128] (rows >= 30 zero), b2 [32]. */
M3SPH_API int m3sph_ml_nparam(int32_t *n);
M3SPH_API int m3sph_ml_set_params(m3sph_mesh *mesh, const float *params, int32_t trained);
M3SPH_API int m3sph_ml_get_params(m3sph_mesh *mesh, float *params);
/* Training data: reserve room for `capacity` samples, then append (local residual, local error)
 * pairs of the current operator: for each of n_iterates seeded white-noise errors e on the free
 * dofs, r = K e with the outer (FP64-accurate) operator, and every `stride`-th element contributes
 * the features of r and its local values of e. */
M3SPH_API int m3sph_ml_reserve(m3sph_mesh *mesh, int64_t capacity);
M3SPH_API int m3sph_ml_collect(m3sph_mesh *mesh, uint64_t seed, int32_t n_iterates, int32_t stride, int64_t *count);
/* Append the pairs of caller vectors: residual r and error e (3*nnod each, rotated frame, fixed dofs
 * ignored), every `stride`-th element from `offset` -- e.g. the residuals and errors of the iterates
 * of a plain multigrid solve. */
M3SPH_API int m3sph_ml_add_pairs(m3sph_mesh *mesh, const double *r, const double *e, int32_t stride, int32_t offset,
                                 int64_t *count);
/* One Adam epoch over the shuffled samples (batch a multiple of 64); mse = mean squared error. */
M3SPH_API int m3sph_ml_train_epoch(m3sph_mesh *mesh, int32_t batch, float lr, uint64_t seed, double *mse);
/* Gradient of the MSE loss (flat layout, same as the parameters) and forward outputs on caller
 * rows X (n x 64 FP32, rounded to BF16), targets T (n x 32): for checks against a CPU autograd. */
M3SPH_API int m3sph_ml_gradients(m3sph_mesh *mesh, const float *X, const float *T, int32_t n, float *grad, double *loss);
M3SPH_API int m3sph_ml_forward(m3sph_mesh *mesh, const float *X, int32_t n, float *Y);
/* One learned sweep of level img (0 or 1) in FP32 as the V-cycle runs it: d += the partition-of-
 * unity sum of the network's element corrections for the residual r - kd (kd may be NULL: r).
 * Host vectors of 3*nnod(img); needs a set-up with precision 1 and parameters loaded. */
/* Inverse diagonal of the FP32 level-img operator (host, ndof of the level; 0 on fixed dofs): the
 * scaling of the weighted-Jacobi sweeps (mgpcg_solver_p.m:397-437). */
M3SPH_API int m3sph_level_inverse_diag32(m3sph_mesh *mesh, int32_t img, float *dinv);
/* Inputs of the learned smoother on level img (0 or 1) for a Jacobi-scaled residual z (host, FP32,
 * 3 nnod of that level): X (host, nel x 52, original element order) = the 30 local values of z
 * divided by their norm, the 10 standardised log-viscosities and the 12 geometry factors;
 * s_norm (host, nel) = the norms. No reference counterpart (the learned part is new); used to
 * check the fused sweep's features against a CPU restatement. */
M3SPH_API int m3sph_ml_features(m3sph_mesh *mesh, int32_t img, const float *z, float *X, float *s_norm);
M3SPH_API int m3sph_ml_sweep32(m3sph_mesh *mesh, int32_t img, const float *r, const float *kd, float *d);

/* Kernel-variant switches for measurement and tests (per process, results equal to rounding):
 * "stream_apply" (streamed finest-level FP32 operator, default 1; 0: one launch per colour),
 * "stream_outer" (streamed double-float / FP64 finest-level operators, default 1),
 * "stream_outer_variant" (warp layout of the double-float kernel, 0-7, default 4),
 * "split_apply" (4-warp per-colour kernels when streaming is off, default 1), "graphs" (CUDA-graph
 * replay of MG-PCG iterations, default 1), "df_outer" (double-float outer operator on the mixed
 * path, default 1), "ml_schedule" (learned smoothing on the two finest levels: 0 learned-Jacobi-
 * learned, 1 one learned sweep per side (default), 3 learned + one Jacobi sweep per side; 2 one
 * learned sweep per side on the finest level only; per handle), "fp32_operator" (finest-level FP32
 * V-cycle operator: 1 partially assembled, default; 0 streamed stored matrices; takes effect at the
 * next set-up), "ml_omega_pct" (relaxation weight of the learned correction
 * in percent, 10-300, default 100; per handle), "ml_infer" (learned sweep kernels: 1 fused tcgen05 sweep, default;
 * 0 WMMA tile kernel), "stream_f32_variant" (slot-ring depth / gather warps of the streamed FP32
 * kernel, 0-3, default 0), "coarse_f64_direct_max" (plain FP64 path: coarsest levels up to this many
 * dofs get an FP64 dense inverse, larger ones the FP32 inverse refined against the FP64 coarsest
 * operator in every coarse solve; default 6000; takes effect at the next set-up), "coarse_refine_sweeps"
 * (refinement steps of that solve, default 3). */
M3SPH_API int m3sph_set_option(m3sph_mesh *mesh, const char *name, int32_t value);
/* Cumulative number of CUDA kernels this library has launched (all handles). */
M3SPH_API int m3sph_launch_count(unsigned long long *count);
/* Operator benchmark: nrep device-resident applications of the level-`img` operator in FP64
 * (precision 0), FP32 (1) or, on the finest level, double-float (2); returns the mean time per
 * full application. */
M3SPH_API int m3sph_apply_timing(m3sph_mesh *mesh, int32_t img, int32_t precision, int32_t nrep, double *ms_per_apply);

/* Replaces tsearch2_sph + local_coords_3d_sph (tsearch2_sph.m:1-424, local_coords_3d_sph.m:28-147):
 * element (1-based, 0 = not found) and own-frame local coordinates (npt x 3) of points given as
 * (theta,phi,r) triplets (npt x 3). els_guess (1-based, may be NULL) seeds the neighbour walk. */
M3SPH_API int m3sph_tsearch_sph(m3sph_mesh *mesh, const double *thphr, int32_t npt, const int32_t *els_guess,
                                int32_t *els_out, double *lc_out, m3sph_locate_info *info);
/* Location benchmark: the points (npt x 3, as for m3sph_tsearch_sph) are uploaded once, then nrep
 * device-resident locations (walk, ring resolution, brute force, counts) are timed with CUDA events;
 * *ms = mean time per location, info = counts of the last one. */
M3SPH_API int m3sph_locate_timing(m3sph_mesh *mesh, const double *thphr, int32_t npt, int32_t nrep, double *ms,
                                  m3sph_locate_info *info);
/* Replaces interp3d_tet (interp3d_tet.m:39-69): V is nnod x nvar (nvar <= 3), Vi npt x nvar.
 * els are 1-based ids of finest-level elements; an id outside 1..nel is M3SPH_ERR_BAD_INPUT (the
 * reference's indexing error). npt = 0 does nothing. The same holds for m3sph_interp3d_cubic. */
M3SPH_API int m3sph_interp3d_tet(m3sph_mesh *mesh, const int32_t *els, const double *lc, int32_t npt,
                                 const double *V, int32_t nvar, int32_t monotonic, double *Vi);
/* Replaces interp3d_cubic_p (interp3d_cubic_p.m:80-382) for one nodal field V (nnod). */
M3SPH_API int m3sph_interp3d_cubic(m3sph_mesh *mesh, const int32_t *els, const double *lc, int32_t npt,
                                   const double *V, int32_t monotonic, int32_t method_wght, double *Vi);
/* Allocation-free variant of m3sph_interp3d_cubic (no counterpart in the reference). For callers
 * that cannot allocate device memory while they run: a host that owns all device memory through
 * its own pool, a time loop with a fixed memory footprint, or a host with work in flight on other
 * streams that a cudaMalloc / cudaFree (which may synchronise the device) would stall.
 * els (npt, 1-based), lc (npt x 3), V (nnod) and Vi (npt) must be memory the device can access
 * (device, managed or mapped pinned host memory), with the inputs complete before the call; the
 * work runs on the handle's stream (m3sph_stream), which is synchronised before returning. The ids
 * are not read on the host: a point whose id is outside 1..nel gets NaN.
 * Scratch lives in one fixed 8 MiB array per device that every call shares (7 values per element
 * + 4 per vertex, about 120k elements of a spherical-shell mesh; larger meshes are rejected with
 * M3SPH_ERR_BAD_INPUT). The array's device address is looked up, and this entry point's kernels
 * are loaded, when the mesh handle is created (m3sph_mesh_create), so under CUDA's lazy module
 * loading the array is committed at start-up and not inside a call. Calls that overlap on the GPU
 * (two handles on two threads) race on the shared scratch. It calls no cudaMalloc / cudaFree. It
 * synchronises the handle's stream before returning, so it cannot be called while that stream is
 * being captured into a CUDA graph. */
M3SPH_API int m3sph_interp3d_cubic_noalloc(m3sph_mesh *mesh, const int32_t *els, const double *lc, int32_t npt,
                                           const double *V, int32_t monotonic, int32_t method_wght, double *Vi);
/* Replaces advect3d_slm_p_sph (advect3d_slm_p_sph.m:1-139): Ux,Uy,Uz Cartesian nodal velocity,
 * T (nnod) advected in place over dt. els_BT / els_INTERP (nnod, 1-based, 0 = unknown) are the
 * WS_SLM search guesses, updated on return (predictor and departure elements). */
M3SPH_API int m3sph_advect_slm(m3sph_mesh *mesh, const double *Ux, const double *Uy, const double *Uz, double *T,
                               double dt, const m3sph_slm_opts *opts, int32_t *els_BT, int32_t *els_INTERP,
                               m3sph_locate_info *info);

/* Replaces one mgpcg_solver_p call (mgpcg_solver_p.m:1-743) on the current operator: solves
 * K1 x = b on the free dofs of the rotated frame (b, x: 3*nnod, fixed dofs ignored / zero).
 * tol is absolute on normdf(r) if is_abs_tol, else relative to the initial residual. */
M3SPH_API int m3sph_mgpcg(m3sph_mesh *mesh, const double *b, double *x, double tol, int32_t is_abs_tol,
                int32_t itmax, int32_t *itCG, double *rrms_final);

/* Operator-level entry points (replace MUTILS spmv on the assembled matrices):
 * y = K1 x with K1 = RR' K RR on free dofs (fixed dofs give 0), x,y 3*nnod rotated frame. */
M3SPH_API int m3sph_stokes_apply(m3sph_mesh *mesh, const double *x, double *y);
/* y = GG q (3*nnod <- nvnod, rotated frame) and s = GG' z (nvnod <- 3*nnod) */
M3SPH_API int m3sph_grad_apply(m3sph_mesh *mesh, const double *q, double *y);
M3SPH_API int m3sph_div_apply(m3sph_mesh *mesh, const double *z, double *s);
/* Buoyancy force vector Fb = RR' Fb_xyz (3*nnod) */
M3SPH_API int m3sph_force_vector(m3sph_mesh *mesh, double *Fb);
/* Copy out the element matrices of level 0 in the rotated, BC-masked frame:
 * K: nel x 900 (full 30x30, row-major), G: nel x 120 (30x4 row-major), M: nel x 16. */
M3SPH_API int m3sph_element_matrices(m3sph_mesh *mesh, double *K, double *G, double *M);
/* y = KK{img} x on level img (0-based, img>=1: Galerkin coarse operator), vectors 3*nnod(img) */
M3SPH_API int m3sph_level_apply(m3sph_mesh *mesh, int32_t img, const double *x, double *y);
/* The FP32 operator of level img as used inside the V-cycle (streamed element apply on the finest
 * level, assembled blocks on coarse levels); needs a set-up with precision 1. */
M3SPH_API int m3sph_level_apply32(m3sph_mesh *mesh, int32_t img, const float *x, float *y);
/* Replaces intermesh_transfer_matrix(GCOORD,EL2NOD,GCOORD_c,EL2NOD_c,1) (intermesh_transfer_matrix.m:
 * 1-62) for levels img (fine) and img+1: the scalar Ic2f (nnod(img) x nnod(img+1)) as 1-based
 * (row, col, value) triplets of the handle's transfer operator, ready for MATLAB's sparse(). Call
 * with rows/cols/vals NULL to get *nnz, then with arrays of that size. The vector form for ndof = 3
 * is kron(Ic2f, eye(3)). */
M3SPH_API int m3sph_transfer_matrix(const m3sph_mesh *mesh, int32_t img, int64_t *nnz, int32_t *rows, int32_t *cols,
                                    double *vals);
/* Ic2f{img} (intermesh_transfer_matrix): prolong x_c (3*nnod(img+1)) -> x_f (3*nnod(img)) and
 * restrict r_f -> r_c with Ic2f' (free-dof masked as in restrict_stiffmat.m:94-96). */
M3SPH_API int m3sph_prolong(m3sph_mesh *mesh, int32_t img, const double *xc, double *xf);
M3SPH_API int m3sph_restrict(m3sph_mesh *mesh, int32_t img, const double *rf, double *rc);
/* One V-cycle (MG_V_cycle_v2, mgpcg_solver_p.m:388-596) in the setup precision: d = B r. */
M3SPH_API int m3sph_vcycle(m3sph_mesh *mesh, const double *r, double *d);

#ifdef __cplusplus
}
#endif
#endif /* M3SPH_H */
