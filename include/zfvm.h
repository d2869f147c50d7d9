/*
 * zfvm.h -- C ABI of the GB300 rate-of-change / SSP-RK solver.
 *
 * Every entry point returns an int status (ZFVM_OK = 0).  The reference
 * reports failures through LOG_ERR (log + abort); here a non-zero status is
 * returned instead and zfvm_last_error() gives the message of the calling
 * thread's last failure.  A mesh or solver handle is externally synchronised:
 * one host thread at a time, like the reference's non-re-entrant objects
 * (LocalReconstruction keeps mutable caches).  Distinct handles may be driven
 * from distinct threads; each solver owns one CUDA stream.
 *
 * Layouts at this boundary are the reference's: cell-major AoS conserved
 * variables (rho, m1, m2, m3, E) as in GridVariables
 * (model/grid_variables_decl.hpp:17-36); vertex coordinates n x 3 and
 * cell->vertex indices n x (n_dims + 1) as in the .msh.h5 schema
 * (grid/grid.cpp:889-901).
 */
#ifndef ZFVM_H
#define ZFVM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum zfvm_status {
  ZFVM_OK = 0,
  ZFVM_EINVAL = 1,        /* bad argument or unsupported configuration      */
  ZFVM_ENOMEM = 2,        /* host or device allocation failed               */
  ZFVM_ENONPHYSICAL = 3,  /* rho <= 0, E <= 0 or a non-finite state         */
  ZFVM_ENEWTON = 4,       /* local equilibrium solve did not converge       */
  ZFVM_ETIMEDOUT = 5,     /* a host wait passed its deadline                */
  ZFVM_ECUDA = 6,         /* CUDA runtime error                             */
  ZFVM_ESETUP = 7         /* mesh / stencil set-up failed                   */
};

#define ZFVM_MAX_STENCILS 5
#define ZFVM_MAX_L2G 40
#define ZFVM_MAX_STENCIL_SIZE 24

typedef struct zfvm_rawmesh zfvm_rawmesh;
typedef struct zfvm_mesh zfvm_mesh;
typedef struct zfvm_solver zfvm_solver;

/* ---- meshes ---------------------------------------------------------------
 * Synthetic generators (the reference loads gmsh meshes, grid/grid.cpp:907-922).
 * kind 0: periodic unit square, iparams = {n, halo}, dparams = {jitter}
 * kind 1: disk, iparams = {n_rings}, dparams = {radius, jitter}
 * kind 2: unit cube of tetrahedra, iparams = {n}, dparams = {jitter}
 * The mesh is renumbered along a Hilbert curve when `renumber` is non-zero
 * (src/renumber_grid.cpp:46-135). */
int zfvm_rawmesh_generate(int32_t kind, const int64_t *iparams, const double *dparams,
                          uint64_t seed, int32_t renumber, zfvm_rawmesh **out);
int zfvm_rawmesh_sizes(const zfvm_rawmesh *m, int32_t *n_dims, int64_t *n_vertices,
                       int64_t *n_cells, int32_t *has_ghosts);
/* Copies vertices (n_vertices x 3), vertex_indices (n_cells x (n_dims+1)),
 * ghost mask (n_cells, may be NULL) and periodic sources (n_cells, may be NULL). */
int zfvm_rawmesh_copy(const zfvm_rawmesh *m, double *vertices, int64_t *vertex_indices,
                      uint8_t *ghost, int64_t *source);
int zfvm_rawmesh_destroy(zfvm_rawmesh *m);

typedef struct {
  int32_t n_dims;                 /* 2 (triangles) or 3 (tetrahedra)                 */
  int64_t n_vertices;
  int64_t n_cells;
  const double *vertices;         /* n_vertices x 3                                   */
  const int64_t *vertex_indices;  /* n_cells x (n_dims + 1)                           */
  const uint8_t *ghost;           /* optional ghost-cell mask (grid.cpp:1122-1137)    */
  const int64_t *source;          /* optional periodic source of every ghost cell     */
  int32_t quad_edge;              /* quadrature.edge   (numerical_experiment.cpp:193) */
  int32_t quad_volume;            /* quadrature.volume                                */
  int32_t quad_moments;           /* quadrature.moments                               */
  int32_t n_stencils;             /* reconstruction.orders / biases / overfit_factors */
  int32_t orders[ZFVM_MAX_STENCILS];
  int32_t biased[ZFVM_MAX_STENCILS];
  double overfit[ZFVM_MAX_STENCILS];
} zfvm_mesh_desc;

/* Geometry, stencil families and least-squares pseudo-inverses
 * (Grid::Grid grid.cpp:651-723, compute_stencil_families stencil_family.cpp:99-118,
 * LSQSolver lsq_solver.cpp:104-112).  Host only; device arrays are made by
 * zfvm_solver_create. */
int zfvm_mesh_create(const zfvm_mesh_desc *desc, zfvm_mesh **out);
int zfvm_mesh_destroy(zfvm_mesh *m);

typedef struct {
  int32_t n_dims;
  int64_t n_cells, n_interior_cells, n_edges, n_interior_edges;
  int32_t n_cell_qp, n_face_qp, n_moments;
  double min_inradius, max_circum_radius, total_volume;
  /* wall time of zfvm_mesh_create's phases: geometry and quadrature, stencil
   * families, least-squares pseudo-inverses */
  double setup_geometry_s, setup_stencils_s, setup_lsq_s;
} zfvm_mesh_info;
int zfvm_mesh_get_info(const zfvm_mesh *m, zfvm_mesh_info *info);

/* Export the stencil families: n_stencils[n], k_high[n], n_l2g[n],
 * l2g[n * ZFVM_MAX_L2G], order/size/bias[n * ZFVM_MAX_STENCILS],
 * local[n * ZFVM_MAX_STENCILS * ZFVM_MAX_STENCIL_SIZE]. */
int zfvm_mesh_get_stencils(const zfvm_mesh *m, int8_t *n_stencils, int8_t *k_high, int8_t *n_l2g,
                           int32_t *l2g, int8_t *order, int8_t *size, int8_t *bias, int8_t *local);
/* Export the pseudo-inverse of stencil k of cell i, (cols x rows) row-major. */
int zfvm_mesh_get_pinv(const zfvm_mesh *m, int64_t cell, int32_t k, double *P, int32_t *rows,
                       int32_t *cols);
/* Geometry export: volumes[n], inradii[n], centers[n x 3], flags[n]. */
int zfvm_mesh_get_geometry(const zfvm_mesh *m, double *volumes, double *inradii, double *centers,
                           uint8_t *flags);
/* Connectivity export, n_cells x (n_dims + 1) each: the neighbour across local
 * face k (-1 on the boundary) and the face's number (Grid::neighbours,
 * Grid::edge_indices, grid/grid.cpp:385-413: interior faces first, numbered in
 * the order of their lower cell, then boundary faces in cell order).  Local
 * face k of a triangle joins its vertices k and k+1 (mod 3), after the
 * counter-clockwise reordering of grid/grid.cpp:152-203.  Either pointer may be
 * null. */
int zfvm_mesh_get_connectivity(const zfvm_mesh *m, int64_t *neighbours, int64_t *edge_indices);
/* Face export, n_edges entries each: left and right cell (right = -1 on the
 * boundary; left < right inside), the unit normal out of the left cell
 * (n_edges x 3) and the face's area (length in 2D).  Any pointer may be null. */
int zfvm_mesh_get_faces(const zfvm_mesh *m, int64_t *left, int64_t *right, double *normals, double *areas);

/* ---- initial data (cell averages with the volume quadrature) ---------------
 * kind 0: isentropic vortex (2D) / vortex tube along z (3D);
 *         dparams = {gamma, beta, x0, y0, length, rho_inf, u_inf, v_inf, p_inf}
 * kind 1: polytrope rho = rho_c - k r^2 / 4 ... for gamma = 2, K and phi = k r^2/2,
 *         plus a Gaussian pressure bump;
 *         dparams = {gamma, K, rho_c, k_phi, amplitude, width, x0, y0}
 * kind 2: isentropic polytrope in one of the radial potentials, h(x) = h_c + phi(0) - phi(x)
 *         with h_c the enthalpy of rho_c (for POLYTROPE_RADIAL and gamma = 2 the
 *         Lane-Emden profile rho = rho_c sin(a r) / (a r)), plus the same bump;
 *         dparams = {gamma, K, rho_c, amplitude, width, x0, y0, zfvm_gravity kind,
 *                    gravity_strength, gravity_params[0..4]} (no RADIAL_TABLE)
 * Output: n_cells x 5 AoS. */
int zfvm_initial_conditions(const zfvm_mesh *m, int32_t kind, const double *dparams,
                            double *cvars);

/* ---- scheme ---------------------------------------------------------------- */
enum zfvm_flux { ZFVM_FLUX_HLLC = 0, ZFVM_FLUX_RUSANOV = 1 };
enum zfvm_equilibrium { ZFVM_EQ_NONE = 0, ZFVM_EQ_ISENTROPIC = 1 };
/* Radial potentials phi(|x|) (model/gravity_decl.hpp, gravity_impl.hpp; built by
 * make_gravity, model/euler_factory.cpp:60-121):
 *   CONSTANT_RADIAL        ConstantGravityRadial: phi = g r (gravity_strength g)
 *   HARMONIC_RADIAL        phi = k r^2 / 2 (gravity_strength k; no counterpart in the reference)
 *   POLYTROPE_RADIAL       PolytropeGravityRadial(rhoC, K, G): gravity_params {rhoC, K, G}
 *   POLYTROPE_JUMP_RADIAL  PolytropeGravityWithJumpRadial(r_crit, rhoC, K_inner, K_outer, G):
 *                          gravity_params {r_crit, rhoC, K_inner, K_outer, G}
 *   POINT_MASS_RADIAL      PointMassGravityRadial(G, M, X): gravity_params {G, M, X}
 *   RADIAL_TABLE           RadialGravity: phi linearly interpolated between the
 *                          gravity_table_n radii gravity_table_r (increasing) and
 *                          potentials gravity_table_phi; the solver copies the table
 *                          at creation and refuses quadrature points beyond its last radius */
enum zfvm_gravity {
  ZFVM_GRAVITY_NONE = 0,
  ZFVM_GRAVITY_CONSTANT_RADIAL = 1,
  ZFVM_GRAVITY_HARMONIC_RADIAL = 2,
  ZFVM_GRAVITY_POLYTROPE_RADIAL = 3,
  ZFVM_GRAVITY_POLYTROPE_JUMP_RADIAL = 4,
  ZFVM_GRAVITY_POINT_MASS_RADIAL = 5,
  ZFVM_GRAVITY_RADIAL_TABLE = 6
};
enum zfvm_flux_bc { ZFVM_FLUX_BC_NONE = 0, ZFVM_FLUX_BC_CONSTANT = 1, ZFVM_FLUX_BC_ISENTROPIC = 2 };
/* Ghost cells (the mesh's ghost mask) are periodic images of their interior
 * source cells, or, when a ghost cell is its own source, frozen at the values
 * it was set to (FrozenBC, boundary/frozen_boundary_condition.cpp:39-55). */
enum zfvm_boundary { ZFVM_BC_NONE = 0, ZFVM_BC_PERIODIC = 1, ZFVM_BC_FROZEN = 2 };
enum zfvm_precision { ZFVM_FP64 = 0, ZFVM_MIXED = 1 };
/* CWENO_AO (reconstruction/cweno_ao.cpp:35-53) or WENO_AO (weno_ao.cpp:14-24);
 * selected like EulerExperiment::deduce_reconstruction (euler_experiment_impl.hpp:363-376) */
enum zfvm_reconstruction { ZFVM_RC_CWENO_AO = 0, ZFVM_RC_WENO_AO = 1 };

typedef struct {
  int32_t flux;                 /* zfvm_flux                                        */
  double gamma;                 /* euler.eos.gamma                                  */
  double specific_gas_constant; /* euler.eos.specific-gas-constant                  */
  double linear_weights[ZFVM_MAX_STENCILS];
  double epsilon;               /* reconstruction.smoothness_indicator.epsilon      */
  double exponent;              /* reconstruction.smoothness_indicator.exponent     */
  int32_t rk_stages;            /* 1 forward Euler, 2 SSP2, 3 SSP3                  */
  double cfl_number;            /* ode.cfl_number                                   */
  int32_t equilibrium;          /* well-balancing.mode: none / isentropic           */
  int32_t gravity;              /* zfvm_gravity                                     */
  double gravity_strength;      /* g for constant, k for phi = k r^2 / 2            */
  int32_t flux_bc;              /* flux-bc.mode                                     */
  int32_t boundary;             /* ghost-cell boundary condition                    */
  int32_t precision;            /* zfvm_precision                                   */
  int32_t steps_per_recompute;  /* reconstruction.steps_per_recompute (>= 1)        */
  double recompute_threshold;   /* reconstruction.recompute_threshold: refresh sooner
                                   when |scaled (rho, E_int) - equilibrium average| >= it */
  int32_t reconstruction;       /* reconstruction.mode: zfvm_reconstruction           */
  double step_rejection_drho;   /* RejectLargeDensityChange drho_crit_rel; 0: RejectNothing */
  int32_t step_rejection_max_exponent; /* smallest step factor 2^-max_exponent       */
  double heating_rate;          /* heating.rate (model/heating.hpp:52-77); 0: none   */
  double heating_r0, heating_r1; /* heating.lower_boundary / upper_boundary           */
  int32_t n_avars;              /* advected variables (AllVariables::avars columns,
                                   choose_n_avars); 0..ZFVM_MAX_AVARS                */
  double gravity_params[5];     /* euler.gravity parameters of zfvm_gravity         */
  const double *gravity_table_r;   /* RADIAL_TABLE: radii, then potentials          */
  const double *gravity_table_phi;
  int64_t gravity_table_n;
} zfvm_scheme_desc;
#define ZFVM_MAX_AVARS 64

int zfvm_solver_create(zfvm_mesh *m, const zfvm_scheme_desc *scheme, zfvm_solver **out);
int zfvm_solver_destroy(zfvm_solver *s);

/* Upload / download the state (n_cells x 5 AoS host doubles) and the time. */
int zfvm_set_state(zfvm_solver *s, const double *cvars, double t);
int zfvm_get_state(zfvm_solver *s, double *cvars, double *t);
/* set_state + advance + get_state in one call with one host synchronisation:
 * upload cvars_in (n_cells x 5) at time t, run n_steps steps (or to t_end;
 * with fixed_dt > 0 every step is fixed_dt long instead of the CFL step),
 * download the result into cvars_out (may be cvars_in) and its time and step
 * count.  The host-driven loop of RungeKutta::compute_step / TimeLoop with
 * host states (ode/runge_kutta.cpp:146-171, fvm_loops/time_loop.cpp:47-81). */
int zfvm_step_host(zfvm_solver *s, const double *cvars_in, double t, int64_t n_steps, double t_end,
                   double fixed_dt, double *cvars_out, double *t_out, int64_t *steps_out);
/* Upload / download the advected variables (AllVariables::avars: mass-weighted
 * tracers mq, n_cells x n_avars row-major).  A solver with n_avars > 0 starts
 * with them zero.  They are reconstructed like the conserved variables but each
 * on its own (LocalReconstruction::compute_tracer, local_reconstruction.hpp:
 * 127-147) and transported with the numerical flux's wave speeds
 * (HLLCBatten::tracer_flux, flux/hllc.hpp:178-197), always in FP64. */
int zfvm_set_avars(zfvm_solver *s, const double *avars);
int zfvm_get_avars(zfvm_solver *s, double *avars);

/* Snapshot files (io/dump_snapshot_impl.hpp:21-38, model/models.cpp:7-27,
 * model/all_variables.cpp:74-113): datasets "time", "n_steps", "rho", "mv1",
 * "mv2", "mv3", "E", "n_avars", "mq0".. under the reference's names, in an
 * uncompressed NumPy .npz file (numpy.load reads it).  cvars is n_cells x 5,
 * avars n_cells x n_avars, both row-major as in AllVariables.  with_clock = 0
 * leaves out "time" and "n_steps" (the steady-state file).  The file is
 * written to "<path>.tmp" and renamed into place; at most 4 GiB. */
int zfvm_snapshot_write(const char *path, int64_t n_cells, const double *cvars, int32_t n_avars,
                        const double *avars, int32_t with_clock, double t, int64_t n_steps);
int zfvm_snapshot_info(const char *path, int64_t *n_cells, int32_t *n_avars, int32_t *has_clock);
/* n_cells and n_avars must match the file; t and n_steps may be null. */
int zfvm_snapshot_read(const char *path, int64_t n_cells, double *cvars, int32_t n_avars, double *avars,
                       double *t, int64_t *n_steps);
/* DumpSnapshot::do_visualization for a solver: its current state and time,
 * with the caller's step count. */
int zfvm_solver_write_snapshot(zfvm_solver *s, const char *path, int64_t n_steps);
/* Restart (LoadSnapshot::do_load, io/load_snapshot.cpp:9-13): state and time
 * from the file; the file's step count is returned in *n_steps (may be null). */
int zfvm_solver_read_snapshot(zfvm_solver *s, const char *path, int64_t *n_steps);

/* The rate of change of the conserved and the advected variables
 * (n_cells x 5 and n_cells x n_avars); ghost-cell rows are zero. */
int zfvm_rate_of_change_all(zfvm_solver *s, double *tendency, double *avars_tendency);

/* One evaluation of the summed rate of change of the current state
 * (SumRatesOfChange::compute, ode/rate_of_change.cpp:21-27); output n_cells x 5.
 * Ghost-cell rows are zero. */
int zfvm_rate_of_change(zfvm_solver *s, double *tendency);

/* Size of the fixed device scratch of zfvm_rate_of_change_noalloc: 16 MiB,
 * present on every device that loads the library until the process exits. */
#define ZFVM_NOALLOC_SCRATCH_BYTES (16u << 20)

/* Same result as zfvm_rate_of_change, for callers that must not allocate device
 * memory inside their loop: an application whose own pool allocator has
 * reserved the device memory it may use, or a time-critical loop that cannot
 * take the device-wide wait of cudaFree (zfvm_rate_of_change allocates and
 * frees a small buffer on every call).  This call allocates nothing: its stage
 * scratch is a fixed array of ZFVM_NOALLOC_SCRATCH_BYTES inside the library.
 * This entry point has no counterpart in the reference.
 *  - Limit: about 40 000 cells for third-order triangles and 20 000 for
 *    third-order tetrahedra; a larger solver fails with ZFVM_EINVAL and a
 *    message giving the bytes it needs.
 *  - The first call on a device looks up the array's device address; make that
 *    first call before any stream capture on that device.
 *  - Every call on a device shares the one array.  Calls return only when their
 *    work is done, so calls from one thread never overlap; calls from several
 *    threads must be serialised by the caller, or they race on the GPU.
 *  - The solver's device must be current; a call made while another device is
 *    current fails with ZFVM_EINVAL instead of handing over that device's array. */
int zfvm_rate_of_change_noalloc(zfvm_solver *s, double *tendency);

/* ---- fluxes and boundary conditions outside the solver's loop ----------------
 * For callers that keep the reference's own loops (FluxLoop with a numerical
 * flux template argument, RungeKutta with a BoundaryCondition object) around
 * the GPU arithmetic.  Each call is one launch over n entries of host arrays,
 * with device scratch allocated for the call: batch many face points per call. */

/* HLLCBatten::flux (flux/hllc.hpp:142-176), or the Rusanov flux, of n pairs of
 * face states in the face frame (rows of 5: rho, normal momentum, tangential
 * momenta, E; ideal gas with gamma).  flux_out: n x 5.  speeds (may be null):
 * n x 3, (s_L, s_star, s_R) of the HLLC fan, (-s_max, 0, s_max) for Rusanov. */
int zfvm_numerical_flux(int32_t flux, double gamma, int64_t n, const double *uL, const double *uR,
                        double *flux_out, double *speeds);

/* HLLCBatten::tracer_flux (flux/hllc.hpp:178-197), or the Rusanov flux, of an
 * advected variable mq for n face points, with the speeds zfvm_numerical_flux
 * returned for the same states.  flux_out: n. */
int zfvm_tracer_flux(int32_t flux, int64_t n, const double *uL, const double *uR, const double *mqL,
                     const double *mqR, const double *speeds, double *flux_out);

/* BoundaryCondition::apply (boundary/boundary_condition.hpp:12-21) with the
 * solver's ghost cells on a host state (n_cells x 5, and n_cells x n_avars
 * when the scheme has advected variables), in place: a frozen ghost cell takes
 * its row of frozen_cvars / frozen_avars (FrozenBC::apply,
 * boundary/frozen_boundary_condition.cpp:39-55; null keeps the row), a periodic
 * image its source cell's row; interior rows are unchanged. */
int zfvm_apply_boundary(zfvm_solver *s, const double *frozen_cvars, const double *frozen_avars, double *cvars,
                        double *avars);

/* EulerGlobalReconstruction::compute (reconstruction/global_reconstruction_impl.hpp:100-163):
 * reconstruct the current state in every interior and first-layer ghost cell;
 * the limited polynomials stay with the solver until the next call. */
int zfvm_reconstruct(zfvm_solver *s);

/* GlobalReconstruction::operator()(i, x) (global_reconstruction_decl.hpp:29) for n
 * points: the reconstruction of cell cells[k] at x[3k .. 3k+2], equilibrium
 * included, as (rho, m1, m2, m3, E) rows of u (n x 5).  Host arithmetic on the
 * records of the last zfvm_reconstruct. */
int zfvm_reconstruction_eval(const zfvm_solver *s, int64_t n, const int64_t *cells, const double *x, double *u);

/* CFL time step of the current state (LocalCFL, local_cfl_condition_impl.hpp:24-40). */
int zfvm_cfl_dt(zfvm_solver *s, double *dt);

/* One Runge-Kutta step of size dt (RungeKutta::compute_step, runge_kutta.cpp:146-171). */
int zfvm_step(zfvm_solver *s, double dt);

/* Steps rejected so far by RejectLargeDensityChange (ode/step_rejection.cpp:17-56,
 * TimeLoop::reject_step time_loop.cpp:182-198): with step_rejection_drho > 0, a
 * step whose density changes anywhere by more than drho * rho is redone from its
 * start with half the time step; two accepted steps in a row double the factor
 * again (at most 1, at least 2^-max_exponent).  Applies to zfvm_advance and to
 * batch slots (a slot steps on the solver's own clock, so the count of a batched
 * run is read from the solver after zfvm_batch_remove); counted since the state
 * was last set (zfvm_set_state, zfvm_step_host, a snapshot read). */
int zfvm_step_rejections(zfvm_solver *s, int64_t *n);

/* TimeLoop (fvm_loops/time_loop.cpp:36-81) without IO: steps with the CFL time
 * step until `n_steps` steps are done (if > 0) or t reaches t_end (if > 0),
 * dt = min(dt_cfl, t_end - t).  The clock stays on the device; the whole loop is
 * replayed from a CUDA graph in chunks of `graph_steps`. */
int zfvm_advance(zfvm_solver *s, int64_t n_steps, double t_end, double *t_out, int64_t *steps_out);

/* Device-timed loop for benchmarks: runs `n_steps` fixed-count steps and returns
 * the milliseconds measured with CUDA events on the solver's stream. */
int zfvm_advance_timed(zfvm_solver *s, int64_t n_steps, float *ms);

/* Average per-launch device time (ms) of the three stage kernels
 * {reconstruct, face flux, update}, measured with CUDA events around every
 * launch on the solver's stream over `n_steps` CFL steps (no graph). */
int zfvm_kernel_times(zfvm_solver *s, int64_t n_steps, float *ms);

/* Number of kernel launches one step issues. */
int zfvm_launches_per_step(const zfvm_solver *s, int32_t *launches);

/* Bytes of device memory the solver holds. */
int zfvm_device_bytes(const zfvm_solver *s, int64_t *bytes);

/* ---- batches -------------------------------------------------------------
 * Many independent solves stepped together: one persistent launch per phase
 * per RK stage covers every slot (of one kernel configuration), each slot with
 * its own clock.  No counterpart class in the reference (it runs one solve per
 * process, or one per MPI rank). */
typedef struct zfvm_batch zfvm_batch;
int zfvm_batch_create(int32_t max_slots, zfvm_batch **out);
int zfvm_batch_destroy(zfvm_batch *b);
/* Add a solver (its state already set) that runs until n_steps (if > 0) or
 * t_end (if > 0).  The solver must not be driven by itself while in a batch. */
int zfvm_batch_add(zfvm_batch *b, zfvm_solver *s, int64_t n_steps, double t_end, int32_t *slot);
int zfvm_batch_remove(zfvm_batch *b, int32_t slot);
/* Replay up to max_steps batched steps; returns the number of slots still running. */
int zfvm_batch_advance(zfvm_batch *b, int32_t max_steps, int32_t *n_running);
/* The batch form of zfvm_step_host, with one host synchronisation for the
 * whole batch: each slot k with states_in[k] non-null takes that state
 * (n_cells x 5 AoS doubles) at the time its clock holds, the batch advances up
 * to max_steps steps (zfvm_batch_advance), and each slot k with states_out[k]
 * non-null is read back into it (states_out[k] may be states_in[k]) once its
 * last step is closed (a rejected step is put back first).  Both
 * arrays are indexed by slot, max_slots long, and may be null.  Every slot's
 * open step is closed before the new states land (a rejected one put back), as
 * zfvm_batch_remove does; advected variables keep their device values.  Host
 * buffers in page-locked memory let the copies run asynchronously.  No
 * counterpart in the reference. */
int zfvm_batch_step_host(zfvm_batch *b, const double *const *states_in, double *const *states_out,
                         int32_t max_steps, int32_t *n_running);
int zfvm_batch_advance_timed(zfvm_batch *b, int32_t n_steps, float *ms);
/* Pick the persistent grid sizes of each group's kernels by timing candidates. */
int zfvm_batch_autotune(zfvm_batch *b, int32_t trial_steps, float *best_ms);

/* The launch shape of each of the batch's kernel groups (solvers of one stencil
 * shape, form, flux and equilibrium): 6 entries per group -- shape id, threads
 * per block (= cells or faces per tile), grids of the reconstruction, face and
 * update kernels (0: one block per tile), 1 when the autotuner chose them.
 * *n_groups is the number of groups; at most max_groups are written.  No
 * counterpart in the reference (it runs one solve per process). */
int zfvm_batch_launch_shapes(const zfvm_batch *b, int32_t max_groups, int32_t *shapes, int32_t *n_groups);
/* Average per-launch device time (ms) of the three batched stage kernels
 * {reconstruct, face flux, update} over `n_steps` steps (events, no graph). */
int zfvm_batch_kernel_times(zfvm_batch *b, int32_t n_steps, float *ms);
int zfvm_batch_slot_status(zfvm_batch *b, int32_t slot, double *t, int64_t *steps, int32_t *done,
                           int32_t *status);
int zfvm_batch_slots(const zfvm_batch *b, int32_t *n_active);

/* ---- serving --------------------------------------------------------------
 * A request loop with continuous batching: solves submitted from any thread
 * wait in a queue, are admitted in arrival order while their device footprint
 * (zfvm_solver_footprint) fits the memory budget and a slot is free (smaller
 * requests may overtake one that does not fit, at most 8 times), join the
 * solves already running in one batch, keep their state on the device and
 * return their final state when done.  One worker thread owns the device work.
 * No counterpart in the reference (one solve per process). */
typedef struct zfvm_server zfvm_server;
typedef struct {
  int64_t hbm_budget_bytes;  /* device bytes the solves may hold (<= 0: 80% of the free memory) */
  int32_t max_slots;         /* concurrent solves                                              */
  int32_t steps_per_round;   /* batched steps between admission and retirement                 */
} zfvm_server_desc;
typedef struct {
  int64_t submitted, completed, failed, queued, running;
  int64_t bytes_in_use, bytes_peak, budget_bytes;
  int64_t cell_stage_updates;  /* work of the completed solves                  */
  int64_t rounds;
  double busy_s;               /* worker time spent stepping running solves      */
  double setup_s;              /* set-up thread time creating solvers and
                                  uploading initial states (overlaps busy_s)     */
} zfvm_server_stats;
/* Device bytes zfvm_solver_create will allocate for this mesh and scheme. */
int zfvm_solver_footprint(const zfvm_mesh *m, const zfvm_scheme_desc *scheme, int64_t *bytes);
int zfvm_server_create(const zfvm_server_desc *desc, zfvm_server **out);
/* Stops the worker; unfinished requests fail.  No thread may be waiting on the server. */
int zfvm_server_destroy(zfvm_server *srv);
/* Queue a solve of `mesh` (kept alive by the caller until the request is
 * waited for) from cvars (n_cells x 5, copied) at time t0 until n_steps steps
 * (if > 0) or time t_end (if > t0).  ZFVM_ENOMEM if its footprint exceeds the budget;
 * ZFVM_EINVAL for a scheme with n_avars > 0 (requests carry conserved variables only). */
int zfvm_server_submit(zfvm_server *srv, zfvm_mesh *mesh, const zfvm_scheme_desc *scheme, const double *cvars,
                       double t0, int64_t n_steps, double t_end, int64_t *id);
/* phase: 0 queued, 1 running, 2 done, 3 failed */
int zfvm_server_poll(zfvm_server *srv, int64_t id, int32_t *phase);
/* Wait (timeout_s < 0: no limit) for a request, copy its final state, time and
 * steps, and release it.  times_ms = {queued, running, submit to result}.  A
 * failed solve returns its error status. */
int zfvm_server_wait(zfvm_server *srv, int64_t id, double timeout_s, double *cvars, double *t, int64_t *steps,
                     double *times_ms);
int zfvm_server_get_stats(zfvm_server *srv, zfvm_server_stats *stats);

const char *zfvm_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
