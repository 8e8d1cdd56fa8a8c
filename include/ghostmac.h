/*
 * ghostmac.h — C ABI of the GB300 ghost-cell MAC AB2/CN library (libghostmac.so).
 *
 * One handle holds one cylinder case: a 2-D staggered (MAC) grid, nx x ny pressure
 * cells, u on vertical faces (ny x (nx+1)), v on horizontal faces ((ny+1) x nx),
 * all arrays float64 and C order.  Setup (classification, ghost stencils, operators,
 * boundary Schur factor) runs once in gm_create; every step runs on the GPU.
 *
 * Pointers: every array argument may be a host pointer or a CUDA device pointer
 * (detected per call with cudaPointerGetAttributes).  Host arrays are copied.
 * Return value: GM_OK or an error class; gm_last_error() gives the message.
 * The classes map 1:1 to the reference's exceptions: GM_EVALUE -> ValueError,
 * GM_ERUNTIME -> RuntimeError (a failed gate), GM_EFLOAT -> FloatingPointError.
 * A handle is not thread safe; it owns one CUDA stream.
 *
 * Each entry point names the reference interface it replaces
 * (paths relative to the reference repository invisce/cfd-cylinder-flow-ghost-cell).
 */
#ifndef GHOSTMAC_H
#define GHOSTMAC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GM_OK 0
#define GM_EVALUE 1     /* ValueError: bad configuration or input */
#define GM_ERUNTIME 2   /* RuntimeError: a solver gate failed */
#define GM_EFLOAT 3     /* FloatingPointError: non-finite force */
#define GM_ECUDA 4      /* CUDA error or no device */
#define GM_ENOTIMPL 5   /* option not built in this library */

typedef struct gm_handle gm_handle;

/* Constructor arguments of MAC_CylinderFlow restricted to the ghost_cell/ab2_cn
 * path (solver/main.py:40-44). */
typedef struct gm_config {
  int32_t nx, ny;
  double Lx, Ly, D, xc, yc, nu, rho, U_inf;
  int32_t inflow;                 /* 0 uniform, 1 parabolic */
  double U_m;                     /* parabolic peak; <= 0 selects 1.5*U_inf */
  int32_t pressure_solver;        /* 0 direct (DCT/DST + boundary Schur), 1 iterative (GMRES) */
  int32_t pressure_extension;     /* 0 neumann, 1 quadratic */
  int32_t velocity_interpolation; /* 0 bilinear, 1 biquadratic */
  int32_t precision;              /* 0 plain FP64, 1 FP32 transforms with FP64 refinement */
} gm_config;

typedef struct gm_sizes {
  int64_t nx, ny, usize, vsize, psize;
  int64_t nu_active, nv_active, np_active, qsize;
  int64_t n_surface;               /* surface quadrature points */
  int64_t rank_p, rank_u, rank_v;  /* boundary Schur ranks (u, v after the first step) */
  int64_t ghost_u, ghost_v, ghost_p;
  double dx, dy, U_ref;
} gm_sizes;

/* Per-step diagnostics: the keys of MAC_CylinderFlow.last_step_diagnostics
 * (solver/main.py:407-413, solver/optimized_ghost_cell.py:269-276,
 * solver/time_integration.py:143-145). */
typedef struct gm_step_diag {
  double time, dt, max_divergence, cfl;
  double cd, cl, cd_pressure, cd_viscous, cl_pressure, cl_viscous;
  double momentum_residual_linf, coupled_momentum_residual_linf;
  double pressure_residual_linf, pressure_residual_relative_l2;
  double forces[6];               /* fx, fy, fx_p, fy_p, fx_v, fy_v */
  int32_t pressure_solve_count, pressure_iterations, pressure_refinement_iterations;
  int32_t momentum_refinement_iterations;
  int32_t status;                 /* 0 ok, else the GM_E* class of the failure */
  int32_t gate;                   /* which gate failed (GM_GATE_*), 0 if none */
} gm_step_diag;

#define GM_GATE_PROJECTION 1   /* solver/optimized_ghost_cell.py:226-228 */
#define GM_GATE_MOMENTUM 2     /* solver/time_integration.py:102-104 */
#define GM_GATE_PRESSURE 3     /* solver/pressure_schur.py:69-70 */
#define GM_GATE_PRESSURE_RHS 4 /* solver/pressure_schur.py:33-34 */
#define GM_GATE_STEP 5         /* solver/main.py:414-415 */
#define GM_GATE_FORCE 6        /* solver/main.py:404-405 */
#define GM_GATE_CFL_SCREEN 7   /* solver/main.py:273-278 */
#define GM_GATE_FINITE 8       /* solver/time_integration.py:15-17 */

typedef struct gm_solve_info {
  double residual_linf, residual_relative_l2, residual_target_linf, roundoff_bound_linf,
      backward_error_linf;
  int32_t iterations, refinement_iterations, status, rank;
} gm_solve_info;

/* --- lifecycle ------------------------------------------------------------ */

/* Replaces MAC_CylinderFlow.__init__ ghost/ab2_cn branch (solver/main.py:40-242):
 * builds the mask check, inlet profile, GhostCellIntegrator
 * (solver/optimized_ghost_cell.py:61-150) and the initial projection
 * (solver/main.py:229-230).  The initial state is then readable with gm_get_state. */
int gm_create(const gm_config* cfg, gm_handle** out);
int gm_destroy(gm_handle* h);
/* Setup only, on the host: classification, stencils, operators and Schur rows without
 * touching a GPU.  The geometry accessors below work on such a handle; state, step and
 * operator calls return GM_ECUDA. */
int gm_create_host(const gm_config* cfg, gm_handle** out);
/* Build the CN Helmholtz data for a timestep (solver/optimized_ghost_cell.py:243-255);
 * gm_step does this itself when dt changes.  On a host-only handle only the rows are built. */
int gm_prepare_dt(gm_handle* h, double dt);
/* Message of the last error on this handle (or of the last failed gm_create when h is NULL). */
const char* gm_last_error(const gm_handle* h);
int gm_get_sizes(const gm_handle* h, gm_sizes* out);
/* Optional: run this handle's work on an external stream (e.g. torch.cuda.current_stream()). */
int gm_set_stream(gm_handle* h, void* cuda_stream);

/* --- geometry (host arrays) ------------------------------------------------ */

/* Active flat indices ui, vi, pi (solver/optimized_ghost_cell.py:66-79). */
int gm_get_indices(const gm_handle* h, int64_t* ui, int64_t* vi, int64_t* pi);
/* Ghost rows of the extension operators E (u, v) and P (pressure):
 * which = 0 (u), 1 (v), 2 (p).  rows: grid flat index of each ghost point;
 * ptr (n+1), cols (grid flat indices of active points), vals.  Pass NULL to
 * query the counts through *n_rows and *nnz (solver/optimized_ghost_cell.py:14-58). */
int gm_get_ghost_stencils(const gm_handle* h, int32_t which, int64_t* n_rows, int64_t* nnz,
                          int64_t* rows, int64_t* ptr, int64_t* cols, double* vals);
/* Boundary Schur rows (rectangle flat indices) for which = 0 (pressure),
 * 1 (u Helmholtz), 2 (v Helmholtz) (solver/pressure_schur.py:77-91). */
int gm_get_schur_rows(const gm_handle* h, int32_t which, int64_t* n, int64_t* rows);
/* Circle quadrature points (y, x) pairs (solver/cut_cell_solver.py:70-77). */
int gm_get_surface_points(const gm_handle* h, double* yx);
/* Quadratic point-pressure reconstruction at n_points (y, x) pairs (replaces
 * build_pressure_reconstruction, solver/cut_cell_solver.py:25-55, as used by CylinderSamples,
 * postprocessing/cylinder_observables.py:38-39): a CSR matrix of n_points rows over the grid flat
 * pressure indices.  *nnz is always set; ptr (n_points + 1), cols and vals (nnz) are filled when
 * not NULL, so a first call with them NULL sizes the arrays.  Points outside the domain, inside
 * the solid or not finite give GM_EVALUE with the reference's message.  Works on host-only
 * handles. */
int gm_pressure_reconstruction(gm_handle* h, const double* yx, int32_t n_points, int64_t* nnz, int64_t* ptr,
                               int64_t* cols, double* vals);

/* --- state ----------------------------------------------------------------- */

/* u (ny x nx+1), v (ny+1 x nx), p (ny x nx); any may be NULL to skip. */
int gm_set_state(gm_handle* h, const double* u, const double* v, const double* p);
int gm_get_state(gm_handle* h, double* u, double* v, double* p);
/* Inlet profile u_inlet[ny] (solver/main.py:281-286 writes it; solver/optimized_ghost_cell.py:238-242 reads it). */
int gm_set_inlet(gm_handle* h, const double* u_inlet);
/* AB2/CN history for checkpoints (solver/main.py:511-516, 558-566):
 * previous_advection[qsize], half_pressure[np_active], previous_dt.
 * has_history = 0 clears it (next step uses the projected midpoint start-up). */
int gm_set_history(gm_handle* h, int32_t has_history, const double* previous_advection,
                   const double* half_pressure, double previous_dt);
int gm_get_history(gm_handle* h, int32_t* has_history, double* previous_advection,
                   double* half_pressure, double* previous_dt);

/* --- the step ----------------------------------------------------------------- */

/* n_steps of MAC_CylinderFlow.solve's loop body for this path (solver/main.py:271-429:
 * CFL screen every 100 steps counted from first_step_index, gg.advance
 * (solver/optimized_ghost_cell.py:236-278 -> solver/time_integration.py:7-145),
 * surface forces, coefficient and divergence/CFL gates).  The inlet is held fixed.
 * diag receives n_steps records (host pointer).  A failed gate stops the run:
 * the return value is its class and diag[k].status/gate tell where. */
int gm_step(gm_handle* h, double dt, int32_t n_steps, int64_t first_step_index, double start_time,
            gm_step_diag* diag);
/* gm_set_state (u_in, v_in, p_in), gm_set_inlet (u_inlet), gm_step and gm_get_state (u_out,
 * v_out, p_out) in one call, ordered on the handle's stream with one host synchronisation at the
 * end (the reference's solve loop, solver/main.py:265-429, as one call per chunk of steps).  Any
 * pointer may be NULL to skip that transfer.  On a failed gate the outputs may hold the failed
 * step's state; gm_get_state then reads the last good one. */
int gm_solve_io(gm_handle* h, const double* u_in, const double* v_in, const double* p_in, const double* u_inlet,
                double dt, int32_t n_steps, int64_t first_step_index, double start_time, gm_step_diag* diag,
                double* u_out, double* v_out, double* p_out);

/* --- operators (GhostCellIntegrator methods, solver/optimized_ghost_cell.py:174-234) --- */

#define GM_OP_PACK 1        /* (u|v grids, usize+vsize) -> q          :174-177 */
#define GM_OP_UNPACK 2      /* q -> (u|v grids) with ghosts and inlet :179-184 */
#define GM_OP_ADVECTION 3   /* q -> -N(q)                            :186-199 */
#define GM_OP_DIFFUSION 4   /* q -> L q + diff_offset                :201-205 */
#define GM_OP_GRADIENT 5    /* packed p (np_active) -> G p           :207-210 */
#define GM_OP_DIVERGENCE 6  /* q -> D q + div_offset                 :212-216 */
#define GM_OP_H_MATVEC 7    /* q -> q - dt/2 L q (param = dt)        :231-234 */
#define GM_OP_PRESSURE_EXTEND 8 /* packed p -> P p (full grid)       :278    */
int gm_apply(gm_handle* h, int32_t op, double param, const double* x, double* y);

/* project(q, dt) -> (q - dt G phi, phi) with the divergence gate
 * (solver/optimized_ghost_cell.py:218-229). */
int gm_project(gm_handle* h, double dt, const double* q, double* q_out, double* phi,
               gm_solve_info* info);
/* Monitored pressure solve A phi = rhs (solver/pressure_schur.py:16-72 via
 * solver/optimized_ghost_cell.py:110-111): rhs, phi of length np_active. */
int gm_pressure_solve(gm_handle* h, const double* rhs, double* phi, gm_solve_info* info);
/* Separable rectangle inverse (solver/rectangular_inverse.py:8-58): kind 0 pressure,
 * 1 u, 2 v; for u and v, nu_dt = (nu, dt) of the Helmholtz operator.  b and x are
 * rectangle grids (ny x nx, or (ny-1) x nx for v). */
int gm_rectangle_solve(gm_handle* h, int32_t kind, double dt, const double* b, double* x);
/* surface_forces(u, v, p, mu) -> fx, fy, fx_p, fy_p, fx_v, fy_v
 * (solver/optimized_ghost_cell.py:280-286). */
int gm_surface_forces(gm_handle* h, const double* u, const double* v, const double* p, double mu,
                      double out[6]);
/* Fluid-cell divergence statistics of mac_engine.calculate_mac_divergence_cpp
 * (solver/src/bindings.cpp:343-390): out = max, sum div^2, core sum div^2; counts = count, core count. */
int gm_divergence_stats(gm_handle* h, const double* u, const double* v, double out[3], int64_t counts[2]);

/* --- many cases per GPU (no reference counterpart: the reference steps one case) --- */

/* A batch of independent cases (handles created with gm_create) stepped together: each
 * steady step of all cases is one CUDA graph launch with one concurrent branch per case. */
typedef struct gm_batch gm_batch;
int gm_batch_create(gm_handle* const* cases, int32_t n_cases, gm_batch** out);
int gm_batch_destroy(gm_batch* b);
const char* gm_batch_last_error(const gm_batch* b);
/* The launch shapes (row-pass group threads, groups per block, columns per column-solve block)
 * the batch chose by timing its candidates under concurrency at its first steady step (all 0
 * before that), and the candidates' probe times in ms (-1: did not fit), up to n of them. */
int gm_batch_shapes(const gm_batch* b, int32_t shape[3], float* probe_ms, int32_t n);
/* n_steps of every case (as gm_step); start_times[n_cases] may be NULL (time 0);
 * diag (may be NULL) receives n_cases * n_steps records, case-major (diag[c * n_steps + k]).
 * When a gate of some case fails, stepping stops at the end of the current graph batch
 * (at most 64 steps): the failed case is left at its last good step, the others at the
 * batch end; steps_done[n_cases] (may be NULL) receives each case's completed steps and
 * the call returns the first failure's code.  The cases must outlive the batch; each
 * case may still be stepped alone with gm_step between batch calls. */
int gm_batch_step(gm_batch* b, double dt, int32_t n_steps, int64_t first_step_index, const double* start_times,
                  gm_step_diag* diag, int32_t* steps_done);

/* --- periodic Taylor-Green case (verification/taylor_green.py:14-59) ------------- */

/* The AB2/CN step on the periodic staggered grid of [0, 2 pi]^2 (n x n cells, h = 2 pi / n)
 * with the periodic flux-form operators of solver/cut_cell_solver.py:108-130 and
 * Fourier-space pressure and CN solves.  precision 0: FP64; 1: FP32 stencils and
 * transforms with both solves refined against the FP64 operators. */
typedef struct gm_tg gm_tg;
int gm_tg_create(int32_t n, double nu, int32_t precision, gm_tg** out);
int gm_tg_destroy(gm_tg* t);
const char* gm_tg_last_error(const gm_tg* t);
/* q: u (n x n) then v (n x n); p: n x n (host or device pointers); clears the AB2 history */
int gm_tg_set_state(gm_tg* t, const double* q, const double* p);
/* any output may be NULL: velocity, half-step pressure, output pressure of the last step */
int gm_tg_get_state(gm_tg* t, double* q, double* p_half, double* p_out);
/* n_steps AB2/CN steps of size dt; *max_divergence (in/out) is raised to the largest
 * max |div q| after any step */
int gm_tg_step(gm_tg* t, double dt, int32_t n_steps, double* max_divergence);

/* --- learned pressure preconditioner (no reference counterpart) ----------------- */

/* A 4-level convolutional U-Net on the pressure grid (channels 16, 32, 64, 64; 12 3x3
 * convolutions, 253,872 weights + 465 biases), BF16 weights, FP32 activations and
 * accumulation.  It is the learned slot of the GMRES preconditioner.  Weights are passed per
 * call: w_bf16[k] = layer k's weights [cout][cin][3][3] as BF16 bit patterns, bias[k] =
 * [cout] floats (device pointers).  Tensors are [batch][channel][height][width] float32
 * (device); height and width are multiples of 8. */
typedef struct gm_unet gm_unet;
int gm_unet_layers(int32_t* n_layers, int32_t* cin, int32_t* cout);
int gm_unet_create(int32_t batch, int32_t height, int32_t width, gm_unet** out);
int gm_unet_destroy(gm_unet* u);
const char* gm_unet_last_error(const gm_unet* u);
/* the network's own input buffer (batch x 2 x height x width) */
int gm_unet_input(gm_unet* u, float** x);
/* y (batch x 1 x height x width) = net(x); x may be NULL (the input buffer is used); the
 * activations are kept for gm_unet_backward */
int gm_unet_forward(gm_unet* u, const uint16_t* const* w_bf16, const float* const* bias, const float* x, float* y,
                    void* cuda_stream);
/* adds dL/dw and dL/db of the last forward pass for dL/dy = dy to dw[k] ([cout][cin][3][3])
 * and db[k] ([cout]) */
int gm_unet_backward(gm_unet* u, const uint16_t* const* w_bf16, const float* dy, float* const* dw, float* const* db,
                     void* cuda_stream);
/* Attaches a network to a handle's GMRES path (pressure_solver = iterative): the
 * preconditioner becomes z = T^-1 r + s net([r / s, mask]) with s = max |r|.  The network's
 * grid must be the pressure grid (batch 1); the weight arrays stay owned by the caller and
 * must outlive the attachment.  net = NULL detaches. */
int gm_set_learned_preconditioner(gm_handle* h, gm_unet* net, const uint16_t* const* w_bf16,
                                  const float* const* bias);

/* Records the pressure solves of the following steps (the training pairs of the learned
 * preconditioner): solve k stores its right-hand side at rhs + k * nx * ny and its solution at
 * sol + k * nx * ny (pressure grids, zeros off the active cells; device buffers of
 * capacity * nx * ny doubles).  While recording, steps run launch by launch.  capacity 0
 * stops recording. */
int gm_set_pressure_recorder(gm_handle* h, double* rhs, double* sol, int32_t capacity);
int32_t gm_pressure_recorded(const gm_handle* h);

/* --- allocation-free entry point ------------------------------------------------ */

/* No counterpart in the reference.  For callers that cannot call cudaMalloc (code
 * running inside another runtime's fixed device-memory arena, or tools that only
 * borrow device arrays): the fluid-cell divergence statistics of gm_divergence_stats
 * computed from caller-owned DEVICE arrays u (ny x nx+1), v (ny+1 x nx) and mask
 * (ny x nx bytes, nonzero = solid) without any allocation.  Its scratch is a static
 * device array sized for at most GM_NOALLOC_MAX_CELLS cells (larger grids return
 * GM_EVALUE), held by every GPU that loads the library.  The arrays must live on the
 * current device.  The first call on a device looks up that array's address for the
 * device.  Every call is synchronous (it waits for its stream to return the totals), so it
 * must not be made while a stream is being captured.  Calls that overlap on the GPU share
 * the array and race.  out = max |div|, sum div^2, core sum div^2; counts = fluid cells,
 * core cells.  Errors: gm_last_error(NULL), which holds the calling thread's last error. */
#define GM_NOALLOC_MAX_CELLS 1048576
int gm_divergence_stats_noalloc(const double* u, const double* v, const uint8_t* mask, int32_t nx, int32_t ny,
                                double dx, double dy, double out[3], int64_t counts[2], void* cuda_stream);

/* --- the legacy staircase path's native kernels (module mac_engine) ------------- */
/* Arrays are C-order float64 (mask: one byte per pressure cell, nonzero = solid), u ny x (nx+1),
 * v (ny+1) x nx, p / phi / rhs ny x nx, inlet ny; each may be host memory (staged through a
 * per-thread device buffer) or device memory of the current device.  stream: a cudaStream_t or
 * NULL; every call returns with its outputs written.  Invalid sizes and parameters give
 * GM_EVALUE with the reference's message (gm_last_error(NULL)). */
/* u*, v* and the Poisson right-hand side rho/dt div u* (predictor_rhs_cpp,
 * solver/src/bindings.cpp:47-216): upwind (centered = 0) or centred convection, staircase wall
 * reflections, slip or no-slip channel walls.  Bit-identical to the reference's compiled loops. */
int gm_mac_predictor_rhs(const double* u, const double* v, double* u_star, double* v_star, double* rhs,
                         const double* p, const uint8_t* mask, const double* inlet, int32_t nx, int32_t ny, double dx,
                         double dy, double dt, double nu, double rho, int32_t slip_walls, int32_t centered,
                         void* stream);
/* u = u* - dt/rho grad phi with the exact Dirichlet outlet (corrector_cpp,
 * solver/src/bindings.cpp:218-282).  Bit-identical to the reference. */
int gm_mac_corrector(double* u, double* v, const double* u_star, const double* v_star, const double* phi,
                     const uint8_t* mask, const double* inlet, int32_t nx, int32_t ny, double dx, double dy, double dt,
                     double rho, int32_t slip_walls, void* stream);
/* The legacy loop's own AB2 step on u*, v* (centred transport, solver/main.py:315-322):
 * d = (u* - u)/dt on the interior faces, u* += dt alpha (d - prev_d) when has_prev, prev_d = d
 * (prev_du / prev_dv hold d between steps, grid-shaped); and its recomputed Poisson right-hand
 * side rho/dt div u*, zero on masked cells (:337-339).  what: bit 1 runs the AB2 step (centred
 * transport only), bit 2 the right-hand side (the ghost-cell branch sets its ghost faces between
 * the two).  Bit-identical to the reference's numpy arithmetic. */
#define GM_MAC_AB2 1
#define GM_MAC_RHS 2
int gm_mac_ab2_rhs(const double* u, const double* v, double* u_star, double* v_star, double* prev_du,
                   double* prev_dv, double* rhs, const uint8_t* mask, int32_t nx, int32_t ny, double dx, double dy,
                   double dt, double rho, double alpha, int32_t has_prev, int32_t what, void* stream);
/* Image-point ghost velocities of the legacy ghost-cell branch (apply_velocity_ghost_cells,
 * solver/ghost_cell.py:159-184) on one face grid of field_size values: for ghost face g (in the
 * reference's row-major order), field[target[g]] = wall - gamma[g] (ip - wall), ip =
 * sum_q weights[4g+q] * x_q over its four bilinear corners src[4g+q] (corner order 00, 10, 01,
 * 11).  The reference sets the faces in order, so a corner that is a ghost face reads the value
 * that face had before the pass (snap_of[4g+q] = its ghost index) or after it (-1, allowed only
 * when that face sits on a lower level than g); level[g] in [0, n_levels) are launched in turn.
 * The tables come from the geometry (the Python host builds them).  Bit-identical. */
int gm_mac_ghost_apply(double* field, int64_t field_size, int64_t n_ghost, const int64_t* target, const int64_t* src,
                       const int32_t* snap_of, const double* weights, const double* gamma, const int32_t* level,
                       int32_t n_levels, double wall, void* stream);
/* The ghost-cell branch's corrector (solver/main.py:347-370).  boundary_faces = 0: u = u*,
 * minus dt/rho dphi/dx between two fluid cells, zero between two masked cells, the inlet, the
 * Dirichlet outlet u* + 2 dt/rho phi/dx, v likewise with zero wall rows.  boundary_faces = 1:
 * faces between a fluid and a masked cell take u* again (called after the ghost velocities).
 * Bit-identical. */
int gm_mac_ghost_correct(double* u, double* v, const double* u_star, const double* v_star, const double* phi,
                         const uint8_t* mask, const double* inlet, int32_t nx, int32_t ny, double dx, double dy,
                         double dt, double rho, int32_t boundary_faces, void* stream);
/* Pressure and viscous forces on the true circle (extract_true_surface_forces,
 * solver/ghost_cell.py:186-234): n_theta equally spaced points, bilinear p, u, v (zero outside
 * the grid) and central differences of step 1e-4 dx for the velocity gradients.  out = (fx_p,
 * fy_p, fx_v, fy_v), summed in a fixed order (equal to the reference's sums to rounding). */
int gm_mac_ghost_forces(const double* u, const double* v, const double* p, int32_t nx, int32_t ny, double dx,
                        double dy, double xc, double yc, double radius, int32_t n_theta, double mu, double out[4],
                        void* stream);
/* Staircase pressure and shear forces out = (fx_p, fy_p, fx_v, fy_v) (calculate_mac_forces_cpp,
 * solver/src/bindings.cpp:284-341); the sums are reduced in a fixed order. */
int gm_mac_forces(const double* u, const double* v, const double* p, const uint8_t* mask, int32_t nx, int32_t ny,
                  double dx, double dy, double mu, double out[4], void* stream);
/* Fluid-cell divergence statistics without a handle (calculate_mac_divergence_cpp,
 * solver/src/bindings.cpp:343-390): out = (max |div|, sum div^2, core sum div^2),
 * counts = (fluid cells, core cells). */
int gm_mac_divergence(const double* u, const double* v, const uint8_t* mask, int32_t nx, int32_t ny, double dx,
                      double dy, double out[3], int64_t counts[2], void* stream);

/* The pressure system of an aperture-weighted MAC grid alone: the Poisson matrix of
 * build_cut_cell_poisson_matrix (solver/cut_cell_solver.py:132-216) for face open fractions
 * ax, ay and cell classes, which with 0/1 apertures from a cell mask is the staircase matrix of
 * build_poisson_matrix (solver/mac_solver.py:5-87) that the legacy loop factors (solver/main.py:
 * 194-203, 340-345).  Solved by the boundary-corrected separable inverse with residual
 * refinement; rhs and phi are pressure grids (host or device), rhs ignored and phi zero on
 * covered cells; *residual_linf (may be NULL) receives max |rhs - A phi| (cut-cell rows / kappa). */
typedef struct gm_poisson gm_poisson;
int gm_poisson_create(int32_t nx, int32_t ny, double Lx, double Ly, double D, double xc, double yc, const double* ax,
                      const double* ay, const int32_t* cell_type, const double* kappa, gm_poisson** out);
int gm_poisson_destroy(gm_poisson* p);
const char* gm_poisson_last_error(const gm_poisson* p);
int gm_poisson_solve(gm_poisson* p, const double* rhs, double* phi, double* residual_linf);

/* A legacy loop's state on the device (every array device memory of the current device): the
 * fields and work arrays of the legacy step of solver/main.py:303-381, the cell mask, the inlet
 * profile; for the ghost-cell branch the ghost tables of gm_mac_ghost_apply for the u (0) and
 * v (1) face grids and the circle of the force integral. */
typedef struct gm_legacy_state {
  int32_t nx, ny;
  double dx, dy, nu, rho;
  int32_t slip_walls;
  int32_t centered;   /* 1: centred transport with the loop's AB2 step, p = phi; 0: upwind, p += phi */
  int32_t ghost;      /* 0: staircase branch; 1: ghost-cell branch (GhostCellBoundary) */
  double *u, *v, *p, *u_star, *v_star, *rhs, *phi, *prev_du, *prev_dv;
  const double* zero_p;   /* ny x nx zeros: the pressure the centred predictor reads */
  const uint8_t* mask;    /* ny x nx, nonzero on masked cells */
  const double* inlet;    /* ny inlet values of the step */
  int64_t n_ghost[2];
  const int64_t* target[2];
  const int64_t* src[2];
  const int32_t* snap_of[2];
  const double* weights[2];
  const double* gamma[2];
  const int32_t* level[2];
  int32_t n_levels[2];
  double xc, yc, radius;
  int32_t n_theta;
  int32_t has_prev;   /* the AB2 history (prev_du, prev_dv, prev_dt): read and updated */
  double prev_dt;
} gm_legacy_state;
typedef struct gm_legacy_step_diag {
  double forces[4];               /* fx_p, fy_p, fx_v, fy_v */
  double pressure_residual_linf;  /* max |b - A phi| of the step's pressure solve (scaled rows) */
} gm_legacy_step_diag;
/* n_steps of the legacy loop with the same inlet, on the device: the predictor
 * (predictor_rhs_cpp), ghost velocities (ghost-cell branch), the loop's AB2 step, the
 * right-hand side, the pressure solve of `p` (built over the loop's staircase mask), the
 * corrector (corrector_cpp, or the ghost-cell branch's), the pressure update and the forces
 * (calculate_mac_forces_cpp, or extract_true_surface_forces on the circle).  One stream
 * synchronisation per step, at the pressure gate, before the corrector: a failed solve leaves
 * u, v and p as they were.  Ordered after the work on `stream` (a cudaStream_t or NULL) and
 * before later work there. */
int gm_poisson_legacy_step(gm_poisson* p, gm_legacy_state* s, double dt, int32_t n_steps, gm_legacy_step_diag* diag,
                           void* stream);

/* --- snapshot POD (postprocessing/modal_analysis.py:17-98) ------------------------ */
/* Method of snapshots for M snapshots of N points (row-major M x N, host or device memory):
 * gm_pod_gram forms the time mean (summed over the snapshots in order, like numpy's mean
 * along axis 0) and the Gram matrix C = X' X'^T / M of the fluctuations X' = X - mean, which
 * stay on the device; the caller takes the eigen-decomposition of C (M x M) and passes the
 * first k eigenvectors (M x k, row s = snapshot s) and singular values sigma_q =
 * sqrt(M lambda_q) to gm_pod_modes, which returns the spatial modes X'^T v_q / sigma_q (k x N;
 * zero where sigma_q <= 1e-12) and the temporal coefficients X' phi_q (k x M).  Outputs may be
 * host or device memory; both calls return with them written. */
typedef struct gm_pod gm_pod;
int gm_pod_create(int32_t n_snapshots, int64_t n_points, gm_pod** out);
int gm_pod_destroy(gm_pod* p);
const char* gm_pod_last_error(const gm_pod* p);
int gm_pod_gram(gm_pod* p, const double* snapshots, double* mean, double* gram, void* stream);
int gm_pod_modes(gm_pod* p, const double* eigvecs, const double* sigma, int32_t k, double* modes, double* coeffs,
                 void* stream);

/* --- page-locked host memory (no reference counterpart) ------------------------ */

/* Page-locked host allocation (cudaMallocHost) for arrays that cross the bus every step, such
 * as the facade's state arrays: gm_set_state / gm_get_state then copy them by DMA at full link
 * speed instead of staging pageable memory.  *out = NULL and GM_ECUDA when none can be had
 * (no device); callers then use ordinary memory.  gm_host_free(NULL) is a no-op. */
int gm_host_alloc(size_t bytes, void** out);
int gm_host_free(void* p);

/* --- instrumentation (no reference counterpart) -------------------------------- */

/* Number of CUDA kernels this library has launched in this process. */
int64_t gm_kernel_launches(void);
/* Event times (ms) of the last step run by gm_step when the environment variable
 * GHOSTMAC_PHASE_TIMING=1 was set.  out[0..5]: the phases momentum right-hand side, Helmholtz
 * solves, projection 1, defect, projection 2, pressure output / forces / gates.  out[6..13]:
 * the first sweep of projection 1 between consecutive marks: row pass, column solve, the
 * boundary term's three kernels (point values, Schur GEMV, band values and band solve; with
 * the row-transform chain: band row pass, Schur GEMV, band row pass), the band solve of that
 * chain (empty on the direct path), final row pass, residual.  The events are recorded inside
 * the step graphs, so they time graph-replayed steps. */
int gm_phase_timing(const gm_handle* h, double out[14]);
/* No counterpart in the reference.  How the FP32 mode applies its approximate Helmholtz
 * inverse for the current dt: *jacobi_iters FP32 Jacobi iterations per application (0: the FFT
 * and boundary-Schur inverse) and *jacobi_rho, the row-sum norm of the Jacobi iteration matrix
 * that chose them (0 before the first step, and in the plain FP64 mode).  Either may be NULL. */
int gm_solver_info(const gm_handle* h, int32_t* jacobi_iters, double* jacobi_rho);
/* CUDA-event timing of every launch on the stream it runs on, summed per kernel class:
 * 1 row transforms, 2 column solves, 3 momentum right-hand side, 4 operator residual,
 * 5 Schur GEMV, 6 projection pieces, 7 defect and pressure output, 8 ghost rows,
 * 9 forces and maxima, 10 gates and loop control, 11 FP32 Jacobi iterations of the
 * Helmholtz solves, 12 the FP32 mode's pressure row transforms as tensor-core GEMMs.
 * enable = 1 starts (and clears) timing;
 * every call first folds in the launches made since the last step (after a device
 * synchronisation), then returns the totals of kernel_class so far (time, launches and the
 * launches' algorithmic bytes; any output may be NULL); kernel_class 0 with enable = 0 stops timing.
 * While timing is on, steps run launch by launch (no graphs). */
int gm_kernel_timing(int32_t kernel_class, int32_t enable, double* total_ms, int64_t* count, double* bytes);

/* --- cut-cell AB2/CN path ---------------------------------------------------------------
 * One gm_cc handle holds one cut-cell (embedded-boundary) cylinder case: MAC_CylinderFlow
 * (boundary='cut_cell', time_scheme='ab2_cn') with CutCellBoundary.advance_ab2_cn
 * (solver/cut_cell_solver.py:370-1015).  The geometry-dependent data (fractions, merge tables,
 * owned volumes, the wall and curved-face stencils of solver/cut_cell_geom.py and
 * solver/staggered_wall.py) come from the caller's host setup; the pressure operator, its
 * boundary-corrected inverse, the surface quadrature and every step run in the library.
 * Field layout as for gm_handle; the packed unknown vector q holds the open u faces of columns
 * 1..nx then the open v faces of rows 1..ny-1 (advance_ab2_cn's pack, :962-971). */
typedef struct gm_cc gm_cc;

/* a CSR matrix over the concatenated face field [u.ravel(), v.ravel()] (host arrays) */
typedef struct gm_csr {
  const int64_t* ptr; /* rows + 1 */
  const int64_t* col;
  const double* val;
} gm_csr;

/* Curved faces of one flux family (solver/staggered_wall.py:63-131, 203-232). */
typedef struct gm_cc_faces {
  /* advective fluxes from the fit: flux-array flat index per face, the Gauss points of all
   * faces (grouped by face, in order: adv_patch[p] = face of point p), their u and v value rows
   * and quadrature weights */
  int64_t n_adv, n_adv_points;
  const int64_t* adv_face;
  const int64_t* adv_patch;
  gm_csr adv_u, adv_v;
  const double* adv_len;
  /* viscous fluxes: flux-array flat index per face and its gradient row (the flux is
   * rho nu gradient . field) */
  int64_t n_dif;
  const int64_t* dif_face;
  gm_csr dif_grad;
} gm_cc_faces;

typedef struct gm_cc_config {
  int32_t nx, ny;
  double Lx, Ly, D, xc, yc, nu, rho, U_inf;
  int32_t inflow;  /* 0 uniform, 1 parabolic */
  double U_m;      /* parabolic peak; <= 0 selects 1.5*U_inf */
  int32_t slip_walls;
  /* geometry (solver/cut_cell_geom.py), C order */
  const double* ax;                /* ny x nx+1 open fractions of the u faces */
  const double* ay;                /* ny+1 x nx of the v faces */
  const double* ax_mid;            /* ny x nx */
  const double* ay_mid;            /* ny x nx */
  const double* ay_u;              /* ny+1 x nx+1 */
  const double* ax_v;              /* ny+1 x nx+1 */
  const int32_t* cell_type;        /* ny x nx: 1 fluid, 0 cut, -1 covered */
  const double* volume_fraction;   /* ny x nx */
  const double* u_volume_fraction; /* ny x nx+1 */
  const double* v_volume_fraction; /* ny+1 x nx */
  /* owned volumes and merged volumes (solver/staggered_wall.py:264-299, cut_cell_solver.py:456-468) */
  const double *u_vol, *v_vol, *u_vol_eff, *v_vol_eff;
  int64_t n_u_merge, n_v_merge;
  const int64_t* u_merge;          /* n_u_merge x 4: js, is, jm, im */
  const int64_t* v_merge;
  int64_t n_u_covered, n_v_covered;
  const int64_t *u_covered, *u_owner, *v_covered, *v_owner; /* flat indices of the u / v grid */
  /* wall Gauss points (solver/staggered_wall.py:235-261) */
  int64_t n_wall;
  gm_csr wall_rate;
  const double *wall_tx, *wall_ty, *wall_ds;
  const int64_t *wall_u, *wall_v;  /* owning u / v face (flat index of its grid) */
  gm_cc_faces faces[4];            /* families (u,x) F_xx, (u,y) F_xy, (v,x) F_yx, (v,y) F_yy */
} gm_cc_config;

/* Per-step diagnostics of the cut-cell step (solver/main.py:416-424, time_integration.py:143-145,
 * cut_cell_solver.py:1008-1013). */
typedef struct gm_cc_step_diag {
  double time, dt, max_divergence, cfl;
  double cd, cl, cd_pressure, cd_viscous, cl_pressure, cl_viscous;
  double momentum_residual_linf, coupled_momentum_residual_linf, predicted_divergence;
  double forces[6];                /* fx, fy, fx_p, fy_p, fx_v, fy_v */
  int32_t momentum_iterations;     /* GMRES iterations of the CN solve */
  int32_t pressure_solves;
  int32_t status;                  /* 0 ok, else the GM_E* class of the failure */
  int32_t gate;                    /* GM_GATE_* of the failure, 0 if none */
  double pressure_residual_linf;   /* legacy step: max |b - A phi| of its pressure solve */
  double pressure_residual_l2;     /* legacy step: ||b - A phi||_2 (AB2/CN step: NaN) */
} gm_cc_step_diag;

/* Replaces the cut_cell/ab2_cn branch of MAC_CylinderFlow.__init__ (solver/main.py:140-240):
 * pressure operator and inverse, inlet profile, initial field and its projection. */
int gm_cc_create(const gm_cc_config* cfg, gm_cc** out);
int gm_cc_destroy(gm_cc* c);
/* message of the last error on c (or of the last failed gm_cc_create when c is NULL) */
const char* gm_cc_last_error(const gm_cc* c);
int gm_cc_get_sizes(const gm_cc* c, gm_sizes* out);
/* active flat indices of the u, v and pressure grids (the packed order of q) */
int gm_cc_get_indices(const gm_cc* c, int64_t* ui, int64_t* vi, int64_t* pi);
/* surface quadrature points (y, x) (build_surface_pressure_quadrature, cut_cell_solver.py:70-77) */
int gm_cc_get_surface_points(const gm_cc* c, double* yx);
int gm_cc_set_state(gm_cc* c, const double* u, const double* v, const double* p);
int gm_cc_get_state(gm_cc* c, double* u, double* v, double* p);
int gm_cc_set_inlet(gm_cc* c, const double* u_inlet);
/* restart history of advance_ab2_cn: cn_advection (packed), cn_pressure (p grid), cn_dt */
int gm_cc_set_history(gm_cc* c, int32_t has_history, const double* prev_adv, const double* half_p, double prev_dt);
int gm_cc_get_history(gm_cc* c, int32_t* has_history, double* prev_adv, double* half_p, double* prev_dt);
/* n_steps of advance_ab2_cn with the step gates of solver/main.py:416-424; diag (may be NULL)
 * receives one record per step.  A failed gate stops the loop after that step with its class. */
int gm_cc_step(gm_cc* c, double dt, int32_t n_steps, double start_time, gm_cc_step_diag* diag);
/* n_steps of the legacy cut-cell loop (MAC_CylinderFlow(boundary='cut_cell',
 * time_scheme='legacy'), solver/main.py:297-333): the predictor advance_momentum_predictor
 * (solver/cut_cell_solver.py:1017-1033) with centred transport and AB2 (centered = 1; forward
 * Euler on the first step) or upwind transport and forward Euler (centered = 0), the predictor
 * boundary, the projection and p = phi, then the forces.  The state's inlet column enters the
 * predictor as stored (the previous step's inlet), the current inlet (gm_cc_set_inlet) the
 * boundary and the corrector.  Gates: the pressure divergence budget and finite forces. */
int gm_cc_legacy_step(gm_cc* c, double dt, int32_t n_steps, double start_time, int32_t centered,
                      gm_cc_step_diag* diag);
/* The legacy predictor's history: the previous acceleration on the face grid (u grid then v
 * grid, F doubles) and its timestep (prev_au, prev_av, prev_dt of the reference). */
int gm_cc_set_legacy_history(gm_cc* c, int32_t has_history, const double* prev_accel, double prev_dt);
int gm_cc_get_legacy_history(gm_cc* c, int32_t* has_history, double* prev_accel, double* prev_dt);

/* Event times (ms) of the last step when the environment variable GHOSTMAC_PHASE_TIMING=1 was
 * set at gm_cc_create: out[0..7] = advection, start-up / AB2 and CN right-hand side, GMRES,
 * its residual check, projection 1, CN action and defect, projection 2, outputs (pressure,
 * history, step maxima, forces).  No counterpart in the reference. */
int gm_cc_phase_timing(const gm_cc* c, double out[8]);

#define GM_CC_OP_MOMENTUM_ADVECTION 1 /* (u|v grids) -> a (u|v), y2: rhs; compute_momentum_rhs(u, v, 0, rho) :790-957 */
#define GM_CC_OP_MOMENTUM_DIFFUSION 2 /* same with nu = param and include_advection=False */
#define GM_CC_OP_ADVECTION 3          /* q -> advection(q) of advance_ab2_cn :972-974 */
#define GM_CC_OP_DIFFUSION 4          /* q -> diffusion(q) :975-978 */
#define GM_CC_OP_H_MATVEC 5           /* q -> q - dt/2 (diffusion(q) - diffusion(0)), dt = param */
#define GM_CC_OP_PROJECT 6            /* q -> projected q, y2: phi (p grid); step = param :993-1002 */
#define GM_CC_OP_PRESSURE_SOLVE 7     /* rhs (p grid) -> phi; solve_pressure(rhs, dt = param, rho) :688-730 */
#define GM_CC_OP_MOMENTUM_ADVECTION_UPWIND 8 /* op 1 with transport='upwind' */
int gm_cc_apply(gm_cc* c, int32_t op, double param, const double* x, double* y, double* y2);
/* extract_true_surface_forces (cut_cell_solver.py:755-765): fx, fy, fx_p, fy_p, fx_v, fy_v */
int gm_cc_surface_forces(gm_cc* c, const double* u, const double* v, const double* p, double mu, double out[6]);
/* calculate_cut_cell_divergence (cut_cell_solver.py:219-260) of (u, v), or of the state when
 * both are NULL: max |div|, rms div, max |net flux| over the fluid cells */
int gm_cc_divergence_stats(gm_cc* c, const double* u, const double* v, double out[3]);

#ifdef __cplusplus
}
#endif
#endif /* GHOSTMAC_H */
