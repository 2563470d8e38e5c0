/*
 * clbm_gb300.h -- C ABI of the GB300 (sm_103a) D3Q19 cascaded-LBM + immersed-boundary step.
 *
 * The library replaces the device side of two reference objects:
 *   CLBMSolver      clbm_moving.py:41-343    (fluid state, step, rho/ux/uy/uz fields)
 *   DroneMovingIBM  airfoil_moving.py:44-255 (markers, compute_force, fx/fy/fz fields)
 * Plain pointers and sizes only. Every call returns CLBM_OK (0) or a CLBM_ERR_* code; the
 * message of the last failure on the calling thread is clbm_last_error(). All work is
 * queued on the solver's own CUDA stream; calls that hand results to host memory
 * synchronise that stream. Host arrays use the reference layout: (Nx, Ny, Nz) C order,
 * z fastest, and (Nx, Ny, Nz, 19) for populations.
 */
#ifndef CLBM_GB300_H
#define CLBM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CLBM_OK 0
#define CLBM_ERR_CUDA 1     /* a CUDA runtime call failed */
#define CLBM_ERR_ARG 2      /* invalid argument or configuration */
#define CLBM_ERR_DIVERGED 3 /* non-finite or rho < threshold (clbm_check, device monitor) */
#define CLBM_ERR_STATE 4    /* call not valid in the current state */

/* Entries of an IBM's lift/drag history ring (the last this many compute_force calls). */
#define CLBM_HISTORY_CAPACITY 65536

/* Population storage forms. F32 stores f_q; the shifted forms store f_q - w_q. */
#define CLBM_STORE_F32 0
#define CLBM_STORE_F16S 1
#define CLBM_STORE_BF16S 2

typedef struct clbm_solver clbm_solver;
typedef struct clbm_ibm clbm_ibm;

/* Lattice and collision parameters (config_moving.py:28-43, clbm_moving.py:32-35). */
typedef struct clbm_config {
    int32_t nx, ny, nz;     /* lattice, nx >= 3 */
    double s_v;             /* shear rate 1/tau */
    double s_e;             /* trace (bulk) rate; the reference fixes s_q = s_pi = 1 */
    double ux_in, uy_in;    /* Zou-He inlet velocity; also the initial equilibrium */
    int32_t storage;        /* CLBM_STORE_* */
    int32_t device;         /* CUDA device ordinal the solver lives on */
} clbm_config;

/* Prescribed motion (main_moving.py:62-74; config_moving.py:312-318), double precision:
 * xc = x0, yc = y0 + a_heave sin(w t), theta = aoa0 + a_pitch sin(w t + phi_pitch),
 * vx = 0, vy = a_heave w cos(w t), omega = a_pitch w cos(w t + phi_pitch). */
typedef struct clbm_motion {
    double x0, y0, a_heave, a_pitch, phi_pitch, aoa0, w;
} clbm_motion;

/* CLBMSolver.__init__ + _init_feq (clbm_moving.py:54-91): allocate the state and set
 * f = feq(rho = 1, u = (ux_in, uy_in, 0)). */
int clbm_create(const clbm_config* cfg, clbm_solver** out);
int clbm_destroy(clbm_solver* s);

/* CLBMSolver.step(fx, fy, fz) (clbm_moving.py:326-343) with the force fields that the
 * last ibm_compute_force on `ibm` produced (DroneMovingIBM.fx/fy/fz after _clip_forces).
 * ibm == NULL steps with zero force. */
int clbm_step(clbm_solver* s, const clbm_ibm* ibm);

/* CLBMSolver.step with caller-supplied force density fields in device memory, reference
 * layout (Nx, Ny, Nz) float32, used as given (no clip), fz may be NULL. */
int clbm_step_dense_force(clbm_solver* s, const float* fx_dev, const float* fy_dev,
                          const float* fz_dev);

/* Same as clbm_step_dense_force with the three fields in host memory (fz may be NULL);
 * the copies to the device are part of the call. */
int clbm_step_host_force(clbm_solver* s, const float* fx, const float* fy, const float* fz);

/* lbm.rho/ux/uy/uz.to_numpy() (main_moving.py:125-128): macroscopic fields of the
 * current post-stream state without force correction (_macro_post,
 * clbm_moving.py:305-321) copied to host arrays (any may be NULL). */
int clbm_read_macro(clbm_solver* s, float* rho, float* ux, float* uy, float* uz);

/* z-vorticity of plane z as the reference's renderers compute it from lbm.ux/uy
 * (render_2d.py:272-275): d(ux)/dy - d(uy)/dx with NumPy gradient rules (central inside,
 * one-sided at the edges), into host out[Nx * Ny] ((Nx, Ny), y fastest). */
int clbm_read_vorticity_slice(clbm_solver* s, int32_t z, float* out);

/* lbm.f.to_numpy(): post-stream, post-boundary populations (Nx, Ny, Nz, 19) float32. */
int clbm_read_populations(clbm_solver* s, float* f_host);
/* lbm.f.from_numpy(): replace the state by host populations (Nx, Ny, Nz, 19). Clears the
 * device status word (a new state starts with a clean divergence record). */
int clbm_write_populations(clbm_solver* s, const float* f_host);

/* Divergence statistics of the current state (main_moving.py:130-145): rho min/max,
 * max |u| and the count of non-finite rho/u values. Returns CLBM_ERR_DIVERGED when
 * nonfinite > 0 or rho_min < rho_floor, or when the device divergence monitor (see
 * clbm_set_rho_floor) recorded a bad density since the state was last written. */
int clbm_check(clbm_solver* s, double rho_floor, double* rho_min, double* rho_max,
               double* u_max, int64_t* nonfinite);

/* DroneMovingIBM.__init__ (airfoil_moving.py:64-95): marker template, X0/Y0 in the body
 * frame, Z0 absolute; n >= 0. The IBM is bound to one solver's lattice and stream. */
int ibm_create(clbm_solver* s, const float* X0, const float* Y0, const float* Z0, int32_t n,
               clbm_ibm** out);
int ibm_destroy(clbm_ibm* ibm);

/* DroneMovingIBM.compute_force(lbm.ux, lbm.uy, xc, yc, theta, vx, vy, omega)
 * (airfoil_moving.py:230-255): marker kinematics, Peskin 4-point interpolation of the
 * solver's current velocity, marker force clip, spreading and Eulerian clip. The six
 * motion values are truncated to float32 as the reference's kernel arguments are. */
int ibm_compute_force(clbm_ibm* ibm, double xc, double yc, double theta, double vx,
                      double vy, double omega);

/* Same as ibm_compute_force with the motion state of main_moving.py:_motion_state(t)
 * evaluated on the device in double for t = (number of compute_force calls so far) + 1. */
int ibm_compute_force_motion(clbm_ibm* ibm, const clbm_motion* m);

/* ibm.fx/fy/fz.to_numpy(): the clipped Eulerian force fields (Nx, Ny, Nz) (any NULL). */
int ibm_read_forces(const clbm_ibm* ibm, float* fx, float* fy, float* fz);

/* Marker arrays of the last compute_force: X, Y, Z, VX_body, VY_body, U_k, V_k, FX_k,
 * FY_k, each n floats, concatenated in that order into out[9 * n]. */
int ibm_read_markers(const clbm_ibm* ibm, float* out);

/* Lift/drag support (not in the reference): per compute_force call, double sums of the
 * clipped Eulerian force over all cells (sx, sy) and of the marker forces (mx, my).
 * Reads the last `count` entries (oldest first) of the device history ring into
 * out[4 * count]; the force on the body is minus these sums. */
int ibm_read_force_history(const clbm_ibm* ibm, int32_t count, double* out);
/* Number of compute_force calls made on this IBM (the device step counter). */
int ibm_step_count(const clbm_ibm* ibm, int64_t* out);

/* ---- Checkpoint / resume (no counterpart: the reference's frames hold rho and u only,
 * main_moving.py:124-200, so its runs cannot be resumed) ----------------------------------
 * The solver's state is its population buffer as stored (padded layout, storage form) and
 * its macro fields: clbm_state_bytes gives the size, clbm_save_state copies it to host
 * memory with *flags (bit 0: the buffer holds a post-stream state, bit 1: the macro fields
 * are those of that state), clbm_load_state puts it back into a solver of the same lattice
 * and storage form. An IBM's state is its call counter and its history:
 * ibm_load_state(ibm, calls, hist, count) sets the counter to `calls` (the motion law's
 * step), writes the last `count` history entries (4 doubles each, as
 * ibm_read_force_history returns them; count <= min(calls, CLBM_HISTORY_CAPACITY)) and
 * clears the force fields, which the next compute_force writes again. A run resumed from
 * a saved step continues bit for bit as the run that was saved. */
int clbm_state_bytes(const clbm_solver* s, int64_t* bytes);
int clbm_save_state(clbm_solver* s, void* out, int64_t bytes, int32_t* flags);
int clbm_load_state(clbm_solver* s, const void* in, int64_t bytes, int32_t flags);
int ibm_load_state(clbm_ibm* ibm, int64_t calls, const double* hist, int32_t count);

/* No counterpart in the reference. Allocation-free force sums for callers that cannot call
 * cudaMalloc when they need lift/drag: real-time loops whose device memory budget is fixed
 * up front, and hosts whose device memory belongs to a pool allocator they cannot reach.
 * Computes the same sums as one entry of ibm_read_force_history -- sum of fx, fy clipped
 * to +-0.05 over all cells, and sum of FX_k, FY_k -- over caller-owned device arrays fx, fy
 * in the reference layout (Nx, Ny, Nz) and FXk, FYk (n markers; may be NULL when n == 0),
 * written to host out[4]. Runs on `stream` (a cudaStream_t; NULL for the default stream)
 * and is synchronous: it copies the sums to host memory and waits for `stream` before it
 * returns. It must therefore run outside stream capture: a call on a stream that is being
 * captured is refused with CLBM_ERR_STATE before any work is issued (the capture stays
 * valid). Its scratch is a fixed file-scope device array that every GPU loading this
 * library holds until exit; lattices above 67,108,864 cells are rejected with
 * CLBM_ERR_ARG. All calls on a device share the array: calls that overlap on the GPU (on
 * different streams or host threads) race and must not be made. A CUDA error already
 * pending from the caller's own work is reported (CLBM_ERR_CUDA) and left pending. The
 * array's device address is looked up on the first call on each device and kept, so
 * cudaDeviceReset is not supported while this library is in use. */
int ibm_force_sums_noalloc(const float* fx, const float* fy, int32_t nx, int32_t ny, int32_t nz,
                           const float* FXk, const float* FYk, int32_t n, void* stream,
                           double* out);

/* The driver loop of main_moving.py:116-122 for nsteps steps: per step
 * ibm_compute_force_motion then clbm_step. use_graph != 0: eight steps are captured once
 * into a CUDA graph (motion law on the device) and replayed; a remainder below eight runs as
 * direct launches (motion law on the host). ibm may be NULL (zero force). Graph replays
 * stop themselves on divergence (main_moving.py:143-145): each replay copies the device
 * status word to pinned host memory, at most four replays are in flight, and when the
 * divergence monitor has fired the call returns CLBM_ERR_DIVERGED within five replays (40
 * steps) of the step that diverged. */
int clbm_run(clbm_solver* s, clbm_ibm* ibm, const clbm_motion* m, int32_t nsteps,
             int32_t use_graph);

/* Batched ensemble (no counterpart in the reference, which runs one case per process):
 * many independent solvers, each with its own IBM (or NULL) and motion law, stepped
 * together -- each step is six batched launches over all members (markers, force-box
 * offsets, band macro, interpolation/spreading, force sums, force-box pass) and the bulk
 * stream-collide over every member's cells (one launch over a flat tile list, one launch
 * per row width, or one single-lattice launch per member, run concurrently; timed at
 * creation), or one persistent launch when the ensemble is
 * created with CLBM_ENS_STEP=persistent (clbm_ensemble_schedule). Members keep their buffers and
 * all per-member reads (clbm_read_macro, ibm_read_force_history, ...) keep working; the
 * members must be fresh or at the same step, share storage form and device, and outlive
 * the ensemble. clbm_ensemble_create times the bulk-pass tile width and block schedule
 * and keeps the fastest (clbm_ensemble_tuning reports them). */
typedef struct clbm_ensemble clbm_ensemble;
int clbm_ensemble_create(clbm_solver* const* solvers, clbm_ibm* const* ibms,
                         const clbm_motion* motions, int32_t n, clbm_ensemble** out);
/* nsteps steps of every member (main_moving.py:116-122 with the motion law evaluated on the
 * device), as a two-step CUDA graph replay when use_graph != 0. */
int clbm_ensemble_run(clbm_ensemble* e, int32_t nsteps, int32_t use_graph);
int clbm_ensemble_stream(const clbm_ensemble* e, void** out);
/* The bulk-pass schedule chosen at creation: tile width (cells; 0: whole rows per block,
 * members grouped by row width, one launch per group; -1: one single-lattice launch per
 * member over concurrent streams, blocks = tiles = members), blocks, tiles, the time of one
 * bulk pass of all members with it, alone, in milliseconds, and in the row mode the rows
 * one block computes per tile (0 otherwise). Any pointer may be NULL. */
int clbm_ensemble_tuning(const clbm_ensemble* e, int32_t* tile_width, int32_t* blocks,
                         int64_t* tiles, float* bulk_ms, int32_t* rows_per_block);
/* Step form of the ensemble: *persistent = 1 when each step is one persistent cooperative
 * launch (every block resident; the IBM phases separated by a grid barrier with bounded
 * waits, the bulk pass's tiles shared out over the phases), chosen by the environment
 * variable CLBM_ENS_STEP=persistent when the ensemble is created (at most 128 members:
 * their constants travel in the launch's parameter table), with *blocks its grid;
 * 0 and 0 for separate launches. Both forms give the same bits. A barrier wait that ran
 * out is reported by the next clbm_ensemble_run (CLBM_ERR_STATE). Any pointer may be
 * NULL. */
int clbm_ensemble_schedule(const clbm_ensemble* e, int32_t* persistent, int32_t* blocks);
/* Phase clock of the last persistent step, in microseconds (5 entries): markers; box
 * offsets + bulk share; band prepare + bulk share; interpolation/spreading + bulk share; and
 * force sums, box pass and the rest of the bulk pass as seen by block 0 (the launch ends
 * when its last block does). Waits for the ensemble's stream. CLBM_ERR_STATE for separate
 * launches. */
int clbm_ensemble_phase_times(clbm_ensemble* e, double* us);
int clbm_ensemble_destroy(clbm_ensemble* e);

/* Wait for all queued work of the solver. Returns CLBM_ERR_STATE when a bounded device
 * wait gave up, CLBM_ERR_DIVERGED when the divergence monitor fired. */
int clbm_synchronize(clbm_solver* s);

/* Divergence monitor (the device form of main_moving.py:143-145, which stops a run when
 * rho_min < 0.3 or a field is not finite): every collision of every step compares its
 * cell's density with this floor, and a density below it or not finite sets a sticky
 * bit of the device status word, reported by clbm_synchronize, clbm_check and clbm_run.
 * Default 0.3; a negative floor keeps only the non-finite test. Set it before creating an
 * ensemble that holds this solver (the ensemble copies the coefficients). No reference
 * counterpart beyond the host check it replaces. */
int clbm_set_rho_floor(clbm_solver* s, double rho_floor);

/* Failure-detection self test (no counterpart in the reference, which has no device
 * waits): runs one launch of the shared-memory-staged stream-collide kernel whose block
 * barrier expects 16 bytes more than are ever copied, so each block's bounded wait gives
 * up after `spin_limit` (>= 1024) polls and sets the device status word instead of hanging. Returns
 * CLBM_ERR_STATE when the timeout was reported (the expected outcome), leaves the state
 * unchanged (no block writes results) and clears the status word. */
int clbm_selftest_wait_timeout(clbm_solver* s, int32_t spin_limit);

/* Bounds-checked build (the same library compiled with -DCLBM_CHECK, a debug build for
 * finding out-of-range accesses without a sanitizer): the population, force-field,
 * macro-field and stencil accesses of the stream-collide, band and IBM kernels test their
 * index first; one outside its array is skipped and reported by clbm_synchronize
 * (CLBM_ERR_STATE). clbm_bounds_checked tells which build is loaded (*on = 1: checked);
 * clbm_selftest_bounds makes one index test past the end (no access) and returns
 * CLBM_ERR_STATE when it was reported (the expected outcome; CLBM_ERR_STATE also in the
 * normal build, where there is nothing to test). */
int clbm_bounds_checked(int32_t* on);
int clbm_selftest_bounds(clbm_solver* s);

/* Failure-detection self test of the persistent ensemble step's grid barrier: a
 * cooperative launch of `blocks` (1..16) blocks whose barrier waits for one block more than
 * the launch has, so every block's bounded wait gives up (well under a second) and sets the
 * error bits instead of hanging. Returns CLBM_ERR_STATE when the timeout was reported (the
 * expected outcome). */
int clbm_selftest_grid_barrier(int32_t blocks);

/* The solver's CUDA stream (cudaStream_t), for callers that record events or order their
 * own work against the solver. The stream stays owned by the solver. An IBM step runs its
 * bulk pass on a second stream and leaves it running there, so the next compute_force's
 * marker kernel overlaps it; every later call on the solver or its IBMs, the end of
 * clbm_run, clbm_synchronize and this call join it into the solver stream first, so work
 * queued before this call is complete on the returned stream. */
int clbm_stream(const clbm_solver* s, void** out);

/* Kernel timing for roofline reporting: while enabled, each fused stream-collide launch is
 * bracketed by CUDA events on the solver stream. clbm_profile_read synchronises and
 * returns the summed device time (ms) and launch count of the fused kernel since the last
 * enable, and the total number of kernels this solver launched since creation. */
int clbm_profile_enable(clbm_solver* s, int32_t on);
int clbm_profile_read(clbm_solver* s, double* fused_ms, int64_t* fused_launches,
                      int64_t* total_launches);
/* The same device time split by pass: an IBM step launches a bulk pass over the cells
 * outside the force box and a box pass over the cells inside it; other steps count as
 * bulk. */
int clbm_profile_read_split(clbm_solver* s, double* bulk_ms, int64_t* bulk_launches,
                            double* box_ms, int64_t* box_launches);

/* Bytes of device memory owned by the solver (populations, macro fields). */
int clbm_device_bytes(const clbm_solver* s, int64_t* out);

/* Full-grid stream-collide kernel chosen at creation (0 one cell per thread, 1 two cells
 * per thread, 2 rows staged in shared memory) and, when ms_per_launch is not NULL (3
 * entries), the autotune time per launch of each variant in milliseconds (0 for variants
 * not timed:
 * lattices below 2^20 cells and forced choices skip the timing). No reference
 * counterpart: the reference has one kernel per phase (clbm_moving.py:326-343). */
int clbm_kernel_variant(const clbm_solver* s, int32_t* variant, float* ms_per_launch);

/* Architecture of the loaded device code as the CUDA runtime reports it for the bulk
 * stream-collide kernel (cudaFuncGetAttributes): *binary = major * 10 + minor of the SASS
 * (103 for sm_103a), *ptx the PTX version it was generated from. Needs a GPU. */
int clbm_binary_version(int32_t* binary, int32_t* ptx);

/* ---- Learned sub-grid closure --------------------------------------------------------
 * A 19 -> 32 -> 32 -> 1 network (GELU, BF16 weights, FP32 accumulation) maps the 19
 * normalised non-equilibrium central moments of a cell to the relaxation rate s_h of its
 * third- and fourth-order central moments, which the reference relaxes fully (s_q = s_pi
 * = 1 in _collide, clbm_moving.py:186-194). Not part of the reference.
 *
 * Parameter array offsets (floats): out[0..18] = mu, sinv, W1, b1, W2, b2, W3, b3, span,
 * total, inputs (19), hidden width (32), higher-order targets per sample (9), trainable
 * count, floats per training sample (38), mode, nu, sub-grid stress values per sample
 * (10), statistics count (40). mode 0: the rate of the third/fourth-order moments,
 * s_h = 1 + span tanh(z3); mode 1: an eddy viscosity, the deviatoric second-order moments
 * relax with 1 / (1/2 + 3 nu 2^(span g)), g = tanh(z3) where positive and tanh(z3) / 20
 * below, nu the solver's viscosity (the nu entry is the viscosity the training assumes). */
int clbm_closure_layout(int32_t* out);

/* Enable the closure for the bulk pass of later steps (params: host array of the layout
 * above, copied), or disable it (params NULL: the plain cascaded collision, the
 * fallback). Cells of the IBM force box and dense-force steps keep the plain collision. */
int clbm_closure_set(clbm_solver* s, const float* params);

/* Trainer: samples from box-filtered fields of a fine lattice (twice the coarse one in
 * each direction, float32 storage) and Adam training on the device. Sample i holds 19
 * features (moments of the filtered pre-collision state), 9 higher-order targets (moments
 * of the ideal post-collision state f*_q(x) = f_q(x + e_q) one coarse step later) and 10
 * sub-grid stress values (deviatoric parts of tau = <u u> - <u><u> of the filtered fine
 * velocity and of the filtered strain rate). fine may be NULL (samples written by the
 * caller). */
typedef struct clbm_trainer clbm_trainer;
int clbm_trainer_create(int32_t device, const clbm_solver* fine, int64_t capacity, clbm_trainer** out);
int clbm_trainer_destroy(clbm_trainer* t);
/* Filter the fine lattice's current post-stream state into slot 0 or 1. */
int clbm_trainer_capture(clbm_trainer* t, int32_t slot);
/* A captured slot in the reference layout (nx/2, ny/2, nz/2, 28), z fastest: 19 filtered
 * populations, the filtered velocity (3) and velocity products (xx, yy, zz, xy, xz, yz). */
int clbm_trainer_read_slot(clbm_trainer* t, int32_t slot, float* out);
/* Append samples at coarse cells (x + nx (y + ny z), 1 <= x <= nx - 2) from slots 0 -> 1. */
int clbm_trainer_extract(clbm_trainer* t, const int64_t* cells, int64_t n);
int clbm_trainer_count(const clbm_trainer* t, int64_t* n);
/* Samples as [n][38] host rows. */
int clbm_trainer_write_samples(clbm_trainer* t, int64_t off, int64_t n, const float* in);
int clbm_trainer_read_samples(clbm_trainer* t, int64_t off, int64_t n, float* out);
/* Sums of the 19 features, of their squares, of the squared third/fourth-order features
 * and of the squared deviatoric sub-grid stress over a sample range (40 doubles). */
int clbm_trainer_stats(clbm_trainer* t, int64_t off, int64_t n, double* out);
/* Loss summed over a sample range: mode 0, sum_j (t_j - (1 - s_h) p_j)^2 over the nine
 * higher-order moments; mode 1, sum_j (tau_j + 2 nu_t S_j)^2 over the five deviatoric
 * components; times wscale. */
int clbm_trainer_loss(clbm_trainer* t, const float* params, int64_t off, int64_t n, float wscale,
                      double* loss_sum);
/* Gradient of the mean loss over a sample range w.r.t. W1, b1, W2, b2, W3, b3 (in the
 * order of the parameter array from W1 on). */
int clbm_trainer_grad(clbm_trainer* t, const float* params, int64_t off, int64_t n, float wscale,
                      float* grad, double* loss_sum);
/* Adam with a cosine learning-rate decay over random minibatches of a sample range;
 * params updated in place; loss_hist (iters doubles, may be NULL) gets minibatch sums. */
int clbm_trainer_fit(clbm_trainer* t, float* params, int64_t off, int64_t n, int32_t iters, int64_t batch,
                     float lr, float wscale, uint64_t seed, double* loss_hist);
/* Tensor-core self test: D (128 x n) = A (128 x kdim) B^T (n x kdim), BF16 operands,
 * kdim 32 or 128, n 32 or 112 (the operand layouts of the closure kernels). */
int clbm_tc_selftest(int32_t device, const float* A, const float* B, float* D, int32_t kdim, int32_t n);

/* Page-locked host buffers for fast transfers. */
int clbm_host_alloc(int64_t bytes, void** out);
int clbm_host_free(void* p);

/* Message of the last failing call on this thread ("" if none). */
const char* clbm_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* CLBM_GB300_H */
