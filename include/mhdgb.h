/*
 * mhdgb — C ABI of the GB300-native 3D incompressible MHD right-hand side and RK4 / LSRK4 step.
 *
 * This is the drop-in boundary for MHDFlows.jl's MHD hot path.  Each entry point replaces one
 * piece of the reference's interface (paths are inside the MHDFlows.jl project):
 *
 *   mhd_create / mhd_destroy   Problem(dev; nx, Lx, nu, eta, nnu, B_field=true, stepper, T=Float32, dt)
 *                              src/pgen.jl:64-127, src/Problems.jl:118-140 (grid, vars, params,
 *                              equation with L = 0, time stepper, sol = zeros(nkr, n, n, 6))
 *   mhd_set_physical           SetUpProblemIC!(prob; ux, uy, uz, bx, by, bz)  src/utils/IC.jl:41-109
 *                              (host physical field -> device -> forward r2c into sol)
 *   mhd_set_state / get_state  prob.sol (nkr, n, n, 6) ComplexF32, column-major  src/Problems.jl:130
 *   mhd_step                   stepforward!(prob.sol, clock, ts, eqn, vars, params, grid)
 *                              src/timestepper/timestepper.jl:4-6 (FourierFlows RK4 / LSRK4 calling
 *                              MHDcalcN! src/pgen.jl:153-162 -> MHDcalcN_advection!
 *                              src/Solver/MHDSolver.jl:330-351), clock.t += dt, clock.step += 1
 *   mhd_compute_rhs            eqn.calcN!(N, sol, t, clock, vars, params, grid)  src/pgen.jl:153-162
 *   mhd_get_physical           updatevars!(prob): vars.ux..bz <- irfft(sol)  (exported but never
 *                              defined in the reference, src/Solver/MHDSolver.jl:10; refreshed there
 *                              only as a side effect of calcN!, src/Solver/MHDSolver.jl:333-338)
 *   mhd_diagnostics            ProbDiagnostic src/utils/UserInterface.jl:29,65-86 (KE, ME = sum|.|^2 dV),
 *                              Div src/utils/VectorCalculus.jl:72-94 (div B), cross-helicity (new)
 *   mhd_get_clock / set_clock  prob.clock (t, step, dt)  src/Problems.jl:123
 *   mhd_last_error             the message of Julia's error(...) at the failing call
 *
 * Conventions: every function returns MHD_OK (0) or an MHD_ERR_* code and sets a thread-local
 * message readable with mhd_last_error().  Host arrays are plain pointers in the reference's
 * column-major layout; complex values are interleaved float pairs.  A handle owns all of its
 * device memory and one CUDA stream; calls on one handle are not thread-safe, calls on different
 * handles are.  Nothing here calls back into the host language.
 */
#ifndef MHDGB_H
#define MHDGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MHD_OK 0
#define MHD_ERR_INVALID 1     /* bad argument (size, field index, null pointer, unsupported n) */
#define MHD_ERR_CUDA 2        /* CUDA runtime error (launch failure, device fault) */
#define MHD_ERR_OOM 3         /* device or pinned-host allocation failed */
#define MHD_ERR_NONFINITE 4   /* diagnostics found NaN/Inf in the state */
#define MHD_ERR_STATE 5       /* call not valid in the handle's current state */

#define MHD_RK4 0
#define MHD_LSRK4 1

#define MHD_PREC_FP32 0        /* FP32 everywhere (the reference's T = Float32) */
#define MHD_PREC_SPLIT_FP16 1  /* x-row transforms as tensor-core DFT products, FP16 hi+lo operands */
#define MHD_PREC_SPLIT_BF16 2  /* the same with BF16 hi+lo operands (n = 128, 256, 512 only) */
#define MHD_PREC_SPLIT_TF32 3  /* x-row transforms as tcgen05 tensor-core DFT products with TF32 hi+lo
                                  operands, data operand in tensor memory (n = 256 only) */

typedef struct mhd_params {
  int n;          /* grid points per axis (nx = ny = nz); supported: 16,32,48,64,96,128,256,512 */
  double L;       /* box side (Lx = Ly = Lz), default 2*pi */
  double nu;      /* viscosity */
  double eta;     /* resistivity */
  int nnu;        /* hyper-viscosity order; values > 1 are rejected (the MHD path uses nnu <= 1) */
  int neta;       /* hyper-resistivity order; values > 1 are rejected */
  double dt;      /* fixed time step */
  int scheme;     /* MHD_RK4 or MHD_LSRK4 */
  int precision;  /* MHD_PREC_FP32, MHD_PREC_SPLIT_FP16, MHD_PREC_SPLIT_BF16 or MHD_PREC_SPLIT_TF32 */
  int device;     /* CUDA device ordinal */
  int hydro_only; /* 0: MHD (B_field = true, 6 fields); 1: hydrodynamics (B_field = false,
                     HDcalcN! of src/pgen.jl:176-182: 3 fields ux, uy, uz; the state layout of
                     set/get_state is then (nkr, n, n, 3) and field indices are 0..2) */
  int vp;         /* 1: volume penalisation (VP_method = true, see mhd_set_vp); 0: off */
} mhd_params;

typedef struct mhd_problem* mhd_handle;
typedef struct mhd_ensemble_s* mhd_ensemble;

/* Problem construction (Problem(GPU(); ...), src/pgen.jl:64-127). */
int mhd_create(const mhd_params* params, mhd_handle* out);
int mhd_destroy(mhd_handle h);

/* Supported grid sizes; returns 1 if n is supported. */
int mhd_supported_n(int n);

/* Kept (de-aliased) mode counts for size n: kx modes on the rfft axis, kp non-negative and kn
 * negative modes on each full axis (FourierFlows getaliasedwavenumbers with aliased_fraction 1/3). */
int mhd_kept_modes(int n, int* kx, int* kp, int* kn);

/* prob.sol <-> host: complex64 interleaved, column-major (nkr, n, n, 6), nkr = n/2+1.
 * set_state keeps only the retained (de-aliased) band; get_state writes zeros in the alias band. */
int mhd_set_state(mhd_handle h, const float* sol);
int mhd_get_state(mhd_handle h, float* sol);

/* prob.sol as a device array (a CuArray of MHDFlows' Problem(GPU(); ...), src/Problems.jl:130,
 * whose stepforward! updates it in place, src/timestepper/timestepper.jl:4-6): the same layout as
 * mhd_set_state, 16-byte aligned device memory, read or written by a kernel on the device.
 * The kernel runs on `stream`, the caller's cudaStream_t (0 is the legacy default stream; pass
 * mhd_get_stream(h) to stay on the handle's stream), after the handle's earlier work, and the
 * handle's later work waits for it.  Neither call synchronises the host: work the caller issues
 * on `stream` afterwards sees the transfer complete.  get_state_device writes every element
 * (zeros in the alias band). */
int mhd_set_state_device(mhd_handle h, const float* sol_dev, void* stream);
int mhd_get_state_device(mhd_handle h, float* sol_dev, void* stream);

/* SetUpProblemIC!: physical field (n, n, n) float32 column-major -> forward r2c into sol[:,:,:,field]. */
int mhd_set_physical(mhd_handle h, int field, const float* phys);
/* updatevars!: vars.<field> <- normalised c2r of sol[:,:,:,field]. field 0..5 = ux uy uz bx by bz. */
int mhd_get_physical(mhd_handle h, int field, float* phys);

/* stepforward! x nsteps (clock.t += dt, clock.step += 1 per step). Asynchronous on the handle's
 * stream; errors of the launches are reported, device faults surface at the next synchronising call. */
int mhd_step(mhd_handle h, int nsteps);

/* calcN!(N, sol, ...): one right-hand-side evaluation of the current state, written to rhs_out
 * in the prob.sol layout (alias band zero). */
int mhd_compute_rhs(mhd_handle h, float* rhs_out);

/* Clock access. */
int mhd_get_clock(mhd_handle h, double* t, long long* step, double* dt);
int mhd_set_clock(mhd_handle h, double t, long long step, double dt);

/* Diagnostics of the current state (FP64 accumulation on the device):
 * out[0] E_u = sum |u|^2 dV      out[1] E_B = sum |B|^2 dV       (the reference's KE, ME; no 1/2)
 * out[2] H_c = sum u.B dV        out[3] max|k.u_hat|             out[4] max|k.B_hat|
 * out[5] max|div B| (physical)   out[6] non-finite value count   out[7] t
 * nout >= 8. Returns MHD_ERR_NONFINITE (after filling out) if the state holds NaN/Inf. */
int mhd_diagnostics(mhd_handle h, double* out, int nout);

/* getCFL! of TimeIntegrator! (src/integrator.jl:54-58, 158-198) on the device.  While enabled,
 * every step ends with dt = min(coef * dx / vmax, t_diff), vmax = max of |u_i| and |B_i| over
 * the physical fields of the step's last stage (the fields the reference's getCFL! reads from
 * vars), t_diff = coef * dx^2 / max(nu, eta); the clock t then advances on the device and no
 * step synchronises with the host.  Enabling primes vmax from the current state.  Applies to
 * every slot of the handle. */
int mhd_set_cfl(mhd_handle h, int enable, double coef);

/* Wait for all work of the handle. */
int mhd_synchronize(mhd_handle h);

/* Use an external CUDA stream (cudaStream_t) for this handle's work; NULL restores its own. */
int mhd_set_stream(mhd_handle h, void* stream);
void* mhd_get_stream(mhd_handle h);

/* Device bytes held by the handle (state, stage arrays, pass buffers, staging). */
int mhd_memory_bytes(mhd_handle h, long long* bytes);
/* Device bytes a handle of these parameters would hold, without allocating. */
int mhd_footprint_bytes(const mhd_params* params, long long* bytes);

/* Pinned host memory for fast transfers. */
int mhd_host_alloc(size_t bytes, void** ptr);
int mhd_host_free(void* ptr);

/* Per-kernel timing with CUDA events on the handle's stream.  While enabled, mhd_step brackets
 * every launch with events; mhd_profile_read returns, per kernel class, the launch count and the
 * summed device milliseconds since the last enable.  Classes are named by mhd_kernel_class_name. */
int mhd_profile_enable(mhd_handle h, int enable);
int mhd_profile_read(mhd_handle h, long long* launches, double* ms, int nclass);
const char* mhd_kernel_class_name(int cls);
int mhd_kernel_class_count(void);
/* Algorithmic HBM bytes one launch of a kernel class moves for this handle's size. */
int mhd_kernel_class_bytes(mhd_handle h, int cls, double* bytes);

/* ---- Batched solves (no counterpart in the reference, which runs one problem per process).
 * A batch handle is a size class: `capacity` slots of one grid size n, box L and scheme, whose
 * state stays resident in HBM.  mhd_step on a batch advances every active slot by one step in
 * the same launches (persistent kernels walk the active (slot, tile) work-list); each slot has
 * its own nu, eta, dt and clock.  mhd_create is the capacity-1 case with slot 0 active, and the
 * single-problem functions above act on slot 0.  Results of a slot do not depend on which other
 * slots are active (no reduction crosses slots). */
int mhd_batch_create(const mhd_params* params, int capacity, mhd_handle* out);
int mhd_batch_add(mhd_handle h, double nu, double eta, double dt, int* slot);   /* state zeroed */
int mhd_batch_remove(mhd_handle h, int slot);
int mhd_batch_info(mhd_handle h, int* capacity, int* active);
/* Device bytes of one slot and of a size class's shared staging (admission control). */
int mhd_slot_bytes(const mhd_params* params, long long* per_slot, long long* per_class);
int mhd_slot_set_state(mhd_handle h, int slot, const float* sol);
int mhd_slot_get_state(mhd_handle h, int slot, float* sol);
int mhd_slot_set_state_device(mhd_handle h, int slot, const float* sol_dev, void* stream);
int mhd_slot_get_state_device(mhd_handle h, int slot, float* sol_dev, void* stream);
int mhd_slot_set_physical(mhd_handle h, int slot, int field, const float* phys);
int mhd_slot_get_physical(mhd_handle h, int slot, int field, float* phys);
int mhd_slot_diagnostics(mhd_handle h, int slot, double* out, int nout);
int mhd_slot_get_clock(mhd_handle h, int slot, double* t, long long* step, double* dt);
int mhd_slot_set_clock(mhd_handle h, int slot, double t, long long step, double dt);

/* Serving: a continuous-batching scheduler over size classes (no counterpart in the reference,
 * which runs one problem per process).  Requests of any supported n queue in arrival order; a
 * request is admitted when its size class has a free slot or a new class fits the device-memory
 * budget (first fit), runs in the same launches as every other active solve of its class, and
 * retires with its diagnostics (and its final state when keep_states) when its steps are done.
 * The caller drives it: mhd_server_tick admits what fits, advances every active solve by
 * min(steps_per_tick, the smallest remaining step count) and retires the finished ones.
 * A request whose class can never fit the budget, whose class allocation fails, or whose initial
 * state is not finite is rejected / failed alone; mhd_server_cancel frees a slot at once. */
typedef struct mhd_server_s* mhd_server;
typedef struct mhd_server_params {
  double budget_bytes;   /* device memory the size classes may reserve */
  int steps_per_tick;    /* upper bound of the steps one tick advances */
  int scheme;            /* MHD_RK4 or MHD_LSRK4, for every request */
  int device;
  int keep_states;       /* 1: keep each finished request's final state for mhd_server_result */
  int capacity[8];       /* slots per class for n = 16, 32, 48, 64, 96, 128, 256, 512 (0: default) */
} mhd_server_params;
typedef struct mhd_request {
  int n;                 /* grid size (cubic box of side L) */
  double L, nu, eta;
  double dt;             /* <= 0: 0.2 * L / n */
  long long steps;
  const float* sol;      /* initial state, mhd_set_state layout (nkr, n, n, 6); copied at submit */
} mhd_request;
#define MHD_REQ_QUEUED 0
#define MHD_REQ_ACTIVE 1
#define MHD_REQ_DONE 2
#define MHD_REQ_FAILED 3
#define MHD_REQ_REJECTED 4
#define MHD_REQ_CANCELLED 5
int mhd_server_create(const mhd_server_params* params, mhd_server* out);
int mhd_server_destroy(mhd_server s);
int mhd_server_submit(mhd_server s, const mhd_request* req, long long* rid);
/* one scheduling round; *active and *queued count the requests in those states afterwards */
int mhd_server_tick(mhd_server s, int* active, int* queued);
int mhd_server_poll(mhd_server s, long long rid, int* status, long long* steps_done);
/* diag: 8 doubles as mhd_diagnostics (done or failed requests); sol: the final state (done
 * requests with keep_states; may be NULL); the message of a failed / rejected request goes to
 * mhd_last_error */
int mhd_server_result(mhd_server s, long long rid, double* diag, float* sol);
int mhd_server_cancel(mhd_server s, long long rid);
/* device bytes reserved by the server's size classes now, and the peak so far */
int mhd_server_memory(mhd_server s, double* reserved, double* peak);

/* Ensembles of size classes stepped together: one CUDA graph holds one step of every member,
 * each member on its own stream, so boxes of different sizes run concurrently. */
int mhd_ensemble_create(mhd_handle* handles, int count, mhd_ensemble* out);
int mhd_ensemble_step(mhd_ensemble e, int nsteps);
int mhd_ensemble_destroy(mhd_ensemble e);

/* Timing helper: elapsed device milliseconds of nsteps steps measured with events on the stream. */
int mhd_time_steps(mhd_handle h, int nsteps, double* ms);

/* Timing helper: nsteps steps back to back with an event between consecutive steps; fills
 * ms_per_step[0..nsteps) with each step's device milliseconds (synchronises at the end). */
int mhd_step_timed(mhd_handle h, int nsteps, double* ms_per_step);

/* A99 random solenoidal forcing of the velocity, the calcF! hook of MHDcalcN!'s addforcing!
 * (src/pgen.jl:159,231-234) with GetA99vars_And_function / SetUpFk! / A99ForceDriving!
 * (src/pgen/A99ForceDriving_GPU.jl:18-130).  P > 0 turns it on (P = 0 off); kf, sigma, b are
 * SetUpFk!'s arguments.  As in the reference, A is computed from the spectrum peaked at kf, the
 * forcing kernel then uses kf = b (SetUpFk! stores b there), every right-hand-side evaluation
 * draws new random numbers, and the whole velocity right-hand side keeps only its real part on
 * the kx = 0 plane.  The device rand() of the reference is replaced by a counter-based
 * generator of (seed, 8 * step + stage, mode index, draw), so runs are reproducible; the step
 * counter is the slot's clock step (mhd_set_clock sets it).  mhd_get_forcing returns A and the
 * kf the kernel uses. */
int mhd_set_forcing(mhd_handle h, double P, double kf, double sigma, double b, unsigned long long seed);
int mhd_slot_set_forcing(mhd_handle h, int slot, double P, double kf, double sigma, double b,
                         unsigned long long seed);
int mhd_get_forcing(mhd_handle h, int slot, double* A, double* kf_used);

/* Volume penalisation, Problem(...; VP_method = true) (src/pgen.jl:29,111-124): with
 * mhd_params.vp = 1 every right-hand side gains VP_UᵢUpdate! and, for MHD, VP_BᵢUpdate!
 * (src/Solver/VPSolver.jl:20-58, called from src/Solver/MHDSolver.jl:85-88,160-163 and
 * src/Solver/HDSolver.jl:76-79): N_a += -(δ_aj - k_a k_j / k^2) rfft(chi / eta (u_j - U0_j)) and
 * the same with B and B0, eta = 13 dt / 7.  The handle holds per slot the mask chi and the wall
 * fields, all zero at creation.  mhd_set_vp / mhd_slot_set_vp copy them in, in place of writing
 * params.χ, params.U₀x..U₀z, params.B₀x..B₀z: chi is n^3 floats, U0 and B0 are 3 n^3 floats
 * (x, y, z components one after another), all in the reference's (nx, ny, nz) column-major
 * order; NULL sets zero (chi = NULL turns the penalty off for the slot; B0 is unused by HD).
 * mhd_div_correct runs DivVCorrection! (fields & MHD_DIV_U) and DivBCorrection! (fields &
 * MHD_DIV_B) (src/Solver/VPSolver.jl:60-138) on the state: u and B lose their gradient part.
 * mhd_set_div_correction(h, 1) makes every step of every active slot end with both, as
 * TimeIntegrator! does with VP (src/integrator.jl:84-88,118-122); with the on-device CFL the next
 * dt then comes from the corrected fields, as getCFL! reads the corrected vars there.
 * VP needs precision MHD_PREC_FP32. */
/* On-device diagnostics history: the getCFL! / increment!(diags) loop of TimeIntegrator!
 * (src/integrator.jl:108-116, src/DiagnosticWrapper.jl:77-105) without host synchronisation.
 * With freq > 0, every freq-th step of mhd_step (counted from this call) ends with the spectral
 * diagnostics of every active slot, written on the device into the next of `capacity` samples
 * (later samples are dropped); freq = 0 turns it off.  mhd_get_diag_history
 * synchronises and copies up to max_samples samples of `slot`, 8 doubles each: handle step
 * count, t, E_u, E_B, H_c, max|k.u|, max|k.B|, non-finite count (the quantities of
 * mhd_diagnostics but max|div B|); *count is the number of samples stored so far (at most
 * `capacity`). */
int mhd_set_diag_history(mhd_handle h, int freq, int capacity);
int mhd_get_diag_history(mhd_handle h, int slot, double* out, int max_samples, int* count);

/* Failure detection: the device waits of the library (the TMA-fed passes' tile waits) are
 * bounded; a wait that runs out records an error word, the kernel drains its own copies and
 * returns, and mhd_synchronize reports MHD_ERR_CUDA.  mhd_check_bounded_wait exercises that path
 * on `device` without a fault: one thread waits limit_ms (0 < limit_ms <= 1000) on an mbarrier
 * nothing arrives on; *timed_out = 1 and *waited_ms the time it waited.  The context stays usable. */
int mhd_check_bounded_wait(int device, double limit_ms, int* timed_out, double* waited_ms);

/* Memory-safety check: the large device buffers of a handle (states, pass buffers, staging, VP
 * mask and walls) end in 4 KB guard bands filled with a fixed byte; *bad_bytes is the number of
 * guard bytes some kernel overwrote (0 when every write stayed in bounds). */
int mhd_check_guards(mhd_handle h, long long* bad_bytes);

#define MHD_DIV_U 1
#define MHD_DIV_B 2
int mhd_set_vp(mhd_handle h, const float* chi, const float* U0, const float* B0);
int mhd_slot_set_vp(mhd_handle h, int slot, const float* chi, const float* U0, const float* B0);
int mhd_div_correct(mhd_handle h, int fields);
int mhd_slot_div_correct(mhd_handle h, int slot, int fields);
int mhd_set_div_correction(mhd_handle h, int on);

/* Autotuner (no counterpart in the reference, whose FFTs are FFTW / cuFFT plans made with
 * MEASURE).  Each FFT pass class (z_inverse, y_inverse, x_fused, y_forward, z_forward: classes
 * 0..4 of mhd_kernel_class_name) has a default kernel configuration and, for some grid sizes,
 * further candidates (radix plans, kx columns per tile, transforms per exchange round, occupancy
 * bounds).  mhd_autotune times every candidate that fits on the device on the handle's own
 * scratch buffers (the state is not touched; at least one slot must be active) and selects the
 * fastest of each class.  The result is kept for the process and appended to a tuning file
 * ($MHDGB_TUNE_CACHE, else $XDG_CACHE_HOME/mhdgb/tune.txt, else $HOME/.cache/mhdgb/tune.txt;
 * MHDGB_TUNE_CACHE="" disables the file), keyed by device name, SM count and n; handles created
 * later for the same key start from it.  Without MHD_TUNE_FORCE a known result is applied
 * without timing.  Every variant computes the same transforms; results agree to FP32 rounding. */
#define MHD_TUNE_FORCE 1     /* time the candidates even if a result is known */
#define MHD_TUNE_NO_FILE 2   /* do not append to the tuning file */
int mhd_autotune(mhd_handle h, int flags);
int mhd_variant_count(mhd_handle h, int cls, int* count);
/* name of variant idx of class cls (idx < 0: the selected one) into buf[0..len) */
int mhd_variant_name(mhd_handle h, int cls, int idx, char* buf, int len);
int mhd_select_variant(mhd_handle h, int cls, int idx);

/* Allocation-free spectral diagnostics (no counterpart in the reference).  For callers that
 * cannot allocate device memory: a Julia program whose CuArrays come from CUDA.jl's pool or a
 * Python program whose tensors come from PyTorch's caching allocator, where all device memory
 * is meant to go through that pool; real-time loops that must not block on the allocator.
 * Reads sol_dev, a device copy of prob.sol (complex64, column-major (n/2+1, n, n, 6), the
 * mhd_set_state layout), and writes to out_dev[0..6) on the device: E_u, E_B, H_c (sums over the
 * retained band times dV, like mhd_diagnostics), max|k.u_hat|, max|k.B_hat|, non-finite count.
 * Launches on `stream` (a cudaStream_t, NULL = default stream) and does not synchronise.  It
 * calls no allocator; its only scratch is a static 58,368-byte device array inside the library
 * (partial sums of at most 1216 blocks; larger grids are covered by a grid-stride loop), which
 * every GPU that loads the library holds until the process exits.  n must be a supported size
 * (16, 32, 48, 64, 96, 128, 256, 512); others are rejected with MHD_ERR_INVALID.  The first call
 * in each CUDA context (for runtime users: on each device) looks up that array's address with
 * cudaGetSymbolAddress, so make it before any stream capture.  All calls share the array: calls
 * that overlap on the GPU (two streams, two host threads) race on it. */
int mhd_diagnostics_noalloc(const float* sol_dev, int n, double L, double* out_dev, void* stream);

/* Last error message of the calling thread ("" if none). */
const char* mhd_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* MHDGB_H */
