/*
 * spss_gpu.h — C ABI of libspss_gpu.so, the GB300 (sm_103a) implementation of
 * the pairwise-interaction hot path of raven91/spssLangevinIntegration.
 *
 * Plain pointers and sizes only.  Host arrays use the reference's AoS layout:
 * double[n*s], s = 4 (x, y, phi, omega) for the first-order model and s = 6
 * (x, y, v_x, v_y, phi, omega) for the second-order model, in the unit box.
 * Every function returns SPSS_OK (0) or a negative SPSS_ERR_* code and never
 * aborts.  A context owns one CUDA stream and device buffers; it is not
 * thread-safe (like the reference classes, which keep function-local statics).
 *
 * Citations are to the reference source tree (file:line).
 */
#ifndef SPSS_GPU_H
#define SPSS_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPSS_OK 0
#define SPSS_ERR_INVALID_ARGUMENT (-1)
#define SPSS_ERR_CUDA (-2)
#define SPSS_ERR_OUT_OF_MEMORY (-3)
#define SPSS_ERR_NOT_SUPPORTED (-4)
#define SPSS_ERR_NONFINITE (-5)
#define SPSS_ERR_SIZE (-6)

/* Interaction routine (ParticleSystemFirstOrder.hpp:31-50, ParticleSystemSecondOrder.hpp:23-56). */
#define SPSS_VARIANT_DISPATCH 0          /* EvaluateRhs: the reference's choice by interaction radius */
#define SPSS_VARIANT_ALL_PAIRS 1         /* EvaluateInteractionsWithAllPairs */
#define SPSS_VARIANT_LINKED_LIST 2       /* EvaluateInteractionsWithLinkedList */
#define SPSS_VARIANT_VERLET 3            /* EvaluateInteractionsWithVerletNeighborList */
#define SPSS_VARIANT_LINKED_LIST_VERLET 4/* EvaluateInteractionsWithLinkedListAndVerletNeighborList */
#define SPSS_VARIANT_GLOBAL_FIELD 5      /* EvaluateInteractionsWithGlobalPolarOrderField (first order) */

/* Arithmetic of a context. */
#define SPSS_PRECISION_F64 0   /* the reference's FP64 arithmetic, operation for operation */
#define SPSS_PRECISION_F32 1   /* GB300 path: 64-bit fixed-point positions, FP32 pair and stage math */

/* Steppers (Steppers/RungeKutta4Stepper.hpp:15-42, StochasticEulerStepper.hpp:14-60,
 * StochasticEulerStepperPtr.hpp:19-115, StochasticRungeKuttaStepperPtr.hpp:21-85). */
#define SPSS_STEPPER_RK4 0
#define SPSS_STEPPER_STOCHASTIC_EULER 1
#define SPSS_STEPPER_STOCHASTIC_RUNGE_KUTTA 2

typedef struct spss_params
{
  int model;       /* 1 first order, 2 second order */
  int flavor;      /* first-order class: 0 ParticleSystemFirstOrder, 1 ParticleSystemFirstOrderPtr */
  int n;           /* number of particles */
  int variant;     /* SPSS_VARIANT_* used by the steppers */
  int precision;   /* SPSS_PRECISION_* */
  int nc_verlet;   /* cells per side of the Verlet build grid; 0 = int(1/rho) as the reference */
  double v0, xi, xi_r, D_r, xi_phi, D_phi, sigma, rho, alpha;
  double r_max;    /* Verlet radius; 0 = rho + 0.05 (ParticleSystemFirstOrderPtr.cpp:97-98) */
  unsigned long long seed;   /* Philox key of the noise stream */
  unsigned int replica;      /* replica index folded into the Philox counter */
} spss_params;

typedef struct spss_ctx spss_ctx;

/* Construction: the ParticleSystem* constructors (ParticleSystemFirstOrder.cpp:12-66,
 * ParticleSystemSecondOrder.cpp:12-70) together with the steppers' buffers. */
int spss_create(const spss_params *params, spss_ctx **out);
int spss_destroy(spss_ctx *ctx);
const char *spss_error_string(int code);
int spss_version(void);

/* The system state the steppers advance, resident in device memory.
 * Host AoS copies: SimulationEngine*::system_state_ handed to DoStep. */
int spss_set_state(spss_ctx *ctx, const double *state, long len);
int spss_get_state(spss_ctx *ctx, double *state, long len);

/* ParticleSystem*::EvaluateRhs / EvaluateInteractionsWith* on host arrays
 * (ParticleSystemFirstOrder.cpp:90-112, :162-649; ParticleSystemSecondOrder.cpp:85-113,
 * :116-409).  k_next is read and written: components the reference leaves
 * unwritten (isolated particles) keep the caller's values. */
int spss_evaluate_rhs(spss_ctx *ctx, int variant, const double *state, const double *k_prev, double *k_next,
                      double k_coef, double dt);
/* is_higher_order_sde_integration_ and GetComplimentaryAlignmentForce
 * (ParticleSystemFirstOrderPtr.hpp:72-73). */
int spss_set_higher_order(spss_ctx *ctx, int on);
int spss_get_complementary_force(spss_ctx *ctx, double *out, long len);
/* SetNaturalFrequencies (ParticleSystemFirstOrder.cpp:85-88). */
int spss_set_natural_frequencies(spss_ctx *ctx, const double *freqs, long len);

/* CalculateMaxDisplacement (ParticleSystemFirstOrder.cpp:670-696) and the
 * Verlet-list bookkeeping it drives. */
int spss_calculate_max_displacement(spss_ctx *ctx, const double *total_displacement, long len);
int spss_get_verlet_state(spss_ctx *ctx, double *accumulated_displacement, int *should_update_lists,
                          int *uses_verlet_list);
int spss_set_should_update_lists(spss_ctx *ctx, int flag);
/* Number of list builds the context has performed (Verlet lists, and on the
 * GB300 path also the per-step cell re-sorts of cell-list contexts): the
 * rebuilds the trigger above caused.  No reference counterpart (the
 * reference rebuilds silently). */
int spss_get_rebuild_count(spss_ctx *ctx, unsigned long long *count);

/* Lists of the most recent build, reference order (pre_linked_list_,
 * linked_list_, verlet_list_; ParticleSystemFirstOrder.hpp:59-66).
 * Offsets are CSR; *count receives the number of rows / entries. */
int spss_get_pre_linked_list(spss_ctx *ctx, int *out, long len);
int spss_get_cells(spss_ctx *ctx, int *offsets, long offsets_len, int *members, long members_len, int *ncell);
int spss_get_verlet_lists(spss_ctx *ctx, int *offsets, long offsets_len, int *entries, long entries_len,
                          long *total);

/* Stepper::DoStep on the resident state (RungeKutta4Stepper.cpp:29-101,
 * StochasticEulerStepper.hpp:33-51, StochasticEulerStepperPtr.hpp:40-73,
 * StochasticRungeKuttaStepperPtr.hpp:40-76).  Gaussian noise comes from a
 * counter-based Philox4x32-10 stream keyed by (seed, replica, step counter,
 * particle), which advances by one per stochastic step. */
int spss_step(spss_ctx *ctx, int stepper, double t, double dt);
/* nsteps consecutive DoStep calls, issued as one CUDA graph launch where possible. */
int spss_steps(spss_ctx *ctx, int stepper, double t0, double dt, int nsteps);
/* Drop-in DoStep(particle_system, system_state, t, dt) on a host AoS array:
 * reads it in, steps, writes it back.  Pageable arrays are registered as
 * mapped pinned memory on first use; page-locked mapped arrays
 * (spss_pinned_alloc, cudaHostAlloc) are used as they are.  Either way the
 * upload and download kernels read and write the array over the host link
 * directly (StochasticRungeKuttaStepperPtr::DoStep, StochasticRungeKuttaStepperPtr.hpp:40-76,
 * and the other steppers' DoStep). */
int spss_step_host(spss_ctx *ctx, int stepper, double *state, long len, double t, double dt);
int spss_get_step_counter(spss_ctx *ctx, unsigned long long *counter);
int spss_set_step_counter(spss_ctx *ctx, unsigned long long counter);
/* The Gaussian draws the stepper consumes at step counter `step`, in the
 * reference's draw order per particle (what a replayed oracle must see). */
int spss_noise(spss_ctx *ctx, int stepper, unsigned long long step, double *out, long len);

/* PeriodicBoundaryConditions::ApplyPeriodicBoundaryConditions(system_state)
 * (PeriodicBoundaryConditions.cpp:127-135) on the resident state. */
int spss_apply_pbc(spss_ctx *ctx);

/* Observer reductions (BinaryObserverFirstOrder.cpp:125-142,
 * BinaryObserverSecondOrder.cpp:121-138), accumulated in FP64:
 * out = {|<e^{i phi}>|, arg, |<v/|v|>|, arg}; first order repeats the phase pair. */
int spss_order_parameters(spss_ctx *ctx, double *out4);
/* One trajectory frame of the reference's binary observers, the s*n floats
 * that follow the float time stamp in their .bin files: SPSS_FRAME_WRAPPED as
 * BinaryObserverFirstOrder::SaveSystemState (BinaryObserverFirstOrder.cpp:101-123:
 * the state converted to float, positions wrapped into the unit box and the
 * phase into [0, 2 pi), with the reference's float/double rounding steps),
 * SPSS_FRAME_RAW as BinaryObserverSecondOrder::SaveSystemState
 * (BinaryObserverSecondOrder.cpp:101-116: the state converted to float).  The
 * frame is computed on the GPU and copied to `dst` (len = s*n floats) on the
 * context's stream; the call returns without synchronising, so `dst` must stay
 * valid until spss_synchronize (pinned memory from spss_pinned_alloc makes the
 * copy asynchronous; pageable memory works too, with a staged copy). */
#define SPSS_FRAME_RAW 0
#define SPSS_FRAME_WRAPPED 1
int spss_frame_async(spss_ctx *ctx, int mode, float *dst, long len);
/* Page-locked host memory for frames (cudaMallocHost / cudaFreeHost). */
int spss_pinned_alloc(size_t bytes, void **out);
int spss_pinned_free(void *p);
/* Adaptive integration with dense output, the reference's odeint path
 * (SimulationEngineFirstOrder.cpp:158-165: integrate_const with
 * make_dense_output(eps_abs, eps_rel, runge_kutta_dopri5) over the system's
 * operator(), ParticleSystemFirstOrder.cpp:114-120): Dormand-Prince 5(4) over
 * the FP64 right-hand side of the context's variant, the error norm and
 * step-size rule of odeint's documented defaults, the continuous extension of
 * Hairer, Norsett & Wanner for the observer times t0, t0 + dt_out, ... <= t1.
 * The observer (may be NULL) receives the host state at each of those times and
 * returns nonzero to stop.  The context's state ends at the last observer time
 * (or, when stopped, at the last accepted step).  *steps (may be NULL) receives
 * the number of accepted steps.  SPSS_PRECISION_F64 contexts. */
typedef int (*spss_observer_fn)(const double *state, long len, double t, void *user);
int spss_integrate_dopri5(spss_ctx *ctx, double t0, double t1, double dt_out, double eps_abs, double eps_rel,
                          spss_observer_fn observer, void *user, long *steps);
/* AveragingObserver::operator() and the averaged state (AveragingObserver.cpp:29-69). */
int spss_average_accumulate(spss_ctx *ctx);
int spss_average_get(spss_ctx *ctx, double *mean_state, long len, int *count);

int spss_synchronize(spss_ctx *ctx);
/* Number of kernels this context launched since creation. */
int spss_kernel_launches(spss_ctx *ctx, unsigned long long *count);

/* Issue all work of the context on the caller's CUDA stream (a cudaStream_t;
 * NULL returns to the context's own stream).  No reference counterpart: the
 * reference is CPU code. */
int spss_set_stream(spss_ctx *ctx, void *cuda_stream);
/* While timing is on, steps run one by one with CUDA events recorded on the
 * context's stream around the pair-and-update kernel; spss_get_timing returns
 * the summed kernel milliseconds and the number of timed launches.  No
 * reference counterpart. */
int spss_set_timing(spss_ctx *ctx, int on);
int spss_get_timing(spss_ctx *ctx, double *kernel_ms, unsigned long long *timed_launches);

/* Largest particle count spss_order_parameters_noalloc accepts. */
#define SPSS_NOALLOC_MAX_PARTICLES (1L << 30)

/* The order parameters of spss_order_parameters, computed without allocating
 * anything: for callers that must not call cudaMalloc, for instance a host
 * application whose own allocator owns the device memory (a raw cudaMalloc
 * there can fail, or fragment the pool the application manages) or a
 * real-time loop in which cudaMalloc's implicit device synchronisation would
 * stall.  No counterpart in the reference.
 *
 * `state` is a device array of the reference's AoS layout (n*4 or n*6
 * doubles for model 1 or 2), `out4` a device array of 4 doubles that receives
 * {|<e^{i phi}>|, arg, |<v/|v|>|, arg}; both belong to the caller.  The work
 * is queued on `cuda_stream` (NULL: the legacy default stream) and nothing is
 * synchronised.  The reduction's scratch is a fixed 32 KiB array inside the
 * library (1024 block partials), held on every GPU that loads the library
 * until the process exits and shared by all calls: calls that overlap on the
 * GPU race on it; each call rewrites every partial it reads, so nothing needs
 * clearing between calls.  The first call on a device looks up the array's
 * device address, so make that first call before any stream capture.  The
 * address is kept until the process exits: after cudaDeviceReset on a device
 * it is stale, so do not call this entry point on that device again.  Returns
 * SPSS_ERR_SIZE for n <= 0 or n > SPSS_NOALLOC_MAX_PARTICLES. */
int spss_order_parameters_noalloc(int model, const double *state, long n, double *out4, void *cuda_stream);

/* ------------------------------------------------------------------ batches
 *
 * A batch context steps `nsys` independent systems together — the GPU form of
 * the reference's MPI parameter scan, where each rank runs its own parameter
 * point (MPI_PARAMETER_SCAN in the SimulationEngine*Ptr engines): every kernel
 * of a step (binning, lists, pair sums + update, trigger) serves all systems
 * in one launch, and a step is one CUDA graph.  Systems may differ in every
 * physical parameter (n, v0, xi, xi_r, D_r, xi_phi, D_phi, sigma, rho, alpha,
 * r_max, nc_verlet, replica) but share model, flavor, variant, precision
 * (SPSS_PRECISION_F32) and seed; system r draws the noise a single context with
 * its parameters would draw.  State arrays (spss_set_state / spss_get_state /
 * spss_noise) are the systems' AoS arrays concatenated in order.  The Verlet
 * trigger is kept per system; when one system triggers, the lists of all are
 * rebuilt.  No reference counterpart beyond the scan itself. */
#define SPSS_MAX_SYSTEMS 65535
int spss_batch_create(const spss_params *systems, int nsys, spss_ctx **out);
/* Number of systems and (if `first` is not NULL) first[r] = index of system
 * r's first particle, first[nsys] = all particles (nsys + 1 entries).  A
 * single-system context reports one system. */
int spss_batch_size(spss_ctx *ctx, int *nsys, long *first);
/* Order parameters of every system, out[4 r + k] as spss_order_parameters
 * (FP64 sums of the FP32 cos/sin of each phase and of the velocity directions);
 * len = 4 nsys. */
int spss_batch_order_parameters(spss_ctx *ctx, double *out, long len);
/* nsteps steps (graph launches, no host synchronisation until the end).  After
 * every step whose step counter (spss_get_step_counter) is a multiple of
 * sample_every and at least sample_from, the order parameters of every system
 * are added to its running averages; sample_every = 0 takes no samples. */
int spss_batch_run(spss_ctx *ctx, int stepper, double t0, double dt, long nsteps, long sample_every,
                   long sample_from);
#define SPSS_STATS_PER_SYSTEM 5
/* Time averages of every system: out[5 r + 0..4] = mean and variance of the
 * phase order |<e^{i phi}>|, mean and variance of the velocity-direction order
 * |<v/|v|>| (first order: the phase order again), number of samples;
 * len = 5 nsys. */
int spss_batch_stats(spss_ctx *ctx, double *out, long len);
int spss_batch_reset_stats(spss_ctx *ctx);

/* Tiling of the pair-and-update kernel: cells per tile (each row of a
 * system's cell grid is split into ceil(nc / tile_cells) tiles of whole cells;
 * with Verlet lists the tiles of a row hold nearly equal numbers of particles,
 * with cell lists tile_cells cells each; 1 .. 4096) and launch form (0: one CTA per tile; 1: persistent,
 * one wave of CTAs taking tiles from a work counter).  Results do not depend
 * on the tiling; the lists are rebuilt before the next step.  F32 contexts. */
int spss_set_tiling(spss_ctx *ctx, int tile_cells, int persistent);
int spss_get_tiling(spss_ctx *ctx, int *tile_cells, int *persistent);
/* How steps run as CUDA graphs (spss_steps, spss_batch_run) rebuild Verlet
 * lists: 1 (default) the step's control kernel launches the rebuild as a
 * device graph when the trigger fires; 0 a conditional graph node holds the
 * rebuild at the start of each step (the form used where the device refuses
 * device-launched graphs; about 12 us more per step on GB300).  Results are
 * identical.  F32 contexts.  No counterpart in the reference. */
int spss_set_device_rebuild(spss_ctx *ctx, int enabled);
/* Times `steps` steps of every tiling candidate (16 to 64 cells per tile in steps of 4,
 * both launch forms) on the context's current state, keeps the fastest and
 * restores the state, step counter and trigger as they were (the lists are
 * rebuilt before the next step; before the first step that leaves every
 * result identical to an untuned run).  best_ms_per_step may be NULL. */
int spss_autotune(spss_ctx *ctx, int stepper, double dt, int steps, double *best_ms_per_step);

#ifdef __cplusplus
}
#endif

#endif
