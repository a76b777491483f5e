/*
 * teufel_cuda.h -- C-ABI of the GB300 (sm_103a) Lienard-Wiechert field
 * integration for TEUFEL observers.
 *
 * This is the drop-in boundary for TEUFEL's field-integration step.  In the
 * reference the step is reached through the observer API:
 *
 *   BaseObserver::integrate()                     src/observer.h:55
 *     ScreenObserver<Beam>::integrate()           src/screen.cpp:113-146
 *     MeshedScreen<Beam>::integrate()             src/mesh.cpp:289-316
 *     PointObserver<Beam>::integrate()            src/point_observer.cpp:62-66
 *   -> Beam::integrateFieldTrace                  src/beam.cpp:443-451
 *   -> Bunch::integrateFieldTrace                 src/bunch.cpp:739-745
 *   -> ChargedParticle::integrateFieldTrace       src/particle.cpp:771-867
 *
 * and the traces leave through getBuffer() as [pixel][sample][Ex,Ey,Ez,Bx,By,Bz]
 * doubles (src/screen.cpp:249-272, src/mesh.cpp:376-399,
 * src/point_observer.cpp:78-89).  The functions below replace the body of
 * those integrate() specialisations: the caller passes the observation points
 * and per-point trace start times it already holds, and receives the traces
 * in that same buffer layout, accumulated (+=) into what the buffer holds, as
 * FieldTrace::add accumulates into traces that zero() cleared.
 *
 * Conventions
 *  - Plain C types only; every function returns a status code (TEUFEL_OK = 0)
 *    and never throws.  teufel_cuda_status_string() gives a message.
 *  - Trajectories are uploaded once (teufel_cuda_traj_upload) and stay
 *    resident on the device across observers until teufel_cuda_traj_free.
 *  - Calls are asynchronous on the given stream internally and synchronous at
 *    return for host buffers; the *_ex entry with device pointers returns once
 *    the work is enqueued.
 *  - A handle is not re-entrant: one call at a time per teufel_traj_set.
 */
#ifndef TEUFEL_CUDA_H
#define TEUFEL_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define TEUFEL_OK 0
#define TEUFEL_ERR_ARG 1      /* bad argument: null pointer, negative size, non-finite value */
#define TEUFEL_ERR_NOMEM 2    /* device or pinned-host allocation failed */
#define TEUFEL_ERR_CUDA 3     /* a CUDA runtime call failed */
#define TEUFEL_ERR_RANGE 4    /* a deposit fell outside its trace: the condition on which
                                 FieldTrace::add throws IOexception (src/fieldtrace.cpp:185-190);
                                 the offending deposit is skipped, all others are kept */
#define TEUFEL_ERR_TIMEOUT 5  /* a device-side wait ran out: the pair kernels wait for their
                                 bulk copies of trajectory chunks for at most about a second
                                 each, then stop waiting and report this (the traces are then
                                 not to be used) */
#define TEUFEL_ERR_NODEVICE 6 /* no CUDA device, or not an sm_103 device */

/* ---- arithmetic of the integration -------------------------------------- */
#define TEUFEL_PREC_FP32_SPLIT 0 /* FP32 fields with split-form 1-n.beta; FP64 anchors,
                                    bin indices bit-identical to the reference */
#define TEUFEL_PREC_FP64 1       /* plain FP64 throughout, in the reference's operation order */
#define TEUFEL_PREC_FP32_FP64TIME 2 /* FP32 split-form fields with the reference's FP64 arrival
                                       times, bin indices and bin edges: the deposit follows
                                       FP64's own rounding of the arrival times.  Chosen
                                       automatically for TEUFEL_PREC_FP32_SPLIT calls (kernel
                                       variant 0) whose bins are short against that rounding:
                                       2^-52 max|t0| / |dt| > 1e-6 */

typedef struct teufel_traj_set teufel_traj_set; /* opaque, device-resident */
typedef void *teufel_stream_t;                   /* a cudaStream_t; NULL = default stream */

typedef struct teufel_options {
    int precision;        /* TEUFEL_PREC_*                                        */
    int device_pointers;  /* 1: pix_pos, pix_t0 and out are device pointers      */
    int n_slots;          /* particle-range slots reduced in FP64; 0 = automatic  */
    int kernel_variant;   /* FP32 path: 0 = automatic (4), 1 = warp-uniform
                             steps, 2 = per-pixel steps, 3 = warp-uniform steps
                             with registers for 3 blocks of 256 per SM,
                             4/5/6/7 = warp-uniform steps, two particles per
                             thread, 16/12/15/14 resident warps per SM,
                             8 = as 4, with packed deposits of steps that
                             span several bins (short bins), 9 = as 4, with
                             the FP64 arrival times of TEUFEL_PREC_FP32_FP64TIME,
                             10/11 = as 4, staging trajectory chunks of 8/32
                             instead of 16 points                            */
    int timing;           /* 1: time the kernels with CUDA events on the stream,
                             read back by teufel_cuda_last_timing               */
    int max_device_mib;   /* upper bound on the device memory one call may take
                             for its work buffers (staged pixels and traces of a
                             host-buffer call, partial traces) [MiB]; 0 = none:
                             partial traces then take up to 40% of the free
                             memory.  Slots beyond the bound run as successive
                             passes; a call that cannot run one slot within it
                             returns TEUFEL_ERR_NOMEM before touching out.    */
    int overwrite_out;    /* 1: out receives the traces instead of having them
                             added (out is neither read nor uploaded; the
                             result equals adding them to zeroed traces, bit
                             for bit).  For callers whose traces were just
                             cleared (MeshedScreen::zero, src/mesh.cpp:282-286):
                             a host-buffer call then copies only the result
                             back.  0 = accumulate, as FieldTrace::add does.   */
} teufel_options;

/* Fill *opt with the defaults (FP32 split path, host pointers, automatic tiling). */
void teufel_cuda_default_options(teufel_options *opt);

/* Message for a status code. */
const char *teufel_cuda_status_string(int status);

/* Upload the trajectories of a particle set and keep them resident.
 * Replaces the per-pixel reads of ChargedParticle::Time/X/P/A
 * (src/particle.h:417-427) made by integrateFieldTrace.
 *   n_particles          number of particles (>= 0)
 *   n_points[n]          trajectory points per particle (NP, src/particle.h:378)
 *   charge_C[n]          particle charge [C]: ChargedParticle::getCharge() (src/particle.h:115),
 *                        i.e. Charge*ElementaryCharge as the reference forms it
 *   t[Npts]              trajectory times [s], Npts = sum(n_points), particles concatenated
 *   x[Npts][3]           positions [m]
 *   bg[Npts][3]          beta*gamma (TrajMomentum)
 *   a[Npts][3]           d(beta*gamma)/dt [1/s] (TrajAccel)
 * Non-finite inputs are rejected with TEUFEL_ERR_ARG. */
int teufel_cuda_traj_upload(int n_particles, const int *n_points, const double *charge_C,
                            const double *t, const double *x, const double *bg, const double *a,
                            teufel_traj_set **out);

/* The field a device-tracked particle set moves through: the reference's
 * Lattice of a PlanarUndulator (src/undulator.cpp:107-125, one-period linear
 * ramps at both ends) centred at origin, plus a HomogeneousField
 * (src/fields.cpp:150-163); either may be absent. */
typedef struct teufel_lattice {
    int has_undulator;
    double b_peak;     /* peak field [T] */
    double lambda_u;   /* period [m] */
    int n_periods;
    double origin[3];  /* undulator centre [m] */
    int has_homogeneous;
    double E[3];       /* [V/m] */
    double B[3];       /* [T] */
} teufel_lattice;

/* Track particles on the device and keep the trajectories resident, without
 * host trajectory arrays: the reference's ChargedParticle::InitVay and
 * n_steps calls of StepVay (src/particle.cpp:407-512) per particle, giving
 * n_steps+1 points, the first being the initial condition with the
 * acceleration InitVay computes.
 *   init[n][7]     t, x, y, z, beta*gamma x, y, z  (initTrajectory's arguments)
 *   charge_e[n]    charge in units of e (the reference's Charge)
 *   mass[n]        mass in electron masses (the reference's Mass)
 *   tstep > 0, n_steps >= 0
 * The result is a set like one from teufel_cuda_traj_upload, with charge
 * Charge*ElementaryCharge.  FP64 in the reference's operation order: the
 * trajectories agree with the reference's to within the last-ulp differences of
 * sin/cos/sinh/cosh.  A non-finite trajectory returns TEUFEL_ERR_ARG. */
int teufel_cuda_traj_track(int n_particles, const double *init, const double *charge_e,
                           const double *mass, const teufel_lattice *lattice, double tstep,
                           int n_steps, teufel_traj_set **out);

/* Copy a set's trajectories back to the host, in teufel_cuda_traj_upload's
 * layout: t[Npts], x[Npts][3], bg[Npts][3], a[Npts][3] (the reference's
 * ChargedParticle::TrajTime/TrajPoint/TrajMomentum/TrajAccel, src/particle.h).
 * Any pointer may be NULL. */
int teufel_cuda_traj_download(const teufel_traj_set *traj, double *t, double *x, double *bg,
                              double *a);

/* Release a trajectory set and its device memory.  NULL is accepted. */
int teufel_cuda_traj_free(teufel_traj_set *traj);

/* Total trajectory points held by the set (for sizing and diagnostics). */
int64_t teufel_cuda_traj_points(const teufel_traj_set *traj);

/* Integrate the fields of all particles onto Np observation points.
 * Replaces MeshedScreen<Beam>::integrate (src/mesh.cpp:289-316) and
 * ScreenObserver<Beam>::integrate (src/screen.cpp:113-146): pixel i observes
 * at pix_pos[i] with trace t0 = pix_t0[i], step dt, Nt samples; the result is
 * added into out[Np][Nt][6] (host memory).  Nt < 2 or an empty particle set
 * leaves out unchanged, as the reference does (src/particle.cpp:778-783).
 * Synchronous at return.  The work runs on s; out travels on a stream of the
 * set's own, ordered after the work already on s (up during the integration,
 * back in chunks behind the reduction), so pinned memory overlaps the copies
 * with the computation.  dt < 0 is accepted, as by the reference, and runs
 * the FP64 kernel whatever the precision: the window is then reversed
 * (tmin > tmax), and the reference either adds nothing or raises its range
 * error (TEUFEL_ERR_RANGE) for a step straddling that window.  So does a set
 * with a particle whose arrival times can fall along its points (a step
 * backwards in time, or a chord not slower than light). */
int teufel_cuda_integrate_screen(const teufel_traj_set *traj, const double *pix_pos,
                                 const double *pix_t0, double dt, int Nt, int Np, double *out,
                                 teufel_stream_t s);

/* One observation point: replaces PointObserver<Beam>::integrate
 * (src/point_observer.cpp:62-66).  out[Nt][6] (host memory) is added into. */
int teufel_cuda_integrate_point(const teufel_traj_set *traj, const double *pos, double t0,
                                double dt, int Nt, double *out, teufel_stream_t s);

/* As teufel_cuda_integrate_screen, with explicit options (precision, device
 * pointers for pix_pos/pix_t0/out, tiling).  With device pointers the call
 * returns once the work is enqueued on s. */
int teufel_cuda_integrate_screen_ex(const teufel_traj_set *traj, const double *pix_pos,
                                    const double *pix_t0, double dt, int Nt, int Np, double *out,
                                    const teufel_options *opt, teufel_stream_t s);

/* The summed field of all particles at time obs_time on Np points: replaces
 * SnapshotObserver<Beam>::integrate (src/snapshot.cpp:72-80), i.e.
 * Beam/Bunch::RetardedField(double, Vector) (src/beam.cpp:433-441,
 * src/bunch.cpp:729-737) at every point.  pos[Np][3] (host); out[Np][6]
 * (host, Ex,Ey,Ez,Bx,By,Bz) is overwritten, as the snapshot assigns.  FP64 with
 * the reference's algorithm (src/particle.cpp:612-769): a particle contributes
 * nothing where the signal of its last trajectory point has not arrived yet;
 * before its first point it is extrapolated backwards at constant velocity;
 * otherwise the emission point is found by bisection of the trajectory and
 * secant refinement inside the step.  A particle
 * without trajectory points returns TEUFEL_ERR_RANGE (the reference throws
 * RANGEexception).  Synchronous. */
int teufel_cuda_retarded_field(const teufel_traj_set *traj, double obs_time, int Np,
                               const double *pos, double *out, teufel_stream_t s);

/* No counterpart in the reference.  Tunes the FP32 split-precision path for
 * one observer shape: times the kernel variants (warp-uniform; two particles
 * per thread at 13 to 16 resident warps per SM, at 16 with packed
 * multi-bin deposits, and at 16 with trajectory chunks of 8 and of 32
 * points) at the automatic slot count -- or only the FP64-time
 * kernel (9) where TEUFEL_PREC_FP32_FP64TIME's rule selects it --
 * then the fastest at half and twice as many slots, on these very inputs,
 * writing the trial traces to a scratch buffer (out-free: nothing is added
 * anywhere).  A later candidate wins only when more than 0.5% faster than the
 * best so far, so near-ties keep the default kernel and slot count.  *best
 * receives *opt with kernel_variant and n_slots set to the winner, *best_ms
 * (may be NULL) its time.  The choice is also remembered for
 * the shape class -- the log2 sizes of Np, Nt, the particle count and the
 * points per particle -- so later calls with kernel_variant = 0 on a similar
 * shape use it.  opt->device_pointers says where pix_pos/pix_t0 live.
 * Synchronous; runs the integration about ten times. */
int teufel_cuda_autotune(const teufel_traj_set *traj, const double *pix_pos,
                         const double *pix_t0, double dt, int Nt, int Np,
                         const teufel_options *opt, teufel_options *best, double *best_ms);

/* ---- batched observers ---------------------------------------------------- */

/* One observer of a batch: its observation points and traces (the arguments
 * of teufel_cuda_integrate_screen) and the trajectory set it integrates.
 * Pointers are device pointers (a batch is planned once and then replayed). */
typedef struct teufel_observer {
    const teufel_traj_set *traj;
    const double *pix_pos; /* [Np][3] */
    const double *pix_t0;  /* [Np]    */
    double dt;             /* > 0 for an observer with Np > 0 and Nt >= 2; the set
                              must have increasing arrival times (every step
                              forward in time and slower than light) */
    int Nt;
    int Np;
    double *out;           /* [Np][Nt][6], added into */
} teufel_observer;

typedef struct teufel_batch teufel_batch;

/* No single counterpart in the reference, whose driver integrates observer
 * after observer (src/teufel_hybrid.cpp:692-709, each a call to
 * BaseObserver::integrate).  Plans the FP32 split-precision integration of
 * n_obs observers of uneven sizes -- mesh sizes, trace lengths, particle
 * counts and trajectory lengths -- as ONE persistent kernel launch that takes
 * (observer, pixel tile, particle range) work items from a device queue,
 * largest first, followed by one reduction launch.  The plan (queue, slots,
 * partial-trace memory) is built here; the launches are captured once into a
 * CUDA graph, which teufel_cuda_batch_run replays.  Observers may share a
 * trajectory set.  opt: precision must be TEUFEL_PREC_FP32_SPLIT;
 * device_pointers must be 1; n_slots (0 = automatic) caps the particle
 * ranges per observer.  A batch always uses the chained FP32 arrival times:
 * an observer whose bins are short against FP64's rounding of its arrival
 * times (where teufel_cuda_integrate_screen switches to
 * TEUFEL_PREC_FP32_FP64TIME) gets traces closer to the exact arrival times
 * than the FP64 reference's, which differ from them at that rounding.  The trajectory sets and device arrays must outlive
 * the batch. */
int teufel_cuda_batch_create(int n_obs, const teufel_observer *obs, const teufel_options *opt,
                             teufel_batch **out);

/* Run a planned batch on stream s: every observer's out is added into.
 * Returns once the work is enqueued; the status of the run is returned by
 * teufel_cuda_batch_status. */
int teufel_cuda_batch_run(teufel_batch *batch, teufel_stream_t s);

/* Synchronizes with the last run of the batch and returns its status
 * (TEUFEL_ERR_RANGE when any deposit of any observer fell outside its
 * trace).  Any pointer may be NULL. */
int teufel_cuda_batch_status(teufel_batch *batch, int64_t *work_items, int64_t *inwindow,
                             double *kernel_ms);

int teufel_cuda_batch_free(teufel_batch *batch);

/* ---- allocation-free integration ---------------------------------------- */

/* Size of the fixed device array the allocation-free entry point keeps its
 * partial traces in (64 MiB, held by every GPU that loads the library). */
#define TEUFEL_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)

/* No counterpart in the reference (TEUFEL allocates its traces on the host).
 * The FP32 split-precision integration of teufel_cuda_integrate_screen_ex for
 * callers that cannot let the library call cudaMalloc: applications whose
 * device memory belongs to another allocator, or that must not allocate once
 * running because cudaMalloc/cudaFree can synchronize the device.  It makes no
 * device allocation: the partial traces live in a fixed file-scope array of
 * TEUFEL_NOALLOC_SCRATCH_BYTES.
 *   d_pix_pos[Np][3], d_pix_t0[Np], d_out[Np][Nt][6]  device pointers; d_out is added into
 * Limit: Np*Nt*6*sizeof(float) must not exceed TEUFEL_NOALLOC_SCRATCH_BYTES,
 * otherwise TEUFEL_ERR_ARG is returned and nothing runs; dt must be > 0 and
 * every step of the set forward in time and slower than light.  Larger observers
 * run in several passes of as many slots as fit.  Synchronous at return.
 * The array is shared by all calls and keeps the last call's contents (each
 * call clears what it uses first); calls that overlap on the GPU race.  The
 * first call on a device looks the array's address up on that device.  Every
 * call waits for its stream s (after each pass and before it returns), so it
 * must not be called while s, or any stream it would wait on, is being
 * captured into a CUDA graph. */
int teufel_cuda_integrate_screen_noalloc(const teufel_traj_set *traj, const double *d_pix_pos,
                                         const double *d_pix_t0, double dt, int Nt, int Np,
                                         double *d_out, teufel_stream_t s);

/* ---- diagnostics used by the parity tests and the benchmark -------------- */

/* Per trajectory point of particle m, as observed from pos with a trace
 * (t0, dt, Nt), the decision the device path takes: the bin index
 * round((ts-t0)/dt) clamped to [-2, Nt+1], flags bit0 = (ts <= tmin),
 * bit1 = (ts < tmax), bit2 = resolved by the exact FP64 fallback; and u_est,
 * the FP32-path estimate of (ts-t0)/dt.  The same device functions as the
 * main FP32 kernel are used, so this is the FP32 path's decision; sets whose
 * arrival times can fall along the points, and dt < 0, run on the FP64
 * kernel instead, whose decisions are the reference's.  Arrays have
 * n_points[m] entries (host memory). */
int teufel_cuda_point_decisions(const teufel_traj_set *traj, int m, const double *pos, double t0,
                                double dt, int Nt, int64_t *idx, int *flags, double *u_est,
                                float *band);

/* The decisions the shipping FP32 kernels take, recorded by their recording
 * instantiations (the same source compiled with one more store per point).
 * Runs teufel_cuda_integrate_screen_ex with host buffers on kernel variant 4
 * (the default, also for 0), 8 or 9 (opt->kernel_variant; opt->n_slots is
 * honoured; opt may be NULL) and adds the traces into out[Np][Nt][6].
 * rec[Np][n_particles][max_points] (host, max_points = the longest particle's
 * point count) receives, for every point a kernel evaluated for a pixel as
 * part of a particle's steps, its decision: (bin index round((ts-t0)/dt)
 * clamped to [-2, Nt+1]) + 4 in bits 0-26, the flags of
 * teufel_cuda_point_decisions in bits 27-29, bit 30 set when one point got two
 * different decisions (the last point of a slot is evaluated again as the
 * first of the next); 0 where no decision was taken.  Needs dt > 0 and
 * increasing arrival times (the FP32 kernels' domain); synchronous. */
int teufel_cuda_record_decisions(const teufel_traj_set *traj, const double *pix_pos,
                                 const double *pix_t0, double dt, int Nt, int Np,
                                 const teufel_options *opt, int32_t *rec, double *out);

/* The same record for observer obs of a batch, taken by the recording
 * instantiation of the persistent batched kernel: one run of the whole batch
 * (every observer's out is added into, as by teufel_cuda_batch_run) in which
 * observer obs records its decisions into rec[Np][n_particles][max_points]
 * (host).  Synchronous. */
int teufel_cuda_batch_record_decisions(teufel_batch *batch, int obs, int32_t *rec);

/* Run the device deposit routine on injected arrival times and fields (the
 * reference's known-answer test, tests/teufel.integrate_field.cpp:51-78,
 * injects them by overriding RetardedTime/RetardedField).  n_points[n],
 * ts[Npts], f[Npts][6] (host).  precision selects the FP64 or FP32 deposit.
 * trace[Nt][6] (host) is added into. */
int teufel_cuda_deposit_injected(int n_particles, const int *n_points, const double *ts,
                                 const double *f, double t0, double dt, int Nt, int precision,
                                 double *trace);

/* In-window step count of the last integrate call on this handle: the
 * number of (pixel, particle, step) triples whose arrival interval overlapped
 * the trace window (the reference's condition at src/particle.cpp:793). */
int teufel_cuda_last_inwindow(const teufel_traj_set *traj, int64_t *inwindow,
                              int64_t *fallback_points);

/* Work and timing of the last integrate call on this handle: deposits =
 * bin contributions made (>= in-window steps; multi-bin steps add one per
 * extra bin), evaluations = trajectory-point evaluations made (in-window
 * points, plus the points a warp walks for its neighbouring pixels),
 * launches = kernels launched, and -- when it ran with options.timing -- the
 * summed CUDA-event durations of the integration kernels and of the
 * reduction kernels [ms].  Synchronizes the device.  Any pointer may be NULL. */
int teufel_cuda_last_timing(const teufel_traj_set *traj, int64_t *deposits,
                            int64_t *evaluations, int *launches, double *kernel_ms,
                            double *reduce_ms);

/* Peak FMA throughput of the current device (TFLOP/s, FMA = 2 flops), each
 * measured with independent FMA chains: scalar FP32 (FFMA), packed two-wide
 * FP32 (fma.rn.f32x2) and FP64 (DFMA).  Any pointer may be NULL. */
int teufel_cuda_probe_peaks(double *fp32_tflops, double *fp32x2_tflops, double *fp64_tflops);

/* Diagnostic for the tests: the FP64-time mode's quotients against the IEEE
 * division on the device.  For i < n: q[2i] = a[i]/b as that mode forms it
 * (a product with RN(1/b), one FMA correction, the IEEE division where the
 * correction cannot prove the rounded quotient), q[2i+1] = the IEEE a[i]/b;
 * k[2i] = the bin round((ts[i] - t0)/dt) clamped to [-2, nt+1] as that mode
 * forms it (a product with RN(1/dt)), k[2i+1] = the same with the IEEE
 * quotient (the reference's).  Host pointers; dt > 0. */
int teufel_cuda_check_fixed_division(int n, const double *a, double b, const double *ts,
                                     double t0, double dt, int nt, double *q, int32_t *k);

#ifdef __cplusplus
}
#endif

#endif /* TEUFEL_CUDA_H */
