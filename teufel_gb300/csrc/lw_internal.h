// lw_internal.h -- structures shared by the host side of the C-ABI and the
// kernels of the Lienard-Wiechert field integration.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace teufel {

// Physical constants, src/global.h:36-44 of the reference.
constexpr double kC = 2.99792458e8;
constexpr double kE = 1.6021766208e-19;
constexpr double kPi = 3.1415926535897932384626433832795029;
constexpr double kEps0 = 8.854187817e-12;

// Trajectory points are grouped into segments of kSegLen steps.  Segment k of
// a particle owns steps [k*kSegLen, (k+1)*kSegLen) and its first point is the
// FP64 anchor from which the FP32 path measures positions and arrival times.
// Segments are also the unit in which particle ranges are split over slots.
constexpr int kSegShift = 7;
constexpr int kSegLen = 1 << kSegShift;
// The warp kernel stages trajectory data into shared memory in chunks of
// kChunkLen points; a chain may start at any chunk boundary.
constexpr int kChunkShift = 5;
constexpr int kChunkLen = 1 << kChunkShift;

// float4 per pair-point of the pair kernel's interleaved data (lw_fp32_pair.cu)
constexpr int kPairPoint = 10;

// The frame the FP32 per-point vectors of a set are expressed in: v' = R v
// (row-major r).  Its z axis is the set's mean direction of motion, so that
// the transverse components of all directions that matter stay small and
// FP32 keeps their angles to ~1e-7 relative; identity = 1 when the set moves
// along a coordinate axis already (then nothing is rotated).
struct Frame {
    double r[9];
    int identity;
};

// Device view of a resident trajectory set.
struct DevTraj {
    int n_particles;
    int64_t n_points;           // total points
    int64_t n_segments;         // total segments
    const int64_t* offsets;     // [n+1] first point of each particle
    const int64_t* seg_offsets; // [n+1] first segment of each particle
    const double* charge;       // [n] Coulomb
    const double4_32a* vhat;        // [n] frame direction of each particle (mean velocity);
                                    // w = smallest arrival advance of a step, min(dt - |dx|/c),
                                    // 0 when some step is not forward in time and slower than c
    const double4_32a* tx;          // [Npts] t, x, y, z                 (FP64, as uploaded)
    const double4_32a* pp;          // [Npts] beta*gamma, w unused        (FP64)
    const double4_32a* aa;          // [Npts] d(beta*gamma)/dt, w unused  (FP64)
    const float4* q0;           // [Npts] e = x - x_anchor (xyz), duration of the step from here
    const float4* q1;           // [Npts] beta-hat (xyz), eps = 1 - |beta|
    const float4* q2;           // [Npts] A/gamma*scale/c (xyz), scale/gamma^2
    const float4* q3;           // [Npts] chord direction of the step from here (xyz),
                                //        1 - |chord velocity|/c
    // Particles pair_members[2j] and pair_members[2j+1] form pair j (-1: the
    // pair has one particle, the last pair of an odd set).  Pairs are formed
    // in the order of the particles' arrival (c t - n.x of the first point,
    // n the mean direction of the first points' momenta), so that the two
    // particles of a pair see a trace window at nearly the same trajectory
    // steps.  A pair is as long as its longer particle; its per-point
    // data interleaves the two particles' q0..q2 and the chord offsets
    // component by component, kPairPoint float4 per pair-point, e.g.:
    //   (e.x a, e.x b, e.y a, e.y b) (e.z a, e.z b, dt a, dt b)
    //   (bx a, bx b, by a, by b)     (bz a, bz b, eps a, eps b)
    //   (cx a, cx b, cy a, cy b)     (cz a, cz b, cw a, cw b)
    //   (chx a, chx b, chy a, chy b) (chz a, chz b, ceps a, ceps b)
    // where b = beta-hat, c = q2, ch = chord direction; beyond the end of the
    // shorter particle its last point is repeated.
    Frame frame;
    // 1 when some particle's arrival times can fall along its points (a step
    // backwards in time or not slower than light): the set then runs on the
    // FP64 kernel, whose decisions are the reference's for any step
    int non_monotone;
    int n_pairs;
    int64_t n_pair_segments;
    const int* pair_members;          // [n_pairs][2]
    const int64_t* pair_offsets;      // [n_pairs+1] first pair-point of each pair
    const int64_t* pair_seg_offsets;  // [n_pairs+1] first pair-segment of each pair
    const float4* pq;                 // [pair-points][kPairPoint]
};

// One observer handed to a kernel launch.
struct DevScreen {
    const double* pix_pos;  // [Np][3]
    const double* pix_t0;   // [Np]
    int np;
    int nt;
    double dt;
};

// Work split: slot s integrates global segments [slot_seg[s], slot_seg[s+1])
// (particle segments, or pair segments for the pair kernel).
struct DevWork {
    int n_slots;
    const int64_t* slot_seg;  // [n_slots+1]
    void* scratch;            // per-slot partial traces
    int64_t slot_stride;      // elements between slots
    unsigned int* status;     // bit mask of TEUFEL_ERR_* seen on the device
    Frame frame;              // the set's frame: the FP32 reduction turns fields back
    unsigned long long* counters;  // [0] in-window triples, [1] exact-fallback points,
                                   // [2] bin contributions (deposits), [3] point
                                   // evaluations (in window or walked for a neighbour)
    // Decision record (the recording instantiations of the pair kernels only;
    // nullptr otherwise): rec[(pixel * n_particles + m) * rec_stride + i] of
    // point i of particle m receives the decision the kernel took for it,
    // encoded by rec_encode.
    int* rec;
    int64_t rec_stride;
    // 1: the reduction stores the traces into out (out treated as zero)
    // instead of adding them
    int overwrite;
    // 1: the reduction clears the partial traces it has read, for a next use
    // of the memory without a memset (the batch's graph replays); 0: the
    // caller clears them before their next use
    int clear;
};

// A point decision as recorded: bin index + 4 in bits 0-26, the window and
// exact flags (kLeTmin | kLtTmax | kExact) in bits 27-29; bit 30 marks two
// different decisions recorded for one point.  0 means "not recorded".
constexpr int kRecFlagShift = 27;
constexpr int kRecConflict = 1 << 30;
__host__ __device__ constexpr int rec_encode(int idx, int flags) {
    return (idx + 4) | (flags << kRecFlagShift);
}

}  // namespace teufel

// Kernel launchers (defined in the .cu files)
namespace teufel {
// FP32 kernel variants: the 32 pixels of a warp walk the same steps (warp,
// registers sized for 2 or 3 resident blocks per SM), or every pixel walks
// its own in-window steps (lanes).
constexpr int kVariantUniform = 0;
constexpr int kVariantLanes = 1;
constexpr int kVariantWarp3 = 2;
// two particles per thread, packed FP32 pairs, one-warp blocks, with a
// register budget of 128 / 160 / 136 / 144 per thread (16 / 12 / 15 / 14
// resident warps per SM)
constexpr int kVariantPair = 3;
constexpr int kVariantPair160 = 4;
constexpr int kVariantPair136 = 5;
constexpr int kVariantPair144 = 6;
// 16 resident warps per SM, with the packed deposit of steps spanning several bins
constexpr int kVariantPairMulti = 7;
// 16 resident warps per SM, FP32 fields with the reference's FP64 arrival
// times and bin edges (where FP64's own rounding of the arrival times is not
// negligible against the bin width)
constexpr int kVariantPairTime = 8;
// as kVariantPair, with chunks of 8 / 32 pair-points instead of 16
constexpr int kVariantPairC8 = 9;
constexpr int kVariantPairC32 = 10;
constexpr bool is_pair_variant(int v) { return v >= kVariantPair && v <= kVariantPairC32; }
cudaError_t launch_fp32(const DevTraj& tr, const DevScreen& sc, const DevWork& w, int variant,
                        cudaStream_t s);
cudaError_t launch_fp32_warp(const DevTraj& tr, const DevScreen& sc, const DevWork& w,
                             int variant, cudaStream_t s);
cudaError_t launch_fp64(const DevTraj& tr, const DevScreen& sc, const DevWork& w, int threads,
                        cudaStream_t s);
// out += sum of the slots' partial traces over bins [e0, e1) (e1 < 0: all)
cudaError_t launch_reduce_fp32(const DevWork& w, const DevScreen& sc, double* out,
                               cudaStream_t s, int64_t e0 = 0, int64_t e1 = -1);
cudaError_t launch_reduce_fp64(const DevWork& w, const DevScreen& sc, double* out,
                               cudaStream_t s, int64_t e0 = 0, int64_t e1 = -1);
cudaError_t launch_point_decisions(const DevTraj& tr, int m, double3 pos, double t0, double dt,
                                   int nt, int64_t n_points, int64_t* idx, int* flags,
                                   double* u_est, float* band, cudaStream_t s);
cudaError_t launch_deposit_injected(int n_part, const int64_t* offs, const double* ts,
                                    const double* f, double t0, double dt, int nt, int precision,
                                    double* trace, unsigned int* status, cudaStream_t s);
cudaError_t launch_prep_particles(const DevTraj& tr, cudaStream_t s);
cudaError_t launch_prep_points(const DevTraj& tr, cudaStream_t s);
cudaError_t launch_prep_pairs(const DevTraj& tr, cudaStream_t s);
cudaError_t launch_fp32_pair(const DevTraj& tr, const DevScreen& sc, const DevWork& w,
                             int variant, cudaStream_t s);
cudaError_t launch_deposit_injected32(int n_part, const int64_t* offs, const double* ts,
                                      const double* f, double t0, double dt, int nt,
                                      double* trace, float* trace32, unsigned int* status,
                                      cudaStream_t s);
int probe_peaks(double* fp32_tflops, double* fp32x2_tflops, double* fp64_tflops);
int fixed_division_check(int n, const double* a, double b, const double* ts, double t0,
                         double dt, int nt, double* q, int* k);

// The lattice the device pusher tracks through (lw_track.cu): a planar
// undulator centred at `origin` and a homogeneous field; kz = 2 pi / lambda_u.
struct TrackLattice {
    int has_undulator;
    double b_peak, lambda_u, kz;
    int n_periods;
    double origin[3];
    int has_homogeneous;
    double e[3], b[3];
};
cudaError_t launch_vay_track(int n, const double* init, const double* charge_e,
                             const double* mass, const TrackLattice& L, double tstep, int n_steps,
                             double4_32a* tx, double4_32a* pp, double4_32a* aa,
                             unsigned int* status, cudaStream_t s);

// RetardedField(t, X) summed over a particle set (lw_snapshot.cu): the
// particle chunks to split a set into for np points, and the launch.
int retarded_field_chunks(int np, int n_particles);
cudaError_t launch_retarded_field(const DevTraj& tr, double obs_time, int np, const double* pos,
                                  int n_chunks, double* partial, double* out, cudaStream_t s);

// One work item of a batched launch: a pixel tile of an observer against one
// slot (particle range) of its trajectory set.
struct BatchItem {
    int obs;
    int tile;
    int slot;
};
// The persistent batched kernel (pair kernel body) and the batched reduction.
cudaError_t launch_fp32_pair_batch(const DevTraj* trs, const DevScreen* scs, const DevWork* wks,
                                   const BatchItem* items, int n_items, unsigned int* head,
                                   int n_blocks, cudaStream_t s, bool record = false);
int pair_batch_blocks_per_sm();
// resident one-warp blocks per SM of the pair kernel of a variant (0: unknown)
int pair_blocks_per_sm(int variant);
constexpr int kPairTile = 32;  // pixels per tile of the pair kernel
cudaError_t launch_reduce_fp32_batch(const DevWork* wks, const DevScreen* scs,
                                     double* const* outs, const int64_t* bin_prefix, int n_obs,
                                     int64_t n_bins, cudaStream_t s);
}  // namespace teufel

struct teufel_traj_set;
namespace teufel {
// device view and status word of a trajectory handle (teufel_abi.cu)
const DevTraj* traj_device_view(const teufel_traj_set* traj, unsigned int** status);
// the longest particle's point count of a handle (the decision record's stride)
int64_t traj_max_points(const teufel_traj_set* traj);
}  // namespace teufel
