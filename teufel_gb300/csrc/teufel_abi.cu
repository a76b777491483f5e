// teufel_abi.cu -- host side of the C-ABI declared in include/teufel_cuda.h.
//
// Owns the device-resident trajectory store, the per-slot partial traces and
// the staging of observer buffers; launches the field-integration kernels
// and the FP64 reduction.  Every entry point returns a status code and
// never throws across the ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <tuple>
#include <vector>

#include "lw_internal.h"
#include "teufel_cuda.h"

using namespace teufel;

struct teufel_traj_set {
    int device = 0;
    DevTraj dev{};
    std::vector<void*> owned;  // trajectory arrays
    // grow-only work buffers
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    int64_t* slot_seg = nullptr;
    int slot_cap = 0;
    double* d_pix = nullptr;
    size_t pix_cap = 0;  // doubles
    double* d_out = nullptr;
    size_t out_cap = 0;  // doubles
    unsigned int* d_status = nullptr;
    unsigned long long* d_counters = nullptr;
    unsigned long long last_counters[4] = {0, 0, 0, 0};
    // kernel timing of the last call (options.timing)
    std::vector<cudaEvent_t> ev;
    int n_ev_used = 0;
    int last_launches = 0;
    bool last_timed = false;
    std::vector<int64_t> h_seg_offsets;
    int64_t max_points = 0;  // the longest particle's point count
    int last_slots = 0;
    bool counted = false;  // included in the live-set count of its device
    // host-buffer calls: a copy stream that moves the trace buffer while the
    // integration runs, and its events ([0] caller's work issued, [1] traces
    // uploaded, [2] copies done, then one per reduced chunk)
    cudaStream_t copy_s = nullptr;
    std::vector<cudaEvent_t> cev;
};

namespace {

constexpr int kThreads = 128;
constexpr int64_t kMaxParticlesPerSlotFp32 = 2048;

#define TRY_CUDA(call)                              \
    do {                                            \
        cudaError_t e_ = (call);                    \
        if (e_ != cudaSuccess) return cuda_fail(e_); \
    } while (0)

int cuda_fail(cudaError_t e) {
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return TEUFEL_ERR_NOMEM;
    }
    cudaGetLastError();
    return TEUFEL_ERR_CUDA;
}

int check_device() {
    int dev = 0, n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return TEUFEL_ERR_NODEVICE;
    }
    if (cudaGetDevice(&dev) != cudaSuccess) return TEUFEL_ERR_NODEVICE;
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (major != 10 || minor != 3) return TEUFEL_ERR_NODEVICE;
    return TEUFEL_OK;
}

template <class T>
int dev_alloc(teufel_traj_set* h, T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * count);
    if (e != cudaSuccess) return cuda_fail(e);
    h->owned.push_back(*p);
    return TEUFEL_OK;
}

int grow(void** p, size_t* cap, size_t bytes, bool zero) {
    if (*cap >= bytes && *p) return TEUFEL_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e != cudaSuccess) return cuda_fail(e);
    if (zero) {
        e = cudaMemset(*p, 0, bytes ? bytes : 16);
        if (e != cudaSuccess) return cuda_fail(e);
    }
    *cap = bytes;
    return TEUFEL_OK;
}

__global__ void pack_points_kernel(int64_t n, const double* t, const double* x, const double* bg,
                                   const double* a, double4_32a* tx, double4_32a* pp, double4_32a* aa,
                                   unsigned int* status) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v[10] = {t[i],          x[3 * i],      x[3 * i + 1],  x[3 * i + 2], bg[3 * i],
                    bg[3 * i + 1], bg[3 * i + 2], a[3 * i],      a[3 * i + 1], a[3 * i + 2]};
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 10; k++) ok = ok && isfinite(v[k]);
    if (!ok) atomicOr(status, 1u << TEUFEL_ERR_ARG);
    tx[i] = make_double4_32a(v[0], v[1], v[2], v[3]);
    pp[i] = make_double4_32a(v[4], v[5], v[6], 0.0);
    aa[i] = make_double4_32a(v[7], v[8], v[9], 0.0);
}

int status_from_mask(unsigned int mask) {
    if (mask & (1u << TEUFEL_ERR_ARG)) return TEUFEL_ERR_ARG;
    if (mask & (1u << TEUFEL_ERR_RANGE)) return TEUFEL_ERR_RANGE;
    if (mask & (1u << TEUFEL_ERR_TIMEOUT)) return TEUFEL_ERR_TIMEOUT;
    if (mask) return TEUFEL_ERR_CUDA;
    return TEUFEL_OK;
}

bool finite_array(const double* p, int64_t n) {
    for (int64_t i = 0; i < n; i++)
        if (!std::isfinite(p[i])) return false;
    return true;
}

// Device part of an integration: partial traces per slot, then the FP64
// reduction into out (device pointers).  Enqueued on s.
// ---- partial-trace memory ----
// The FP32 partial traces of an integration come from a stream-ordered pool
// of the library's own, one per device, allocated on the call's stream and
// returned to the pool when the call's work is done.  Trajectory handles thus
// share this memory instead of each keeping its own; the pool keeps what it
// has (no release threshold) until the last handle of the device is freed.
std::mutex g_pool_mu;
std::map<int, cudaMemPool_t> g_pools;
std::map<int, int> g_live_sets;

cudaMemPool_t scratch_pool(int dev) {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    auto it = g_pools.find(dev);
    if (it != g_pools.end()) return it->second;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    g_pools[dev] = pool;
    return pool;
}

// Free device memory plus what the pool holds but does not use.
size_t available_bytes(cudaMemPool_t pool) {
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    uint64_t reserved = 0, used = 0;
    if (pool) {
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved);
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used);
    }
    return free_b + (size_t)(reserved > used ? reserved - used : 0);
}

// ---- tuned choices per shape class (teufel_cuda_autotune) ----
struct TuneKey {
    int np, nt, parts, pts;  // log2 buckets of pixels, samples, particles, points/particle
    bool operator<(const TuneKey& o) const {
        return std::tie(np, nt, parts, pts) < std::tie(o.np, o.nt, o.parts, o.pts);
    }
};
struct TuneChoice {
    int variant;      // kernel_variant
    int slot_pct;     // slot count relative to the automatic one [%]
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneChoice> g_tuned;

int log2_bucket(int64_t v) {
    int b = 0;
    while (v > 1) {
        v >>= 1;
        b++;
    }
    return b;
}
TuneKey tune_key(const teufel_traj_set* h, int np, int nt) {
    const int64_t n = std::max<int64_t>(h->dev.n_particles, 1);
    return TuneKey{log2_bucket(np), log2_bucket(nt), log2_bucket(n),
                   log2_bucket(h->dev.n_points / n)};
}

// A host trace buffer behind d_out: the reduction waits for its upload
// (uploaded, on the copy stream) and the last pass reduces in n_chunks row
// chunks, each copied back on the copy stream as soon as it is final.
struct HostOut {
    double* host;
    cudaStream_t cs;
    cudaEvent_t uploaded;
    const cudaEvent_t* chunk_ev;
    int n_chunks;
};

// Bounds of the slots in work units (segments).  Blocks are dispatched slot by
// slot, so with equal slots the last of several waves drains unevenly;
// geometric sizes (first slot largest, last ~6% of it) put the shortest blocks
// at the end.  Equal slots where the geometric first slot would hold more
// than max_units units (particles or pairs), the FP32 accumulation limit.
std::vector<int64_t> slot_bounds(int64_t G, int64_t slots, int64_t units, int64_t max_units,
                                 bool geometric) {
    std::vector<int64_t> b(slots + 1);
    for (int64_t k = 0; k <= slots; k++) b[k] = G * k / slots;
    if (!geometric || slots < 2 || G < 4 * slots) return b;
    const double r = std::pow(0.06, 1.0 / (double)(slots - 1));
    const double total = (1.0 - std::pow(r, (double)slots)) / (1.0 - r);
    std::vector<int64_t> g(slots + 1);
    g[0] = 0;
    double acc = 0.0;
    for (int64_t k = 1; k <= slots; k++) {
        acc += std::pow(r, (double)(k - 1));
        g[k] = std::min<int64_t>(G, (int64_t)std::llround(G * acc / total));
        g[k] = std::max<int64_t>(g[k], g[k - 1] + 1);
    }
    g[slots] = G;
    if (g[slots - 1] >= G) return b;
    // the first slot's units, at the set's average segments per unit
    const double per_unit = (double)G / (double)std::max<int64_t>(units, 1);
    if ((double)g[1] / per_unit + 1.0 > (double)max_units) return b;
    return g;
}

// The slot count near `slots` that best fills the last wave of the pair
// kernel's grid (pixel tiles x slots one-warp blocks, equal work each): the
// estimated time ceil(blocks / resident) / slots is minimised over
// [3/4, 3/2] x slots, taking the smallest count within 2% of the best, since
// every slot adds a partial trace to reduce.
// one-warp blocks of the pair kernel of `variant` resident on the device
// (0: unknown)
int64_t resident_pair_blocks(const teufel_traj_set* h, int variant) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return (int64_t)pair_blocks_per_sm(variant) * sms;
}

int64_t fill_waves(const teufel_traj_set* h, int np, int variant, int64_t slots) {
    const int64_t resident = resident_pair_blocks(h, variant);
    const int64_t tiles = (np + kPairTile - 1) / kPairTile;
    if (resident <= 0 || tiles <= 0) return slots;
    const int64_t lo = std::max<int64_t>(1, (3 * slots + 3) / 4);
    const int64_t hi = std::max<int64_t>(lo, std::min<int64_t>(3 * slots / 2,
                                                               h->dev.n_pair_segments));
    auto cost = [&](int64_t s) {
        return (double)((tiles * s + resident - 1) / resident) / (double)s;
    };
    double best = cost(slots);
    for (int64_t s = lo; s <= hi; s++) best = std::min(best, cost(s));
    for (int64_t s = lo; s <= hi; s++)
        if (cost(s) <= 1.02 * best) return s;
    return slots;
}

// FP64's rounding of an arrival time near t0, in bins: 2^-52 |t0| / |dt|.
// Above kFp64TimeRatio the automatic FP32 choice is the FP64-time mode, whose
// deposit follows that rounding as the reference's does (the chained FP32
// arrival times are more accurate than FP64's, and differ from them by about
// this much).
constexpr double kFp64TimeRatio = 1.0e-6;
__global__ void max_abs_kernel(const double* v, int n, unsigned long long* out) {
    unsigned long long m = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double a = fabs(v[i]);
        // non-negative doubles order like their bit patterns
        m = max(m, (unsigned long long)__double_as_longlong(isfinite(a) ? a : 0.0));
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}
// max |t0| over the pixels (device array), read back synchronously on s
int max_abs_t0(teufel_traj_set* h, const double* d_t0, int np, cudaStream_t s, double* out) {
    TRY_CUDA(cudaMemsetAsync(h->d_counters, 0, sizeof(unsigned long long), s));
    max_abs_kernel<<<std::min(64, (np + 255) / 256), 256, 0, s>>>(d_t0, np, h->d_counters);
    TRY_CUDA(cudaGetLastError());
    unsigned long long bits = 0;
    TRY_CUDA(cudaMemcpyAsync(&bits, h->d_counters, sizeof(bits), cudaMemcpyDeviceToHost, s));
    TRY_CUDA(cudaStreamSynchronize(s));
    double v;
    std::memcpy(&v, &bits, sizeof(v));
    *out = v;
    return TEUFEL_OK;
}
bool needs_fp64_time(double max_abs_t0, double dt) {
    return std::ldexp(max_abs_t0, -52) > kFp64TimeRatio * std::fabs(dt);
}

int run_device(teufel_traj_set* h, const double* d_pos, const double* d_t0, double dt, int nt,
               int np, double* d_out, const teufel_options& opt_in, cudaStream_t s,
               int slot_pct = 100, const HostOut* ho = nullptr, int* d_rec = nullptr,
               size_t staged_bytes = 0, double t0max_known = -1.0) {
    teufel_options opt = opt_in;
    // dt < 0 reverses the reference's window (tmin = t0 - dt/2 > tmax): a
    // step then deposits only when its arrivals straddle that window, and
    // the deposit goes to a negative bin, which FieldTrace::add rejects
    // (src/particle.cpp:780-823, src/fieldtrace.cpp:185-190).  The FP64
    // kernel takes exactly the reference's decisions there (no deposit, or
    // the range error); the FP32 kernels assume dt > 0.  The same holds for
    // sets whose arrival times can fall along a particle's points (a step
    // backwards in time or not slower than light, DevTraj::non_monotone).
    const bool fp64 = opt.precision == TEUFEL_PREC_FP64 || dt < 0.0 || h->dev.non_monotone;
    if (!fp64 && opt.precision == TEUFEL_PREC_FP32_FP64TIME) opt.kernel_variant = 9;
    if (!fp64 && opt.kernel_variant == 0) {
        // automatic: the FP64-time mode where FP64's rounding of the arrival
        // times is not negligible against the bins
        // (known on the host for host-buffer calls; else a device reduction)
        double t0max = t0max_known;
        if (!(t0max >= 0.0)) {
            int rc = max_abs_t0(h, d_t0, np, s, &t0max);
            if (rc) return rc;
        }
        if (needs_fp64_time(t0max, dt)) opt.kernel_variant = 9;
    }
    if (!fp64 && opt.kernel_variant == 0) {
        // else a tuned choice for this shape class, if there is one
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tuned.find(tune_key(h, np, nt));
        if (it != g_tuned.end()) {
            opt.kernel_variant = it->second.variant;
            if (opt.n_slots <= 0) slot_pct = it->second.slot_pct;
        }
    }
    const int variant = opt.kernel_variant == 1   ? kVariantUniform
                        : opt.kernel_variant == 2 ? kVariantLanes
                        : opt.kernel_variant == 3 ? kVariantWarp3
                        : opt.kernel_variant == 5 ? kVariantPair160
                        : opt.kernel_variant == 6 ? kVariantPair136
                        : opt.kernel_variant == 7 ? kVariantPair144
                        : opt.kernel_variant == 8 ? kVariantPairMulti
                        : opt.kernel_variant == 9 ? kVariantPairTime
                        : opt.kernel_variant == 10 ? kVariantPairC8
                        : opt.kernel_variant == 11 ? kVariantPairC32
                                                  : kVariantPair;  // 0 (automatic), 4
    const bool pairs = !fp64 && is_pair_variant(variant);
    // work units: particle segments, or pair segments for the pair kernel
    const int64_t G = pairs ? h->dev.n_pair_segments : h->dev.n_segments;
    const int64_t units = pairs ? h->dev.n_pairs : h->dev.n_particles;
    const int64_t max_units_per_slot = pairs ? kMaxParticlesPerSlotFp32 / 2
                                             : kMaxParticlesPerSlotFp32;
    const size_t elem = fp64 ? sizeof(double) : sizeof(float);
    const size_t slot_bytes = (size_t)np * (size_t)nt * 6 * elem;
    const int pix_blocks = (np + kThreads - 1) / kThreads;
    int64_t target = opt.n_slots > 0 ? opt.n_slots
                                     : (152LL * 512 * 4 + (int64_t)pix_blocks * kThreads - 1) /
                                           ((int64_t)pix_blocks * kThreads);
    if (opt.n_slots <= 0) target = std::max<int64_t>(1, target * slot_pct / 100);
    int64_t slots_total = std::max<int64_t>(target, 1);
    if (!fp64 && opt.n_slots <= 0)
        slots_total = std::max<int64_t>(slots_total,
                                        (units + max_units_per_slot - 1) / max_units_per_slot);
    if (pairs && opt.n_slots <= 0) slots_total = fill_waves(h, np, variant, slots_total);
    slots_total = std::min<int64_t>(slots_total, std::max<int64_t>(G, 1));
    cudaMemPool_t pool = scratch_pool(h->device);
    if (!pool) return TEUFEL_ERR_CUDA;
    size_t budget = std::min<size_t>((size_t)48 << 30,
                                     (size_t)(0.4 * (double)available_bytes(pool)));
    if (opt.max_device_mib > 0) {
        // the caller's bound, less what the call has staged already
        const size_t cap = (size_t)opt.max_device_mib << 20;
        if (cap < staged_bytes + slot_bytes) return TEUFEL_ERR_NOMEM;
        budget = std::min(budget, cap - staged_bytes);
    }
    int64_t per_pass = slot_bytes ? (int64_t)(budget / slot_bytes) : slots_total;
    per_pass = std::max<int64_t>(1, std::min<int64_t>(per_pass, slots_total));
    const size_t scratch_bytes = std::max<size_t>(slot_bytes * (size_t)per_pass, 256);
    void* scratch = nullptr;
    TRY_CUDA(cudaMallocFromPoolAsync(&scratch, scratch_bytes, pool, s));
    // returned to the pool on every exit, in stream order after the work
    struct Release {
        void* p;
        cudaStream_t s;
        ~Release() { cudaFreeAsync(p, s); }
    } release{scratch, s};
    h->last_slots = (int)slots_total;
    // geometric slot sizes for the pair kernel's grids of three waves or more
    // (below that the longest blocks set the time, and equal slots are best)
    bool geometric = false;
    if (pairs) {
        const int64_t resident = resident_pair_blocks(h, variant);
        const int64_t tiles = (np + kPairTile - 1) / kPairTile;
        geometric = resident > 0 && tiles * slots_total >= 3 * resident;
    }
    std::vector<int64_t> bounds =
        slot_bounds(G, slots_total, units, max_units_per_slot, geometric);
    if (h->slot_cap < slots_total + 1) {
        if (h->slot_seg) cudaFree(h->slot_seg);
        h->slot_seg = nullptr;
        h->slot_cap = 0;
        TRY_CUDA(cudaMalloc(&h->slot_seg, sizeof(int64_t) * (slots_total + 1)));
        h->slot_cap = (int)(slots_total + 1);
    }
    TRY_CUDA(cudaMemcpyAsync(h->slot_seg, bounds.data(), sizeof(int64_t) * (slots_total + 1),
                             cudaMemcpyHostToDevice, s));
    TRY_CUDA(cudaMemsetAsync(h->d_status, 0, sizeof(unsigned int), s));
    TRY_CUDA(cudaMemsetAsync(h->d_counters, 0, sizeof(h->last_counters), s));
    h->n_ev_used = 0;
    h->last_launches = 0;
    h->last_timed = opt.timing != 0;
    const int64_t n_passes = (slots_total + per_pass - 1) / per_pass;
    if (h->last_timed && (int64_t)h->ev.size() < 4 * n_passes) {
        while ((int64_t)h->ev.size() < 4 * n_passes) {
            cudaEvent_t e;
            TRY_CUDA(cudaEventCreate(&e));
            h->ev.push_back(e);
        }
    }
    DevScreen sc{d_pos, d_t0, np, nt, dt};
    for (int64_t p0 = 0; p0 < slots_total; p0 += per_pass) {
        DevWork w{};
        w.n_slots = (int)std::min<int64_t>(per_pass, slots_total - p0);
        // the first pass stores the traces when asked to, the others add
        w.overwrite = opt.overwrite_out && p0 == 0;
        w.slot_seg = h->slot_seg + p0;
        w.scratch = scratch;
        w.slot_stride = (int64_t)np * nt * 6;
        // the slots this pass accumulates into start from zero; the reduction
        // leaves them as they are
        TRY_CUDA(cudaMemsetAsync(scratch, 0, slot_bytes * (size_t)w.n_slots, s));
        w.status = h->d_status;
        w.frame = h->dev.frame;
        w.counters = h->d_counters;
        w.rec = d_rec;
        w.rec_stride = h->max_points;
        if (h->last_timed) TRY_CUDA(cudaEventRecord(h->ev[h->n_ev_used], s));
        cudaError_t e = fp64 ? launch_fp64(h->dev, sc, w, kThreads, s)
                             : launch_fp32(h->dev, sc, w, variant, s);
        if (e != cudaSuccess) return cuda_fail(e);
        if (h->last_timed) TRY_CUDA(cudaEventRecord(h->ev[h->n_ev_used + 1], s));
        if (ho && p0 == 0 && !opt.overwrite_out) TRY_CUDA(cudaStreamWaitEvent(s, ho->uploaded, 0));
        if (ho && p0 + per_pass >= slots_total) {
            const int64_t n_bins = (int64_t)np * nt;
            for (int k = 0; k < ho->n_chunks; k++) {
                const int64_t e0 = n_bins * k / ho->n_chunks, e1 = n_bins * (k + 1) / ho->n_chunks;
                e = fp64 ? launch_reduce_fp64(w, sc, d_out, s, e0, e1)
                         : launch_reduce_fp32(w, sc, d_out, s, e0, e1);
                if (e != cudaSuccess) return cuda_fail(e);
                TRY_CUDA(cudaEventRecord(ho->chunk_ev[k], s));
                TRY_CUDA(cudaStreamWaitEvent(ho->cs, ho->chunk_ev[k], 0));
                if (e1 > e0)
                    TRY_CUDA(cudaMemcpyAsync(ho->host + 6 * e0, d_out + 6 * e0,
                                             sizeof(double) * 6 * (size_t)(e1 - e0),
                                             cudaMemcpyDeviceToHost, ho->cs));
            }
        } else {
            e = fp64 ? launch_reduce_fp64(w, sc, d_out, s) : launch_reduce_fp32(w, sc, d_out, s);
            if (e != cudaSuccess) return cuda_fail(e);
        }
        if (h->last_timed) {
            TRY_CUDA(cudaEventRecord(h->ev[h->n_ev_used + 2], s));
            h->n_ev_used += 4;
        }
        h->last_launches += 2;
    }
    return TEUFEL_OK;
}

int finish(teufel_traj_set* h, cudaStream_t s) {
    unsigned int mask = 0;
    TRY_CUDA(cudaMemcpyAsync(&mask, h->d_status, sizeof(mask), cudaMemcpyDeviceToHost, s));
    TRY_CUDA(cudaMemcpyAsync(h->last_counters, h->d_counters, sizeof(h->last_counters),
                             cudaMemcpyDeviceToHost, s));
    TRY_CUDA(cudaStreamSynchronize(s));
    return status_from_mask(mask);
}

bool valid_screen_args(const teufel_traj_set* traj, const double* pos, const double* t0,
                       double dt, int nt, int np, const double* out) {
    if (!traj || nt < 0 || np < 0) return false;
    if (np > 0 && nt > 0 && (!pos || !t0 || !out)) return false;
    if (!std::isfinite(dt)) return false;
    return true;
}

}  // namespace

namespace teufel {
// device view and status word of a handle, for the allocation-free entry point
const DevTraj* traj_device_view(const teufel_traj_set* traj, unsigned int** status) {
    if (status) *status = traj->d_status;
    return &traj->dev;
}
int64_t traj_max_points(const teufel_traj_set* traj) { return traj->max_points; }
}  // namespace teufel

Frame identity_frame() {
    Frame f{};
    f.r[0] = f.r[4] = f.r[8] = 1.0;
    f.identity = 1;
    return f;
}

// The set's frame from its particles' directions of motion (vhat, the first
// to last point of each trajectory): z' along their mean.  A set moving
// within 1e-4 rad of a coordinate axis keeps the identity, which leaves its
// arithmetic untouched.
cudaError_t set_frame(DevTraj& d) {
    d.frame = identity_frame();
    d.non_monotone = 0;
    if (d.n_particles == 0) return cudaSuccess;
    std::vector<double4_32a> v((size_t)d.n_particles);
    cudaError_t e = cudaMemcpy(v.data(), d.vhat, sizeof(double4_32a) * v.size(),
                               cudaMemcpyDeviceToHost);
    if (e) return e;
    for (const auto& q : v)
        if (!(q.w > 0.0)) d.non_monotone = 1;
    double n[3] = {0.0, 0.0, 0.0};
    for (const auto& q : v) {
        n[0] += q.x;
        n[1] += q.y;
        n[2] += q.z;
    }
    const double L = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (!(L > 0.0)) return cudaSuccess;
    for (double& c : n) c /= L;
    const double big = std::max(std::fabs(n[0]), std::max(std::fabs(n[1]), std::fabs(n[2])));
    if (big > 1.0 - 5.0e-9) return cudaSuccess;  // along an axis already
    // x' from the coordinate axis least aligned with n, made orthogonal to n
    int k = 0;
    for (int j = 1; j < 3; j++)
        if (std::fabs(n[j]) < std::fabs(n[k])) k = j;
    double ax[3] = {0.0, 0.0, 0.0};
    ax[k] = 1.0;
    const double an = ax[0] * n[0] + ax[1] * n[1] + ax[2] * n[2];
    double ex[3] = {ax[0] - an * n[0], ax[1] - an * n[1], ax[2] - an * n[2]};
    const double le = std::sqrt(ex[0] * ex[0] + ex[1] * ex[1] + ex[2] * ex[2]);
    for (double& c : ex) c /= le;
    const double ey[3] = {n[1] * ex[2] - n[2] * ex[1], n[2] * ex[0] - n[0] * ex[2],
                          n[0] * ex[1] - n[1] * ex[0]};
    for (int j = 0; j < 3; j++) {
        d.frame.r[j] = ex[j];
        d.frame.r[3 + j] = ey[j];
        d.frame.r[6 + j] = n[j];
    }
    d.frame.identity = 0;
    return cudaSuccess;
}

// Builds a trajectory set: allocates the store, lets `fill` write the FP64
// points (tx, pp, aa) of N > 0 points on stream s (synchronized on return),
// then derives the FP32 per-point data and the pair layout.
// The order in which particles are paired: by the arrival of their first
// point at a far observer ahead, c t - n.x, n the mean direction of the
// first points' momenta (first[m] = t, x, y, z, bgx, bgy, bgz); particles
// without points last.  Stable, so equal keys keep the caller's order.
std::vector<int> pairing_order(int n_particles, const int* n_points, const double* first) {
    std::vector<int> order(n_particles);
    for (int m = 0; m < n_particles; m++) order[m] = m;
    if (!first) return order;
    double n[3] = {0.0, 0.0, 0.0};
    for (int m = 0; m < n_particles; m++) {
        if (n_points[m] <= 0) continue;
        const double* f = first + 7 * (size_t)m;
        const double b = std::sqrt(f[4] * f[4] + f[5] * f[5] + f[6] * f[6]);
        if (b > 0.0)
            for (int k = 0; k < 3; k++) n[k] += f[4 + k] / b;
    }
    const double L = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (!(L > 0.0)) return order;
    std::vector<double> key(n_particles, HUGE_VAL);
    for (int m = 0; m < n_particles; m++) {
        if (n_points[m] <= 0) continue;
        const double* f = first + 7 * (size_t)m;
        key[m] = kC * f[0] - (n[0] * f[1] + n[1] * f[2] + n[2] * f[3]) / L;
        if (!std::isfinite(key[m])) key[m] = HUGE_VAL;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
    return order;
}

template <class Fill>
int build_set(int n_particles, const int* n_points, const double* charge_C, const double* first,
              Fill fill, teufel_traj_set** out) {
    if (!out) return TEUFEL_ERR_ARG;
    *out = nullptr;
    if (n_particles < 0 || (n_particles > 0 && (!n_points || !charge_C))) return TEUFEL_ERR_ARG;
    int rc = check_device();
    if (rc) return rc;
    std::vector<int64_t> offs(n_particles + 1, 0), segs(n_particles + 1, 0);
    for (int m = 0; m < n_particles; m++) {
        if (n_points[m] < 0) return TEUFEL_ERR_ARG;
        offs[m + 1] = offs[m] + n_points[m];
        int64_t nseg = n_points[m] >= 1 ? ((int64_t)(n_points[m] - 1) >> kSegShift) + 1 : 0;
        segs[m + 1] = segs[m] + nseg;
    }
    const int64_t N = offs[n_particles];
    // pairs (2j, 2j+1): as long as the longer particle
    const int n_pairs = (n_particles + 1) / 2;
    const std::vector<int> order = pairing_order(n_particles, n_points, first);
    std::vector<int> members(2 * (size_t)n_pairs + 1, -1);
    std::vector<int64_t> poffs(n_pairs + 1, 0), psegs(n_pairs + 1, 0);
    for (int j = 0; j < n_pairs; j++) {
        members[2 * j] = order[2 * j];
        members[2 * j + 1] = 2 * j + 1 < n_particles ? order[2 * j + 1] : -1;
        int np = n_points[members[2 * j]];
        if (members[2 * j + 1] >= 0) np = std::max(np, n_points[members[2 * j + 1]]);
        poffs[j + 1] = poffs[j] + np;
        psegs[j + 1] = psegs[j] + (np >= 1 ? ((int64_t)(np - 1) >> kSegShift) + 1 : 0);
    }
    const int64_t NP = poffs[n_pairs];
    if (!finite_array(charge_C, n_particles)) return TEUFEL_ERR_ARG;
    teufel_traj_set* h = new (std::nothrow) teufel_traj_set();
    if (!h) return TEUFEL_ERR_NOMEM;
    h->h_seg_offsets = segs;
    for (int m = 0; m < n_particles; m++)
        h->max_points = std::max<int64_t>(h->max_points, n_points[m]);
    cudaGetDevice(&h->device);
    auto fail = [&](int code) {
        teufel_cuda_traj_free(h);
        return code;
    };
    DevTraj& d = h->dev;
    d.n_particles = n_particles;
    d.n_points = N;
    d.n_segments = segs[n_particles];
    d.n_pairs = n_pairs;
    d.n_pair_segments = psegs[n_pairs];
    int64_t *p_off, *p_seg, *p_poff, *p_pseg;
    int* p_members;
    float4* p_pq;
    double* p_charge;
    double4_32a *p_vhat, *p_tx, *p_pp, *p_aa;
    float4 *p_q0, *p_q1, *p_q2, *p_q3;
    if ((rc = dev_alloc(h, &p_off, n_particles + 1)) || (rc = dev_alloc(h, &p_seg, n_particles + 1)) ||
        (rc = dev_alloc(h, &p_charge, n_particles)) || (rc = dev_alloc(h, &p_vhat, n_particles)) ||
        (rc = dev_alloc(h, &p_tx, N)) || (rc = dev_alloc(h, &p_pp, N)) ||
        (rc = dev_alloc(h, &p_aa, N)) || (rc = dev_alloc(h, &p_q0, N)) ||
        (rc = dev_alloc(h, &p_q1, N)) || (rc = dev_alloc(h, &p_q2, N)) ||
        (rc = dev_alloc(h, &p_q3, N)) || (rc = dev_alloc(h, &p_poff, n_pairs + 1)) ||
        (rc = dev_alloc(h, &p_pseg, n_pairs + 1)) ||
        (rc = dev_alloc(h, &p_members, members.size())) ||
        (rc = dev_alloc(h, &p_pq, (size_t)kPairPoint * NP)))
        return fail(rc);
    if (cudaMalloc(&h->d_status, sizeof(unsigned int)) != cudaSuccess ||
        cudaMalloc(&h->d_counters, sizeof(h->last_counters)) != cudaSuccess)
        return fail(cuda_fail(cudaErrorMemoryAllocation));
    d.offsets = p_off;
    d.seg_offsets = p_seg;
    d.charge = p_charge;
    d.vhat = p_vhat;
    d.tx = p_tx;
    d.pp = p_pp;
    d.aa = p_aa;
    d.q0 = p_q0;
    d.q1 = p_q1;
    d.q2 = p_q2;
    d.q3 = p_q3;
    d.pair_offsets = p_poff;
    d.pair_seg_offsets = p_pseg;
    d.pair_members = p_members;
    d.pq = p_pq;
    cudaStream_t s = 0;
    if (cudaMemcpy(p_off, offs.data(), sizeof(int64_t) * (n_particles + 1), cudaMemcpyHostToDevice) ||
        cudaMemcpy(p_seg, segs.data(), sizeof(int64_t) * (n_particles + 1), cudaMemcpyHostToDevice) ||
        cudaMemcpy(p_poff, poffs.data(), sizeof(int64_t) * (n_pairs + 1), cudaMemcpyHostToDevice) ||
        cudaMemcpy(p_pseg, psegs.data(), sizeof(int64_t) * (n_pairs + 1), cudaMemcpyHostToDevice) ||
        cudaMemcpy(p_members, members.data(), sizeof(int) * members.size(),
                   cudaMemcpyHostToDevice) ||
        (n_particles > 0 &&
         cudaMemcpy(p_charge, charge_C, sizeof(double) * n_particles, cudaMemcpyHostToDevice)) ||
        cudaMemset(h->d_status, 0, sizeof(unsigned int)))
        return fail(cuda_fail(cudaGetLastError()));
    d.frame = identity_frame();
    if (N > 0) {
        cudaError_t e = fill(d, s, h->d_status);
        if (!e) e = launch_prep_particles(d, s);
        if (!e) e = cudaStreamSynchronize(s);
        if (!e) e = set_frame(d);
        if (!e) e = launch_prep_points(d, s);
        if (!e) e = launch_prep_pairs(d, s);
        cudaError_t e2 = cudaStreamSynchronize(s);
        if (e || e2) return fail(cuda_fail(e ? e : e2));
    } else if (n_particles > 0) {
        if (launch_prep_particles(d, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
            return fail(cuda_fail(cudaGetLastError()));
    }
    unsigned int mask = 0;
    if (cudaMemcpy(&mask, h->d_status, sizeof(mask), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(cuda_fail(cudaGetLastError()));
    if (mask) return fail(status_from_mask(mask));
    {
        std::lock_guard<std::mutex> lk(g_pool_mu);
        g_live_sets[h->device]++;
        h->counted = true;
    }
    *out = h;
    return TEUFEL_OK;
}

extern "C" {

void teufel_cuda_default_options(teufel_options* opt) {
    if (!opt) return;
    opt->precision = TEUFEL_PREC_FP32_SPLIT;
    opt->device_pointers = 0;
    opt->n_slots = 0;
    opt->kernel_variant = 0;
    opt->timing = 0;
    opt->max_device_mib = 0;
    opt->overwrite_out = 0;
}

const char* teufel_cuda_status_string(int status) {
    switch (status) {
        case TEUFEL_OK: return "ok";
        case TEUFEL_ERR_ARG: return "bad argument";
        case TEUFEL_ERR_NOMEM: return "out of memory";
        case TEUFEL_ERR_CUDA: return "CUDA error";
        case TEUFEL_ERR_RANGE: return "FieldTrace::add - index out of range.";
        case TEUFEL_ERR_TIMEOUT: return "device wait timed out";
        case TEUFEL_ERR_NODEVICE: return "no sm_103 CUDA device";
        default: return "unknown status";
    }
}

int teufel_cuda_traj_track(int n_particles, const double* init, const double* charge_e,
                           const double* mass, const teufel_lattice* lat, double tstep,
                           int n_steps, teufel_traj_set** out) {
    if (!out) return TEUFEL_ERR_ARG;
    *out = nullptr;
    if (n_particles < 0 || n_steps < 0 || !lat || !(tstep > 0.0) || !std::isfinite(tstep) ||
        (n_particles > 0 && (!init || !charge_e || !mass)))
        return TEUFEL_ERR_ARG;
    if (!finite_array(init, 7 * (int64_t)n_particles) || !finite_array(charge_e, n_particles) ||
        !finite_array(mass, n_particles))
        return TEUFEL_ERR_ARG;
    for (int m = 0; m < n_particles; m++)
        if (!(mass[m] != 0.0)) return TEUFEL_ERR_ARG;
    if (lat->has_undulator && !(lat->lambda_u > 0.0)) return TEUFEL_ERR_ARG;
    TrackLattice L{};
    L.has_undulator = lat->has_undulator != 0;
    L.b_peak = lat->b_peak;
    L.lambda_u = lat->lambda_u;
    L.kz = L.has_undulator ? 2.0 * kPi / lat->lambda_u : 0.0;  // src/undulator.cpp:79
    L.n_periods = lat->n_periods;
    L.has_homogeneous = lat->has_homogeneous != 0;
    for (int k = 0; k < 3; k++) {
        L.origin[k] = lat->origin[k];
        L.e[k] = lat->E[k];
        L.b[k] = lat->B[k];
    }
    if (n_steps >= (1 << 30)) return TEUFEL_ERR_ARG;
    std::vector<int> npts(n_particles, n_steps + 1);
    std::vector<double> charge_C(n_particles);
    for (int m = 0; m < n_particles; m++) charge_C[m] = charge_e[m] * kE;  // Charge*ElementaryCharge
    auto fill = [&](DevTraj& d, cudaStream_t s, unsigned int* status) -> cudaError_t {
        double* buf = nullptr;
        const size_t n = (size_t)n_particles;
        cudaError_t e = cudaMalloc(&buf, sizeof(double) * 9 * n);
        if (e) return e;
        e = cudaMemcpyAsync(buf, init, sizeof(double) * 7 * n, cudaMemcpyHostToDevice, s);
        if (!e) e = cudaMemcpyAsync(buf + 7 * n, charge_e, sizeof(double) * n, cudaMemcpyHostToDevice, s);
        if (!e) e = cudaMemcpyAsync(buf + 8 * n, mass, sizeof(double) * n, cudaMemcpyHostToDevice, s);
        if (!e)
            e = launch_vay_track(n_particles, buf, buf + 7 * n, buf + 8 * n, L, tstep, n_steps,
                                 const_cast<double4_32a*>(d.tx), const_cast<double4_32a*>(d.pp),
                                 const_cast<double4_32a*>(d.aa), status, s);
        cudaError_t e2 = cudaStreamSynchronize(s);
        cudaFree(buf);
        return e ? e : e2;
    };
    return build_set(n_particles, npts.data(), charge_C.data(), init, fill, out);
}

int teufel_cuda_traj_download(const teufel_traj_set* traj, double* t, double* x, double* bg,
                              double* a) {
    if (!traj) return TEUFEL_ERR_ARG;
    const int64_t N = traj->dev.n_points;
    if (N == 0) return TEUFEL_OK;
    std::vector<double4_32a> buf((size_t)N);
    const double4_32a* src[3] = {traj->dev.tx, traj->dev.pp, traj->dev.aa};
    double* dst[3] = {x, bg, a};
    for (int k = 0; k < 3; k++) {
        if (!(dst[k] || (k == 0 && t))) continue;
        TRY_CUDA(cudaMemcpy(buf.data(), src[k], sizeof(double4_32a) * N, cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < N; i++) {
            const double4_32a v = buf[i];
            if (k == 0) {
                if (t) t[i] = v.x;
                if (x) {
                    x[3 * i] = v.y;
                    x[3 * i + 1] = v.z;
                    x[3 * i + 2] = v.w;
                }
            } else {
                dst[k][3 * i] = v.x;
                dst[k][3 * i + 1] = v.y;
                dst[k][3 * i + 2] = v.z;
            }
        }
    }
    return TEUFEL_OK;
}

int teufel_cuda_traj_upload(int n_particles, const int* n_points, const double* charge_C,
                            const double* t, const double* x, const double* bg, const double* a,
                            teufel_traj_set** out) {
    int64_t N = 0;
    for (int m = 0; m < n_particles && n_points; m++) N += std::max(n_points[m], 0);
    if (N > 0 && (!t || !x || !bg || !a)) return TEUFEL_ERR_ARG;
    // the raw arrays to the device, then packed there (with a finite check)
    auto fill = [&](DevTraj& d, cudaStream_t s, unsigned int* status) -> cudaError_t {
        double* raw = nullptr;
        cudaError_t e = cudaMalloc(&raw, sizeof(double) * 10 * (size_t)N);
        if (e) return e;
        double *rt = raw, *rx = raw + N, *rb = raw + 4 * N, *ra = raw + 7 * N;
        e = cudaMemcpyAsync(rt, t, sizeof(double) * N, cudaMemcpyHostToDevice, s);
        if (!e) e = cudaMemcpyAsync(rx, x, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, s);
        if (!e) e = cudaMemcpyAsync(rb, bg, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, s);
        if (!e) e = cudaMemcpyAsync(ra, a, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, s);
        if (!e) {
            pack_points_kernel<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(
                N, rt, rx, rb, ra, const_cast<double4_32a*>(d.tx), const_cast<double4_32a*>(d.pp),
                const_cast<double4_32a*>(d.aa), status);
            e = cudaGetLastError();
        }
        cudaError_t e2 = cudaStreamSynchronize(s);
        cudaFree(raw);
        return e ? e : e2;
    };
    // the first point of every particle (t, x, beta*gamma), for the pairing order
    std::vector<double> first;
    if (N > 0 && n_points) {
        first.assign(7 * (size_t)n_particles, 0.0);
        int64_t o = 0;
        for (int m = 0; m < n_particles; m++) {
            if (n_points[m] > 0) {
                double* f = first.data() + 7 * (size_t)m;
                f[0] = t[o];
                for (int k = 0; k < 3; k++) {
                    f[1 + k] = x[3 * o + k];
                    f[4 + k] = bg[3 * o + k];
                }
            }
            o += std::max(n_points[m], 0);
        }
    }
    return build_set(n_particles, n_points, charge_C, first.empty() ? nullptr : first.data(), fill,
                     out);
}

int teufel_cuda_traj_free(teufel_traj_set* traj) {
    if (!traj) return TEUFEL_OK;
    if (traj->counted) {
        // the last set of a device gives the partial-trace pool's memory back
        std::lock_guard<std::mutex> lk(g_pool_mu);
        if (--g_live_sets[traj->device] == 0) {
            auto it = g_pools.find(traj->device);
            if (it != g_pools.end()) {
                cudaDeviceSynchronize();
                cudaMemPoolTrimTo(it->second, 0);
            }
        }
    }
    for (void* p : traj->owned) cudaFree(p);
    if (traj->scratch) cudaFree(traj->scratch);
    if (traj->slot_seg) cudaFree(traj->slot_seg);
    if (traj->d_pix) cudaFree(traj->d_pix);
    if (traj->d_out) cudaFree(traj->d_out);
    if (traj->d_status) cudaFree(traj->d_status);
    if (traj->d_counters) cudaFree(traj->d_counters);
    for (cudaEvent_t e : traj->ev) cudaEventDestroy(e);
    for (cudaEvent_t e : traj->cev) cudaEventDestroy(e);
    if (traj->copy_s) cudaStreamDestroy(traj->copy_s);
    delete traj;
    return TEUFEL_OK;
}

int64_t teufel_cuda_traj_points(const teufel_traj_set* traj) {
    return traj ? traj->dev.n_points : 0;
}

int teufel_cuda_integrate_screen_ex(const teufel_traj_set* traj_c, const double* pix_pos,
                                    const double* pix_t0, double dt, int Nt, int Np, double* out,
                                    const teufel_options* opt_in, teufel_stream_t stream) {
    teufel_traj_set* h = const_cast<teufel_traj_set*>(traj_c);
    if (!valid_screen_args(h, pix_pos, pix_t0, dt, Nt, Np, out)) return TEUFEL_ERR_ARG;
    teufel_options opt;
    teufel_cuda_default_options(&opt);
    if (opt_in) opt = *opt_in;
    if (opt.precision != TEUFEL_PREC_FP32_SPLIT && opt.precision != TEUFEL_PREC_FP64 &&
        opt.precision != TEUFEL_PREC_FP32_FP64TIME)
        return TEUFEL_ERR_ARG;
    for (auto& c : h->last_counters) c = 0;
    h->last_launches = 0;
    h->n_ev_used = 0;
    if (opt.overwrite_out != 0 && opt.overwrite_out != 1) return TEUFEL_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the reference returns early for traces shorter than 2 samples and for
    // trajectories shorter than 2 points (src/particle.cpp:778, 783): out
    // keeps its values, or holds zeros when it is to be overwritten
    if (Nt < 2 || Np == 0 || h->dev.n_particles == 0 || h->dev.n_segments == 0) {
        if (opt.overwrite_out && Np > 0 && Nt > 0) {
            const size_t n = sizeof(double) * 6 * (size_t)Np * (size_t)Nt;
            if (opt.device_pointers) {
                TRY_CUDA(cudaMemsetAsync(out, 0, n, s));
            } else {
                std::memset(out, 0, n);
            }
        }
        return TEUFEL_OK;
    }
    if (!(dt > 0.0) && !(dt < 0.0)) return TEUFEL_ERR_ARG;
    int rc;
    if (opt.device_pointers) {
        return run_device(h, pix_pos, pix_t0, dt, Nt, Np, out, opt, s);
    }
    if (!finite_array(pix_pos, 3 * (int64_t)Np) || !finite_array(pix_t0, Np)) return TEUFEL_ERR_ARG;
    double t0max = 0.0;
    for (int p = 0; p < Np; p++) t0max = std::max(t0max, std::fabs(pix_t0[p]));
    const size_t nout = (size_t)Np * (size_t)Nt * 6;
    // the staged pixel and trace buffers count against the caller's bound
    const size_t staged = sizeof(double) * (4 * (size_t)Np + nout);
    if (opt.max_device_mib > 0) {
        const bool fp64 = opt.precision == TEUFEL_PREC_FP64 || dt < 0.0 || h->dev.non_monotone;
        const size_t slot = nout * (fp64 ? sizeof(double) : sizeof(float));
        if (((size_t)opt.max_device_mib << 20) < staged + slot) return TEUFEL_ERR_NOMEM;
    }
    if ((rc = grow((void**)&h->d_pix, &h->pix_cap, sizeof(double) * 4 * (size_t)Np, false))) return rc;
    if ((rc = grow((void**)&h->d_out, &h->out_cap, sizeof(double) * nout, false))) return rc;
    double* d_pos = h->d_pix;
    double* d_t0 = h->d_pix + 3 * (size_t)Np;
    // The trace buffer moves on the copy stream: up while the integration
    // kernel runs, back chunk by chunk behind the reduction.
    constexpr int kOutChunks = 8;
    if (!h->copy_s) TRY_CUDA(cudaStreamCreateWithFlags(&h->copy_s, cudaStreamNonBlocking));
    while (h->cev.size() < 3 + (size_t)kOutChunks) {
        cudaEvent_t e;
        TRY_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        h->cev.push_back(e);
    }
    TRY_CUDA(cudaEventRecord(h->cev[0], s));
    TRY_CUDA(cudaStreamWaitEvent(h->copy_s, h->cev[0], 0));
    TRY_CUDA(cudaMemcpyAsync(d_pos, pix_pos, sizeof(double) * 3 * Np, cudaMemcpyHostToDevice, s));
    TRY_CUDA(cudaMemcpyAsync(d_t0, pix_t0, sizeof(double) * Np, cudaMemcpyHostToDevice, s));
    // out is uploaded only when the traces are added to it
    if (!opt.overwrite_out)
        TRY_CUDA(cudaMemcpyAsync(h->d_out, out, sizeof(double) * nout, cudaMemcpyHostToDevice,
                                 h->copy_s));
    TRY_CUDA(cudaEventRecord(h->cev[1], h->copy_s));
    const HostOut ho{out, h->copy_s, h->cev[1], h->cev.data() + 3, kOutChunks};
    rc = run_device(h, d_pos, d_t0, dt, Nt, Np, h->d_out, opt, s, 100, &ho, nullptr, staged,
                    t0max);
    if (rc) {
        cudaStreamSynchronize(h->copy_s);
        cudaStreamSynchronize(s);
        return rc;
    }
    TRY_CUDA(cudaEventRecord(h->cev[2], h->copy_s));
    TRY_CUDA(cudaStreamWaitEvent(s, h->cev[2], 0));
    return finish(h, s);
}

int teufel_cuda_autotune(const teufel_traj_set* traj_c, const double* pix_pos,
                         const double* pix_t0, double dt, int Nt, int Np,
                         const teufel_options* opt_in, teufel_options* best, double* best_ms) {
    teufel_traj_set* h = const_cast<teufel_traj_set*>(traj_c);
    if (!best || !valid_screen_args(h, pix_pos, pix_t0, dt, Nt, Np, pix_pos)) return TEUFEL_ERR_ARG;
    teufel_options opt;
    teufel_cuda_default_options(&opt);
    if (opt_in) opt = *opt_in;
    if (opt.precision != TEUFEL_PREC_FP32_SPLIT) return TEUFEL_ERR_ARG;
    *best = opt;
    if (best_ms) *best_ms = 0.0;
    if (Nt < 2 || Np == 0 || h->dev.n_particles == 0 || h->dev.n_segments == 0) return TEUFEL_OK;
    if (!(dt > 0.0) && !(dt < 0.0)) return TEUFEL_ERR_ARG;
    cudaStream_t s = nullptr;
    TRY_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    double* d_pix = nullptr;
    double* d_scr = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&](int rc) {
        if (s) cudaStreamSynchronize(s);
        if (d_pix) cudaFree(d_pix);
        if (d_scr) cudaFree(d_scr);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (s) cudaStreamDestroy(s);
        return rc;
    };
    const double* d_pos = pix_pos;
    const double* d_t0 = pix_t0;
    if (!opt.device_pointers) {
        if (!finite_array(pix_pos, 3 * (int64_t)Np) || !finite_array(pix_t0, Np))
            return cleanup(TEUFEL_ERR_ARG);
        if (cudaMalloc(&d_pix, sizeof(double) * 4 * (size_t)Np) != cudaSuccess ||
            cudaMemcpy(d_pix, pix_pos, sizeof(double) * 3 * Np, cudaMemcpyHostToDevice) ||
            cudaMemcpy(d_pix + 3 * (size_t)Np, pix_t0, sizeof(double) * Np, cudaMemcpyHostToDevice))
            return cleanup(cuda_fail(cudaGetLastError()));
        d_pos = d_pix;
        d_t0 = d_pix + 3 * (size_t)Np;
    }
    // the traces of the trial runs go to a scratch buffer, never to the caller's
    if (cudaMalloc(&d_scr, sizeof(double) * 6 * (size_t)Np * (size_t)Nt) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return cleanup(cuda_fail(cudaGetLastError()));
    opt.device_pointers = 1;
    opt.timing = 0;
    auto trial = [&](int variant, int pct, float* ms) {
        teufel_options o = opt;
        o.kernel_variant = variant;
        if (cudaEventRecord(e0, s) != cudaSuccess) return cuda_fail(cudaGetLastError());
        int rc = run_device(h, d_pos, d_t0, dt, Nt, Np, d_scr, o, s, pct);
        if (rc) return rc;
        if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
            cudaEventElapsedTime(ms, e0, e1) != cudaSuccess)
            return cuda_fail(cudaGetLastError());
        return TEUFEL_OK;
    };
    // variants at the automatic slot count, then the best one at half and
    // twice as many slots; the first trial also loads the modules.  A later
    // candidate must beat the best so far by more than kMargin: single trials
    // vary by a few tenths of a percent, and ties go to the default kernel
    // and the automatic slot count.
    constexpr float kMargin = 0.995f;
    const int variants[] = {4, 7, 6, 5, 8, 10, 11, 1};
    float ms = 0.0f, best_t = 1e30f;
    int bv = 4, bp = 100, rc;
    // bins short against FP64's rounding of the arrival times: only the
    // FP64-time kernel follows the reference there
    double t0max = 0.0;
    if ((rc = max_abs_t0(h, d_t0, Np, s, &t0max))) return cleanup(rc);
    if (needs_fp64_time(t0max, dt)) {
        bv = 9;
        if ((rc = trial(9, 100, &ms))) return cleanup(rc);
        if ((rc = trial(9, 100, &best_t))) return cleanup(rc);
    } else {
        if ((rc = trial(4, 100, &ms))) return cleanup(rc);
        for (int v : variants) {
            if ((rc = trial(v, 100, &ms))) return cleanup(rc);
            if (ms < best_t * kMargin || best_t == 1e30f) {
                best_t = ms;
                bv = v;
            }
        }
    }
    for (int pct : {50, 200}) {
        if ((rc = trial(bv, pct, &ms))) return cleanup(rc);
        if (ms < best_t * kMargin) {
            best_t = ms;
            bp = pct;
        }
    }
    // the slot count the choice resolves to, for callers that pass it explicitly
    if ((rc = trial(bv, bp, &ms))) return cleanup(rc);
    best->kernel_variant = bv;
    best->n_slots = h->last_slots;
    if (best_ms) *best_ms = best_t;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tuned[tune_key(h, Np, Nt)] = TuneChoice{bv, bp};
    }
    for (auto& c : h->last_counters) c = 0;
    return cleanup(TEUFEL_OK);
}

int teufel_cuda_retarded_field(const teufel_traj_set* traj_c, double obs_time, int Np,
                               const double* pos, double* out, teufel_stream_t stream) {
    teufel_traj_set* h = const_cast<teufel_traj_set*>(traj_c);
    if (!h || Np < 0 || (Np > 0 && (!pos || !out)) || !std::isfinite(obs_time))
        return TEUFEL_ERR_ARG;
    if (Np == 0) return TEUFEL_OK;
    // a particle without trajectory points: the reference throws
    // RANGEexception (src/particle.cpp:615)
    for (int m = 0; m < h->dev.n_particles; m++)
        if (h->h_seg_offsets[m + 1] == h->h_seg_offsets[m]) return TEUFEL_ERR_RANGE;
    if (!finite_array(pos, 3 * (int64_t)Np)) return TEUFEL_ERR_ARG;
    if (h->dev.n_particles == 0) {
        std::memset(out, 0, sizeof(double) * 6 * (size_t)Np);
        return TEUFEL_OK;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int n_chunks = retarded_field_chunks(Np, h->dev.n_particles);
    int rc;
    if ((rc = grow((void**)&h->d_pix, &h->pix_cap, sizeof(double) * 4 * (size_t)Np, false)) ||
        (rc = grow((void**)&h->d_out, &h->out_cap, sizeof(double) * 6 * (size_t)Np, false)) ||
        (rc = grow(&h->scratch, &h->scratch_bytes, sizeof(double) * 6 * (size_t)Np * n_chunks,
                   false)))
        return rc;
    TRY_CUDA(cudaMemcpyAsync(h->d_pix, pos, sizeof(double) * 3 * Np, cudaMemcpyHostToDevice, s));
    TRY_CUDA(launch_retarded_field(h->dev, obs_time, Np, h->d_pix, n_chunks,
                                   static_cast<double*>(h->scratch), h->d_out, s));
    TRY_CUDA(cudaMemcpyAsync(out, h->d_out, sizeof(double) * 6 * Np, cudaMemcpyDeviceToHost, s));
    TRY_CUDA(cudaStreamSynchronize(s));
    return TEUFEL_OK;
}

int teufel_cuda_integrate_screen(const teufel_traj_set* traj, const double* pix_pos,
                                 const double* pix_t0, double dt, int Nt, int Np, double* out,
                                 teufel_stream_t s) {
    return teufel_cuda_integrate_screen_ex(traj, pix_pos, pix_t0, dt, Nt, Np, out, nullptr, s);
}

int teufel_cuda_integrate_point(const teufel_traj_set* traj, const double* pos, double t0,
                                double dt, int Nt, double* out, teufel_stream_t s) {
    if (!pos) return TEUFEL_ERR_ARG;
    return teufel_cuda_integrate_screen_ex(traj, pos, &t0, dt, Nt, 1, out, nullptr, s);
}

int teufel_cuda_last_inwindow(const teufel_traj_set* traj, int64_t* inwindow,
                              int64_t* fallback_points) {
    if (!traj) return TEUFEL_ERR_ARG;
    teufel_traj_set* h = const_cast<teufel_traj_set*>(traj);
    unsigned int mask = 0;
    // device-pointer calls return before the counters are read back
    if (cudaDeviceSynchronize() != cudaSuccess) return cuda_fail(cudaGetLastError());
    if (h->d_counters &&
        (cudaMemcpy(h->last_counters, h->d_counters, sizeof(h->last_counters),
                    cudaMemcpyDeviceToHost) != cudaSuccess ||
         cudaMemcpy(&mask, h->d_status, sizeof(mask), cudaMemcpyDeviceToHost) != cudaSuccess))
        return cuda_fail(cudaGetLastError());
    if (inwindow) *inwindow = (int64_t)h->last_counters[0];
    if (fallback_points) *fallback_points = (int64_t)h->last_counters[1];
    return status_from_mask(mask);
}

int teufel_cuda_last_timing(const teufel_traj_set* traj, int64_t* deposits,
                            int64_t* evaluations, int* launches, double* kernel_ms,
                            double* reduce_ms) {
    if (!traj) return TEUFEL_ERR_ARG;
    teufel_traj_set* h = const_cast<teufel_traj_set*>(traj);
    if (cudaDeviceSynchronize() != cudaSuccess) return cuda_fail(cudaGetLastError());
    if (h->d_counters && cudaMemcpy(h->last_counters, h->d_counters, sizeof(h->last_counters),
                                    cudaMemcpyDeviceToHost) != cudaSuccess)
        return cuda_fail(cudaGetLastError());
    double k = 0.0, r = 0.0;
    if (h->last_timed) {
        for (int i = 0; i + 2 < h->n_ev_used; i += 4) {
            float a = 0.0f, b = 0.0f;
            if (cudaEventElapsedTime(&a, h->ev[i], h->ev[i + 1]) != cudaSuccess ||
                cudaEventElapsedTime(&b, h->ev[i + 1], h->ev[i + 2]) != cudaSuccess)
                return cuda_fail(cudaGetLastError());
            k += a;
            r += b;
        }
    }
    if (deposits) *deposits = (int64_t)h->last_counters[2];
    if (evaluations) *evaluations = (int64_t)h->last_counters[3];
    if (launches) *launches = h->last_launches;
    if (kernel_ms) *kernel_ms = k;
    if (reduce_ms) *reduce_ms = r;
    return TEUFEL_OK;
}

int teufel_cuda_point_decisions(const teufel_traj_set* traj, int m, const double* pos, double t0,
                                double dt, int Nt, int64_t* idx, int* flags, double* u_est,
                                float* band) {
    if (!traj || !pos || !idx || !flags || !u_est || m < 0 || m >= traj->dev.n_particles ||
        Nt < 0 || !(dt != 0.0))
        return TEUFEL_ERR_ARG;
    teufel_traj_set* h = const_cast<teufel_traj_set*>(traj);
    std::vector<int64_t> offs(2);
    TRY_CUDA(cudaMemcpy(offs.data(), h->dev.offsets + m, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost));
    int64_t n = offs[1] - offs[0];
    if (n <= 0) return TEUFEL_OK;
    int64_t* d_idx = nullptr;
    int* d_flags = nullptr;
    double* d_u = nullptr;
    float* d_band = nullptr;
    TRY_CUDA(cudaMalloc(&d_idx, sizeof(int64_t) * n));
    TRY_CUDA(cudaMalloc(&d_flags, sizeof(int) * n));
    TRY_CUDA(cudaMalloc(&d_u, sizeof(double) * n));
    TRY_CUDA(cudaMalloc(&d_band, sizeof(float) * n));
    cudaError_t e = launch_point_decisions(h->dev, m, make_double3(pos[0], pos[1], pos[2]), t0, dt,
                                           Nt, n, d_idx, d_flags, d_u, d_band, 0);
    if (!e) e = cudaMemcpy(idx, d_idx, sizeof(int64_t) * n, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(flags, d_flags, sizeof(int) * n, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(u_est, d_u, sizeof(double) * n, cudaMemcpyDeviceToHost);
    if (!e && band) e = cudaMemcpy(band, d_band, sizeof(float) * n, cudaMemcpyDeviceToHost);
    cudaFree(d_idx);
    cudaFree(d_flags);
    cudaFree(d_u);
    cudaFree(d_band);
    return e ? cuda_fail(e) : TEUFEL_OK;
}

int teufel_cuda_record_decisions(const teufel_traj_set* traj_c, const double* pix_pos,
                                 const double* pix_t0, double dt, int Nt, int Np,
                                 const teufel_options* opt_in, int32_t* rec, double* out) {
    teufel_traj_set* h = const_cast<teufel_traj_set*>(traj_c);
    if (!rec || !valid_screen_args(h, pix_pos, pix_t0, dt, Nt, Np, out)) return TEUFEL_ERR_ARG;
    teufel_options opt;
    teufel_cuda_default_options(&opt);
    if (opt_in) opt = *opt_in;
    opt.device_pointers = 0;
    opt.timing = 0;
    if (opt.precision != TEUFEL_PREC_FP32_SPLIT) return TEUFEL_ERR_ARG;
    // the kernels the automatic choice runs: variant 4 (default) and 8
    if (opt.kernel_variant == 0) opt.kernel_variant = 4;
    if (opt.kernel_variant != 4 && opt.kernel_variant != 8 && opt.kernel_variant != 9)
        return TEUFEL_ERR_ARG;
    const size_t n_rec = (size_t)std::max(Np, 0) * (size_t)h->dev.n_particles *
                         (size_t)h->max_points;
    if (n_rec) std::memset(rec, 0, sizeof(int32_t) * n_rec);
    for (auto& c : h->last_counters) c = 0;
    if (Nt < 2 || Np == 0 || h->dev.n_particles == 0 || h->dev.n_segments == 0) return TEUFEL_OK;
    // the FP32 kernels need dt > 0 and increasing arrivals
    if (!(dt > 0.0) || h->dev.non_monotone) return TEUFEL_ERR_ARG;
    if (!finite_array(pix_pos, 3 * (int64_t)Np) || !finite_array(pix_t0, Np)) return TEUFEL_ERR_ARG;
    const size_t nout = (size_t)Np * (size_t)Nt * 6;
    double* d_pix = nullptr;
    double* d_out = nullptr;
    int* d_rec = nullptr;
    auto cleanup = [&](int rc) {
        cudaDeviceSynchronize();
        if (d_pix) cudaFree(d_pix);
        if (d_out) cudaFree(d_out);
        if (d_rec) cudaFree(d_rec);
        return rc;
    };
    if (cudaMalloc(&d_pix, sizeof(double) * 4 * (size_t)Np) != cudaSuccess ||
        cudaMalloc(&d_out, sizeof(double) * nout) != cudaSuccess ||
        cudaMalloc(&d_rec, sizeof(int) * std::max<size_t>(n_rec, 1)) != cudaSuccess)
        return cleanup(cuda_fail(cudaErrorMemoryAllocation));
    if (cudaMemcpy(d_pix, pix_pos, sizeof(double) * 3 * Np, cudaMemcpyHostToDevice) ||
        cudaMemcpy(d_pix + 3 * (size_t)Np, pix_t0, sizeof(double) * Np, cudaMemcpyHostToDevice) ||
        cudaMemcpy(d_out, out, sizeof(double) * nout, cudaMemcpyHostToDevice) ||
        cudaMemset(d_rec, 0, sizeof(int) * std::max<size_t>(n_rec, 1)))
        return cleanup(cuda_fail(cudaGetLastError()));
    cudaStream_t s = nullptr;
    int rc = run_device(h, d_pix, d_pix + 3 * (size_t)Np, dt, Nt, Np, d_out, opt, s, 100, nullptr,
                        d_rec);
    if (rc) return cleanup(rc);
    rc = finish(h, s);
    if (cudaMemcpy(out, d_out, sizeof(double) * nout, cudaMemcpyDeviceToHost) ||
        (n_rec && cudaMemcpy(rec, d_rec, sizeof(int) * n_rec, cudaMemcpyDeviceToHost)))
        return cleanup(cuda_fail(cudaGetLastError()));
    return cleanup(rc);
}

int teufel_cuda_deposit_injected(int n_particles, const int* n_points, const double* ts,
                                 const double* f, double t0, double dt, int Nt, int precision,
                                 double* trace) {
    if (n_particles < 0 || Nt < 0 || (n_particles > 0 && !n_points) || !trace ||
        (precision != TEUFEL_PREC_FP32_SPLIT && precision != TEUFEL_PREC_FP64))
        return TEUFEL_ERR_ARG;
    int rc = check_device();
    if (rc) return rc;
    std::vector<int64_t> offs(n_particles + 1, 0);
    for (int m = 0; m < n_particles; m++) {
        if (n_points[m] < 0) return TEUFEL_ERR_ARG;
        offs[m + 1] = offs[m] + n_points[m];
    }
    int64_t N = offs[n_particles];
    if (Nt < 2) return TEUFEL_OK;
    if (N > 0 && (!ts || !f)) return TEUFEL_ERR_ARG;
    int64_t* d_off = nullptr;
    double *d_ts = nullptr, *d_f = nullptr, *d_tr = nullptr;
    unsigned int* d_st = nullptr;
    TRY_CUDA(cudaMalloc(&d_off, sizeof(int64_t) * (n_particles + 1)));
    TRY_CUDA(cudaMalloc(&d_ts, sizeof(double) * (N + 1)));
    TRY_CUDA(cudaMalloc(&d_f, sizeof(double) * 6 * (N + 1)));
    TRY_CUDA(cudaMalloc(&d_tr, sizeof(double) * 6 * Nt));
    TRY_CUDA(cudaMalloc(&d_st, sizeof(unsigned int)));
    cudaError_t e = cudaMemcpy(d_off, offs.data(), sizeof(int64_t) * (n_particles + 1),
                               cudaMemcpyHostToDevice);
    if (!e && N) e = cudaMemcpy(d_ts, ts, sizeof(double) * N, cudaMemcpyHostToDevice);
    if (!e && N) e = cudaMemcpy(d_f, f, sizeof(double) * 6 * N, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(d_tr, trace, sizeof(double) * 6 * Nt, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemset(d_st, 0, sizeof(unsigned int));
    if (!e) e = launch_deposit_injected(n_particles, d_off, d_ts, d_f, t0, dt, Nt, precision, d_tr,
                                        d_st, 0);
    unsigned int mask = 0;
    if (!e) e = cudaMemcpy(trace, d_tr, sizeof(double) * 6 * Nt, cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(&mask, d_st, sizeof(mask), cudaMemcpyDeviceToHost);
    cudaFree(d_off);
    cudaFree(d_ts);
    cudaFree(d_f);
    cudaFree(d_tr);
    cudaFree(d_st);
    if (e) return cuda_fail(e);
    return status_from_mask(mask);
}

int teufel_cuda_probe_peaks(double* fp32_tflops, double* fp32x2_tflops, double* fp64_tflops) {
    int rc = check_device();
    if (rc) return rc;
    return probe_peaks(fp32_tflops, fp32x2_tflops, fp64_tflops) ? TEUFEL_ERR_CUDA : TEUFEL_OK;
}

int teufel_cuda_check_fixed_division(int n, const double* a, double b, const double* ts,
                                     double t0, double dt, int nt, double* q, int* k) {
    if (n < 0 || (n > 0 && (!a || !ts || !q || !k)) || !(dt > 0.0) || nt < 0)
        return TEUFEL_ERR_ARG;
    int rc = check_device();
    if (rc) return rc;
    if (n == 0) return TEUFEL_OK;
    return fixed_division_check(n, a, b, ts, t0, dt, nt, q, k) ? TEUFEL_ERR_CUDA : TEUFEL_OK;
}

}  // extern "C"
