// lw_noalloc.cu -- an integration entry point that allocates no device memory.
//
// teufel_cuda_integrate_screen_ex grows its per-slot partial traces with
// cudaMalloc on demand.  Some callers cannot allow that: applications whose
// device memory is handed out by another allocator (a framework's caching
// allocator that has reserved the GPU, or an MPI code that sizes all device
// memory at start-up), and applications that must not allocate once running,
// because cudaMalloc/cudaFree may synchronize the whole device and stall work
// the caller keeps in flight on other streams.  For them this file provides
// teufel_cuda_integrate_screen_noalloc: the same FP32 split-precision kernel
// and FP64 reduction, with the partial traces held in a fixed file-scope
// device array of TEUFEL_NOALLOC_SCRATCH_BYTES instead of allocated memory.
//
// Properties of that array:
//  * every GPU that loads this library holds it (64 MiB) until the process exits;
//  * all calls share it and it keeps the last call's contents, so each call
//    clears the part it uses before the integration starts;
//  * two calls whose work overlaps on the GPU (different streams, or a second
//    call before the first finished on another host thread) use the same
//    memory and race: callers must order them.
//
// Set-up: the device address of the array is looked up once per device with
// cudaGetSymbolAddress, with that device current, by the first call made on
// that device.  Every call synchronizes its stream (after each pass and at the
// end), so no call can be made while that stream is being captured.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <mutex>

#include "lw_internal.h"
#include "teufel_cuda.h"

namespace {

constexpr int kMaxNoallocSlots = 64;
constexpr int kMaxDevices = 64;
constexpr int kNoallocThreads = 128;

// the partial traces of all slots of one call: float [slot][pixel][sample][6]
static __device__ __align__(256) unsigned char g_noalloc_scratch[TEUFEL_NOALLOC_SCRATCH_BYTES];
// segment bounds of the slots of one call
static __device__ __align__(256) int64_t g_noalloc_slot_seg[kMaxNoallocSlots + 1];

struct DeviceSymbols {
    bool ready = false;
    void* scratch = nullptr;
    int64_t* slot_seg = nullptr;
};
DeviceSymbols g_symbols[kMaxDevices];
std::mutex g_symbols_mutex;

// Looks the arrays up on the current device (once per device).
int device_symbols(DeviceSymbols** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return TEUFEL_ERR_NODEVICE;
    }
    std::lock_guard<std::mutex> lock(g_symbols_mutex);
    DeviceSymbols& s = g_symbols[dev];
    if (!s.ready) {
        void* scratch = nullptr;
        void* seg = nullptr;
        if (cudaGetSymbolAddress(&scratch, g_noalloc_scratch) != cudaSuccess ||
            cudaGetSymbolAddress(&seg, g_noalloc_slot_seg) != cudaSuccess) {
            cudaGetLastError();
            return TEUFEL_ERR_CUDA;
        }
        s.scratch = scratch;
        s.slot_seg = static_cast<int64_t*>(seg);
        s.ready = true;
    }
    *out = &s;
    return TEUFEL_OK;
}

int fail(cudaError_t e) {
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? TEUFEL_ERR_NOMEM : TEUFEL_ERR_CUDA;
}

}  // namespace

extern "C" int teufel_cuda_integrate_screen_noalloc(const teufel_traj_set* traj,
                                                    const double* d_pix_pos,
                                                    const double* d_pix_t0, double dt, int Nt,
                                                    int Np, double* d_out, teufel_stream_t stream) {
    using namespace teufel;
    // the warp kernel needs dt > 0 (a negative dt reverses the trace window;
    // teufel_cuda_integrate_screen takes it)
    if (!traj || Nt < 0 || Np < 0 || !std::isfinite(dt) || !(dt > 0.0)) return TEUFEL_ERR_ARG;
    if (Np > 0 && Nt > 0 && (!d_pix_pos || !d_pix_t0 || !d_out)) return TEUFEL_ERR_ARG;
    unsigned int* d_status = nullptr;
    const DevTraj* tr = traj_device_view(traj, &d_status);
    // nor a set whose arrival times can fall along the points (FP64 only)
    if (tr->non_monotone) return TEUFEL_ERR_ARG;
    // as the reference: no work for traces shorter than 2 samples or without steps
    if (Nt < 2 || Np == 0 || tr->n_particles == 0 || tr->n_segments == 0) return TEUFEL_OK;
    // one slot's partial traces must fit into the static array
    const size_t slot_bytes = (size_t)Np * (size_t)Nt * 6 * sizeof(float);
    if (slot_bytes > (size_t)TEUFEL_NOALLOC_SCRATCH_BYTES) return TEUFEL_ERR_ARG;
    DeviceSymbols* sym = nullptr;
    int rc = device_symbols(&sym);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    const int64_t G = tr->n_segments;
    const int64_t fit = (int64_t)(TEUFEL_NOALLOC_SCRATCH_BYTES / slot_bytes);
    const int pix_blocks = (Np + kNoallocThreads - 1) / kNoallocThreads;
    int64_t want = (152LL * 512 * 4 + (int64_t)pix_blocks * kNoallocThreads - 1) /
                   ((int64_t)pix_blocks * kNoallocThreads);
    int64_t per_pass = std::max<int64_t>(1, std::min<int64_t>({want, fit, (int64_t)kMaxNoallocSlots, G}));
    // slots hold at most 2048 particles' contributions in FP32, as the allocating path
    int64_t slots_total = std::max<int64_t>(per_pass, (tr->n_particles + 2047) / 2048);
    slots_total = std::min<int64_t>(slots_total, G);

    cudaError_t e = cudaMemsetAsync(d_status, 0, sizeof(unsigned int), s);
    if (e) return fail(e);
    DevScreen sc{d_pix_pos, d_pix_t0, Np, Nt, dt};
    for (int64_t p0 = 0; p0 < slots_total; p0 += per_pass) {
        const int n = (int)std::min<int64_t>(per_pass, slots_total - p0);
        int64_t bounds[kMaxNoallocSlots + 1];
        for (int k = 0; k <= n; k++) bounds[k] = G * (p0 + k) / slots_total;
        // the array keeps the previous call's contents: clear what this pass uses
        e = cudaMemsetAsync(sym->scratch, 0, slot_bytes * (size_t)n, s);
        if (!e) e = cudaMemcpyAsync(sym->slot_seg, bounds, sizeof(int64_t) * (n + 1),
                                    cudaMemcpyHostToDevice, s);
        // the bounds live on the host stack: wait for the copy before reusing them
        if (!e) e = cudaStreamSynchronize(s);
        if (e) return fail(e);
        DevWork w{};
        w.n_slots = n;
        w.slot_seg = sym->slot_seg;
        w.scratch = sym->scratch;
        w.slot_stride = (int64_t)Np * Nt * 6;
        w.status = d_status;
        w.frame = tr->frame;
        w.counters = nullptr;
        w.rec = nullptr;
        w.rec_stride = 0;
        e = launch_fp32(*tr, sc, w, kVariantUniform, s);
        if (!e) e = launch_reduce_fp32(w, sc, d_out, s);
        if (e) return fail(e);
    }
    unsigned int mask = 0;
    e = cudaMemcpyAsync(&mask, d_status, sizeof(mask), cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
    if (e) return fail(e);
    if (mask & (1u << TEUFEL_ERR_ARG)) return TEUFEL_ERR_ARG;
    if (mask & (1u << TEUFEL_ERR_RANGE)) return TEUFEL_ERR_RANGE;
    return mask ? TEUFEL_ERR_CUDA : TEUFEL_OK;
}
