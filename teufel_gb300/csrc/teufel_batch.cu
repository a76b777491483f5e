// teufel_batch.cu -- batched observers: one persistent launch over a device
// work queue, planned once and replayed as a CUDA graph.
//
// The reference's driver integrates its observers one after another
// (src/teufel_hybrid.cpp:692-709).  Small meshes then leave most of a GPU
// idle and every observer pays its own launches.  A batch instead cuts every
// observer into work items -- a tile of kPairTile pixels against one slot
// (particle range) of its trajectory set -- sorts them largest first, and
// lets a grid of one resident block set per SM drain the queue.  The partial
// traces of all observers are reduced by one more launch.  Both launches and
// the queue reset are captured into a CUDA graph at planning time.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "lw_internal.h"
#include "teufel_cuda.h"

using namespace teufel;

struct teufel_batch {
    int device = 0;
    int n_items = 0;
    int n_blocks = 0;
    std::vector<void*> owned;
    unsigned int* d_head = nullptr;
    unsigned int* d_status = nullptr;
    unsigned long long* d_counters = nullptr;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    bool ran = false;
    // what a recorded run (teufel_cuda_batch_record_decisions) launches again
    const DevTraj* d_tr = nullptr;
    const DevScreen* d_sc = nullptr;
    DevWork* d_wk = nullptr;
    const BatchItem* d_items = nullptr;
    double* const* d_out = nullptr;
    const int64_t* d_prefix = nullptr;
    int n_planned = 0;
    int64_t n_bins = 0;
    std::vector<DevWork> h_wk;
    std::vector<int> plan_of_obs;    // planned index of each observer, -1 without work
    std::vector<int64_t> rec_size;   // per planned observer: Np * particles * max points
};

namespace {

constexpr int64_t kMaxPairsPerSlot = 1024;  // 2048 particles: the FP32 accumulation bound

int fail_cuda(cudaError_t e) {
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? TEUFEL_ERR_NOMEM : TEUFEL_ERR_CUDA;
}

template <class T>
int alloc(teufel_batch* b, T** p, size_t n) {
    *p = nullptr;
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(n, 1));
    if (e != cudaSuccess) return fail_cuda(e);
    b->owned.push_back(*p);
    return TEUFEL_OK;
}

void destroy(teufel_batch* b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->cap) cudaStreamDestroy(b->cap);
    for (cudaEvent_t e : b->ev)
        if (e) cudaEventDestroy(e);
    for (void* p : b->owned) cudaFree(p);
    delete b;
}

struct Plan {
    int obs;
    int tiles;
    int64_t slots;
    double item_cost;  // pixels x pair-points per item, for the ordering
};

}  // namespace

extern "C" {

int teufel_cuda_batch_create(int n_obs, const teufel_observer* obs, const teufel_options* opt,
                             teufel_batch** out) {
    if (!out) return TEUFEL_ERR_ARG;
    *out = nullptr;
    if (n_obs < 0 || (n_obs > 0 && !obs) || !opt) return TEUFEL_ERR_ARG;
    if (opt->precision != TEUFEL_PREC_FP32_SPLIT || !opt->device_pointers) return TEUFEL_ERR_ARG;
    for (int o = 0; o < n_obs; o++) {
        const teufel_observer& ob = obs[o];
        // the batch runs FP32 kernels, which need dt > 0 (a negative dt
        // reverses the trace window; teufel_cuda_integrate_screen takes it)
        if (!ob.traj || ob.Nt < 0 || ob.Np < 0 || !std::isfinite(ob.dt)) return TEUFEL_ERR_ARG;
        if (ob.Np > 0 && ob.Nt >= 2 && !(ob.dt > 0.0)) return TEUFEL_ERR_ARG;
        // nor sets whose arrival times can fall along the points
        if (traj_device_view(ob.traj, nullptr)->non_monotone) return TEUFEL_ERR_ARG;
        if (ob.Np > 0 && ob.Nt > 0 && (!ob.pix_pos || !ob.pix_t0 || !ob.out))
            return TEUFEL_ERR_ARG;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return TEUFEL_ERR_NODEVICE;
    }
    teufel_batch* b = new (std::nothrow) teufel_batch();
    if (!b) return TEUFEL_ERR_NOMEM;
    cudaGetDevice(&b->device);
    auto fail = [&](int rc) {
        destroy(b);
        return rc;
    };

    // ---- plan: observers with work, their slots and tiles ----
    std::vector<const DevTraj*> trv(n_obs);
    std::vector<Plan> plans;
    double total_cost = 0.0;
    for (int o = 0; o < n_obs; o++) {
        trv[o] = traj_device_view(obs[o].traj, nullptr);
        const DevTraj& t = *trv[o];
        // as the reference: no work for traces shorter than 2 samples
        if (obs[o].Nt < 2 || obs[o].Np == 0 || t.n_pair_segments == 0) continue;
        Plan p{o, (obs[o].Np + kPairTile - 1) / kPairTile, 1, 0.0};
        total_cost += (double)obs[o].Np * (double)t.n_points;
        plans.push_back(p);
    }
    int dev_sms = 0;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, b->device);
    b->n_blocks = std::max(1, dev_sms) * pair_batch_blocks_per_sm();
    // aim at about eight items per resident block, each of similar cost
    const double target_item = total_cost / std::max(1.0, 8.0 * b->n_blocks);
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const double budget = std::min(48.0 * (1 << 30), 0.4 * (double)free_b);
    double scratch_total = 0.0;
    for (Plan& p : plans) {
        const DevTraj& t = *trv[p.obs];
        const double cost = (double)obs[p.obs].Np * (double)t.n_points;
        int64_t s = (int64_t)std::llround(cost / std::max(1.0, target_item * p.tiles));
        s = std::max<int64_t>(s, (t.n_pairs + kMaxPairsPerSlot - 1) / kMaxPairsPerSlot);
        if (opt->n_slots > 0) s = std::min<int64_t>(s, opt->n_slots);
        s = std::max<int64_t>(1, std::min<int64_t>(s, t.n_pair_segments));
        p.slots = s;
        p.item_cost = (double)kPairTile * (double)t.n_points / (double)s;
        scratch_total += (double)s * obs[p.obs].Np * obs[p.obs].Nt * 6.0 * sizeof(float);
    }
    // too much partial-trace memory: fewer slots, down to the FP32 bound
    if (scratch_total > budget) {
        const double shrink = budget / scratch_total;
        scratch_total = 0.0;
        for (Plan& p : plans) {
            const DevTraj& t = *trv[p.obs];
            const int64_t lo = (t.n_pairs + kMaxPairsPerSlot - 1) / kMaxPairsPerSlot;
            p.slots = std::max<int64_t>(std::min(lo, t.n_pair_segments),
                                        (int64_t)std::floor(p.slots * shrink));
            p.item_cost = (double)kPairTile * (double)t.n_points / (double)p.slots;
            scratch_total += (double)p.slots * obs[p.obs].Np * obs[p.obs].Nt * 6.0 * sizeof(float);
        }
        if (scratch_total > 0.9 * (double)free_b) return fail(TEUFEL_ERR_NOMEM);
    }

    // ---- device arrays ----
    const int np_ = (int)plans.size();
    std::vector<DevTraj> h_tr(np_);
    std::vector<DevScreen> h_sc(np_);
    std::vector<DevWork> h_wk(np_);
    std::vector<double*> h_out(np_);
    std::vector<int64_t> h_prefix(np_ + 1, 0);
    std::vector<BatchItem> items;
    int64_t seg_total = 0;
    for (int k = 0; k < np_; k++) seg_total += plans[k].slots + 1;
    int rc;
    int64_t* d_seg = nullptr;
    float* d_scratch = nullptr;
    if ((rc = alloc(b, &d_seg, (size_t)seg_total)) ||
        (rc = alloc(b, &d_scratch, (size_t)(scratch_total / sizeof(float)))) ||
        (rc = alloc(b, &b->d_head, 1)) || (rc = alloc(b, &b->d_status, 1)) ||
        (rc = alloc(b, &b->d_counters, 4)))
        return fail(rc);
    std::vector<int64_t> h_seg;
    h_seg.reserve(seg_total);
    size_t scratch_off = 0;
    for (int k = 0; k < np_; k++) {
        const Plan& p = plans[k];
        const teufel_observer& ob = obs[p.obs];
        const DevTraj& t = *trv[p.obs];
        h_tr[k] = t;
        h_sc[k] = DevScreen{ob.pix_pos, ob.pix_t0, ob.Np, ob.Nt, ob.dt};
        DevWork w{};
        w.n_slots = (int)p.slots;
        w.slot_seg = d_seg + h_seg.size();
        for (int64_t s = 0; s <= p.slots; s++) h_seg.push_back(t.n_pair_segments * s / p.slots);
        w.scratch = d_scratch + scratch_off;
        w.frame = t.frame;
        w.slot_stride = (int64_t)ob.Np * ob.Nt * 6;
        w.status = b->d_status;
        w.counters = b->d_counters;
        w.clear = 1;  // cleared at creation, and by each replay's reduction
        scratch_off += (size_t)p.slots * (size_t)w.slot_stride;
        h_wk[k] = w;
        h_out[k] = ob.out;
        h_prefix[k + 1] = h_prefix[k] + (int64_t)ob.Np * ob.Nt;
        for (int tile = 0; tile < p.tiles; tile++)
            for (int s = 0; s < (int)p.slots; s++) items.push_back(BatchItem{k, tile, s});
    }
    // largest items first, so the tail of the queue is made of small ones
    std::stable_sort(items.begin(), items.end(), [&](const BatchItem& x, const BatchItem& y) {
        return plans[x.obs].item_cost > plans[y.obs].item_cost;
    });
    b->n_items = (int)items.size();
    b->plan_of_obs.assign(n_obs, -1);
    for (int k = 0; k < np_; k++) {
        b->plan_of_obs[plans[k].obs] = k;
        b->rec_size.push_back((int64_t)obs[plans[k].obs].Np * trv[plans[k].obs]->n_particles *
                              traj_max_points(obs[plans[k].obs].traj));
        h_wk[k].rec = nullptr;
        h_wk[k].rec_stride = traj_max_points(obs[plans[k].obs].traj);
    }
    DevTraj* d_tr = nullptr;
    DevScreen* d_sc = nullptr;
    DevWork* d_wk = nullptr;
    double** d_out = nullptr;
    int64_t* d_prefix = nullptr;
    BatchItem* d_items = nullptr;
    if ((rc = alloc(b, &d_tr, np_)) || (rc = alloc(b, &d_sc, np_)) || (rc = alloc(b, &d_wk, np_)) ||
        (rc = alloc(b, &d_out, np_)) || (rc = alloc(b, &d_prefix, np_ + 1)) ||
        (rc = alloc(b, &d_items, items.size())))
        return fail(rc);
    if (cudaMemcpy(d_seg, h_seg.data(), sizeof(int64_t) * h_seg.size(), cudaMemcpyHostToDevice) ||
        cudaMemcpy(d_tr, h_tr.data(), sizeof(DevTraj) * np_, cudaMemcpyHostToDevice) ||
        cudaMemcpy(d_sc, h_sc.data(), sizeof(DevScreen) * np_, cudaMemcpyHostToDevice) ||
        cudaMemcpy(d_wk, h_wk.data(), sizeof(DevWork) * np_, cudaMemcpyHostToDevice) ||
        cudaMemcpy(d_out, h_out.data(), sizeof(double*) * np_, cudaMemcpyHostToDevice) ||
        cudaMemcpy(d_prefix, h_prefix.data(), sizeof(int64_t) * (np_ + 1),
                   cudaMemcpyHostToDevice) ||
        (!items.empty() && cudaMemcpy(d_items, items.data(), sizeof(BatchItem) * items.size(),
                                      cudaMemcpyHostToDevice)) ||
        cudaMemset(d_scratch, 0, std::max<size_t>((size_t)scratch_total, 1)))
        return fail(fail_cuda(cudaGetLastError()));

    b->d_tr = d_tr;
    b->d_sc = d_sc;
    b->d_wk = d_wk;
    b->d_items = d_items;
    b->d_out = d_out;
    b->d_prefix = d_prefix;
    b->n_planned = np_;
    b->n_bins = h_prefix[np_];
    b->h_wk = h_wk;

    // ---- the graph: reset the queue and status, integrate, reduce ----
    for (cudaEvent_t& e : b->ev)
        if (cudaEventCreate(&e) != cudaSuccess) return fail(fail_cuda(cudaGetLastError()));
    if (cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) != cudaSuccess)
        return fail(fail_cuda(cudaGetLastError()));
    if (cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return fail(fail_cuda(cudaGetLastError()));
    cudaError_t e = cudaMemsetAsync(b->d_head, 0, sizeof(unsigned int), b->cap);
    if (!e) e = cudaMemsetAsync(b->d_status, 0, sizeof(unsigned int), b->cap);
    if (!e) e = cudaMemsetAsync(b->d_counters, 0, 4 * sizeof(unsigned long long), b->cap);
    if (!e) e = cudaEventRecord(b->ev[0], b->cap);
    if (!e && b->n_items > 0)
        e = launch_fp32_pair_batch(d_tr, d_sc, d_wk, d_items, b->n_items, b->d_head,
                                   std::min(b->n_blocks, b->n_items), b->cap);
    if (!e) e = cudaEventRecord(b->ev[1], b->cap);
    if (!e && h_prefix[np_] > 0)
        e = launch_reduce_fp32_batch(d_wk, d_sc, d_out, d_prefix, np_, h_prefix[np_], b->cap);
    cudaError_t e2 = cudaStreamEndCapture(b->cap, &b->graph);
    if (e || e2) return fail(fail_cuda(e ? e : e2));
    if (cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess)
        return fail(fail_cuda(cudaGetLastError()));
    *out = b;
    return TEUFEL_OK;
}

int teufel_cuda_batch_run(teufel_batch* b, teufel_stream_t stream) {
    if (!b) return TEUFEL_ERR_ARG;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaGraphLaunch(b->exec, s) != cudaSuccess) return fail_cuda(cudaGetLastError());
    if (cudaEventRecord(b->ev[2], s) != cudaSuccess) return fail_cuda(cudaGetLastError());
    b->ran = true;
    return TEUFEL_OK;
}

int teufel_cuda_batch_status(teufel_batch* b, int64_t* work_items, int64_t* inwindow,
                             double* kernel_ms) {
    if (!b) return TEUFEL_ERR_ARG;
    if (work_items) *work_items = b->n_items;
    if (!b->ran) {
        if (inwindow) *inwindow = 0;
        if (kernel_ms) *kernel_ms = 0.0;
        return TEUFEL_OK;
    }
    if (cudaEventSynchronize(b->ev[2]) != cudaSuccess) return fail_cuda(cudaGetLastError());
    unsigned int mask = 0;
    unsigned long long cnt[4] = {0, 0, 0, 0};
    if (cudaMemcpy(&mask, b->d_status, sizeof(mask), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(cnt, b->d_counters, sizeof(cnt), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail_cuda(cudaGetLastError());
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]) != cudaSuccess) {
        cudaGetLastError();
        ms = 0.0f;
    }
    if (inwindow) *inwindow = (int64_t)cnt[0];
    if (kernel_ms) *kernel_ms = ms;
    if (mask & (1u << TEUFEL_ERR_ARG)) return TEUFEL_ERR_ARG;
    if (mask & (1u << TEUFEL_ERR_RANGE)) return TEUFEL_ERR_RANGE;
    return mask ? TEUFEL_ERR_CUDA : TEUFEL_OK;
}

int teufel_cuda_batch_record_decisions(teufel_batch* b, int obs, int32_t* rec) {
    if (!b || !rec || obs < 0 || obs >= (int)b->plan_of_obs.size()) return TEUFEL_ERR_ARG;
    const int k = b->plan_of_obs[obs];
    if (k < 0) return TEUFEL_OK;  // an observer without work records nothing
    const size_t n_rec = (size_t)b->rec_size[k];
    std::memset(rec, 0, sizeof(int32_t) * n_rec);
    int* d_rec = nullptr;
    cudaError_t e = cudaMalloc(&d_rec, sizeof(int) * std::max<size_t>(n_rec, 1));
    if (e) return fail_cuda(e);
    std::vector<DevWork> wk = b->h_wk;
    wk[k].rec = d_rec;
    cudaStream_t s = b->cap;
    e = cudaMemsetAsync(d_rec, 0, sizeof(int) * std::max<size_t>(n_rec, 1), s);
    if (!e) e = cudaMemcpyAsync(b->d_wk, wk.data(), sizeof(DevWork) * wk.size(),
                                cudaMemcpyHostToDevice, s);
    if (!e) e = cudaMemsetAsync(b->d_head, 0, sizeof(unsigned int), s);
    if (!e) e = cudaMemsetAsync(b->d_status, 0, sizeof(unsigned int), s);
    if (!e && b->n_items > 0)
        e = launch_fp32_pair_batch(b->d_tr, b->d_sc, b->d_wk, b->d_items, b->n_items, b->d_head,
                                   std::min(b->n_blocks, b->n_items), s, true);
    if (!e && b->n_bins > 0)
        e = launch_reduce_fp32_batch(b->d_wk, b->d_sc, b->d_out, b->d_prefix, b->n_planned,
                                     b->n_bins, s);
    // the graph's own work descriptors back in place
    if (!e) e = cudaMemcpyAsync(b->d_wk, b->h_wk.data(), sizeof(DevWork) * b->h_wk.size(),
                                cudaMemcpyHostToDevice, s);
    unsigned int mask = 0;
    if (!e) e = cudaMemcpyAsync(&mask, b->d_status, sizeof(mask), cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
    if (!e && n_rec) e = cudaMemcpy(rec, d_rec, sizeof(int) * n_rec, cudaMemcpyDeviceToHost);
    cudaFree(d_rec);
    if (e) return fail_cuda(e);
    if (mask & (1u << TEUFEL_ERR_ARG)) return TEUFEL_ERR_ARG;
    if (mask & (1u << TEUFEL_ERR_RANGE)) return TEUFEL_ERR_RANGE;
    return mask ? TEUFEL_ERR_CUDA : TEUFEL_OK;
}

int teufel_cuda_batch_free(teufel_batch* b) {
    if (!b) return TEUFEL_ERR_ARG;
    cudaDeviceSynchronize();
    destroy(b);
    return TEUFEL_OK;
}

}  // extern "C"
